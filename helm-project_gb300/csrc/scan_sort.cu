// Device prefix sum and stable LSD radix sort (8-bit digits), written for
// this library. Used by the LBVH build (leaf order by Morton code) and by
// the CSR assembly (rows, then columns) of the weight generator.
#include "internal.hpp"

namespace axgb {
namespace {

constexpr int kScanThreads = 256;
constexpr int kScanItems = 8;
constexpr int kScanTile = kScanThreads * kScanItems;

template <class T>
__device__ T block_exclusive_scan(T v, T *total, T *warp_sums) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    T x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        T y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[warp] = x;
    __syncthreads();
    if (warp == 0) {
        T w = lane < nw ? warp_sums[lane] : T(0);
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            T y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        warp_sums[lane] = w;
    }
    __syncthreads();
    T pre = warp > 0 ? warp_sums[warp - 1] : T(0);
    *total = warp_sums[nw - 1];
    __syncthreads();
    return pre + x - v;
}

template <class TIn, class TOut>
__global__ void k_tile_sums(const TIn *in, i64 n, TOut *sums) {
    __shared__ TOut ws[32];
    i64 base = static_cast<i64>(blockIdx.x) * kScanTile;
    TOut s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        i64 i = base + k * kScanThreads + threadIdx.x;
        if (i < n) s += static_cast<TOut>(in[i]);
    }
    TOut tot;
    block_exclusive_scan(s, &tot, ws);
    if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

template <class TOut>
__global__ void k_scan_sums(TOut *sums, i64 nb) {
    __shared__ TOut ws[32];
    TOut carry = 0;
    for (i64 b = 0; b < nb; b += kScanThreads) {
        i64 i = b + threadIdx.x;
        TOut v = i < nb ? sums[i] : TOut(0);
        TOut tot;
        TOut ex = block_exclusive_scan(v, &tot, ws);
        if (i < nb) sums[i] = carry + ex;
        carry += tot;
    }
}

template <class TIn, class TOut>
__global__ void k_tile_scan(const TIn *in, i64 n, const TOut *sums, TOut *out) {
    __shared__ TOut tile[kScanTile + kScanTile / 32];
    __shared__ TOut ws[32];
    auto at = [](int i) { return i + (i >> 5); };  // pad to spread banks
    i64 base = static_cast<i64>(blockIdx.x) * kScanTile;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int i = k * kScanThreads + threadIdx.x;
        tile[at(i)] = (base + i < n) ? static_cast<TOut>(in[base + i]) : TOut(0);
    }
    __syncthreads();
    TOut loc[kScanItems];
    TOut s = 0;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        loc[k] = s;
        s += tile[at(threadIdx.x * kScanItems + k)];
    }
    TOut tot;
    TOut ex = block_exclusive_scan(s, &tot, ws);
    TOut off = sums[blockIdx.x] + ex;
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) tile[at(threadIdx.x * kScanItems + k)] = off + loc[k];
    __syncthreads();
#pragma unroll
    for (int k = 0; k < kScanItems; ++k) {
        int i = k * kScanThreads + threadIdx.x;
        if (base + i < n) out[base + i] = tile[at(i)];
    }
    if (threadIdx.x == 0 && base + kScanTile >= n) out[n] = sums[blockIdx.x] + tot;
}

template <class TIn, class TOut>
void scan_impl(const TIn *in, TOut *out, i64 n, cudaStream_t s) {
    if (n <= 0) {
        AXGB_CUDA(cudaMemsetAsync(out, 0, sizeof(TOut), s));
        return;
    }
    i64 nb = (n + kScanTile - 1) / kScanTile;
    DBuf<TOut> sums(nb);
    k_tile_sums<TIn, TOut><<<static_cast<unsigned>(nb), kScanThreads, 0, s>>>(in, n, sums.p);
    k_scan_sums<TOut><<<1, kScanThreads, 0, s>>>(sums.p, nb);
    k_tile_scan<TIn, TOut><<<static_cast<unsigned>(nb), kScanThreads, 0, s>>>(in, n, sums.p, out);
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
}

// ─── radix sort ────────────────────────────────────────────────────────────

constexpr int kRsThreads = 256;
constexpr int kRsItems = 16;
constexpr int kRsTile = kRsThreads * kRsItems;
constexpr int kRsWarps = kRsThreads / 32;

template <class K>
__global__ void k_rs_hist(const K *keys, i64 n, int shift, int *hist, int nblocks) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    i64 base = static_cast<i64>(blockIdx.x) * kRsTile;
#pragma unroll 4
    for (int k = 0; k < kRsItems; ++k) {
        i64 i = base + k * kRsThreads + threadIdx.x;
        if (i < n) atomicAdd(&h[static_cast<int>((keys[i] >> shift) & 255u)], 1);
    }
    __syncthreads();
    hist[static_cast<i64>(threadIdx.x) * nblocks + blockIdx.x] = h[threadIdx.x];
}

// Stable scatter: item order within a tile is round-major, then warp, then
// lane; ranks are built from per-warp match groups and per-round digit
// prefix sums over warps, plus the running count of earlier rounds.
template <class K>
__global__ void k_rs_scatter(const K *kin, const int *vin, K *kout, int *vout, i64 n, int shift, const int *offs,
                             int nblocks) {
    __shared__ int run[256];
    __shared__ int base_off[256];
    __shared__ int wcnt[kRsWarps][256];
    __shared__ int rtot[256];
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    run[tid] = 0;
    base_off[tid] = offs[static_cast<i64>(tid) * nblocks + blockIdx.x];
    i64 base = static_cast<i64>(blockIdx.x) * kRsTile;
    for (int r = 0; r < kRsItems; ++r) {
#pragma unroll
        for (int q = 0; q < kRsWarps; ++q) wcnt[q][tid] = 0;
        __syncthreads();
        i64 i = base + r * kRsThreads + tid;
        bool valid = i < n;
        K key = valid ? kin[i] : K(0);
        int val = valid ? vin[i] : 0;
        unsigned d = valid ? static_cast<unsigned>((key >> shift) & 255u) : 256u + lane;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int rank = __popc(peers & ((1u << lane) - 1u));
        if (valid && lane == __ffs(peers) - 1) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {
            int acc = 0;
#pragma unroll
            for (int q = 0; q < kRsWarps; ++q) {
                int c = wcnt[q][tid];
                wcnt[q][tid] = acc;
                acc += c;
            }
            rtot[tid] = acc;
        }
        __syncthreads();
        if (valid) {
            int pos = base_off[d] + run[d] + wcnt[warp][d] + rank;
            kout[pos] = key;
            vout[pos] = val;
        }
        __syncthreads();
        run[tid] += rtot[tid];
    }
}

template <class K>
void radix_impl(K *keys, int *vals, i64 n, int key_bits, cudaStream_t s) {
    if (n <= 1 || key_bits <= 0) return;
    if (n >= (i64(1) << 31)) throw Error(AXGB_ERR_UNSUPPORTED, "radix sort: more than 2^31 items");
    int nblocks = static_cast<int>((n + kRsTile - 1) / kRsTile);
    DBuf<K> k2(n);
    DBuf<int> v2(n), hist(static_cast<size_t>(256) * nblocks), offs(static_cast<size_t>(256) * nblocks + 1);
    K *a = keys, *b = k2.p;
    int *av = vals, *bv = v2.p;
    for (int shift = 0; shift < key_bits; shift += 8) {
        k_rs_hist<K><<<nblocks, kRsThreads, 0, s>>>(a, n, shift, hist.p, nblocks);
        scan_impl<int, int>(hist.p, offs.p, static_cast<i64>(256) * nblocks, s);
        k_rs_scatter<K><<<nblocks, kRsThreads, 0, s>>>(a, av, b, bv, n, shift, offs.p, nblocks);
        AXGB_CUDA(cudaGetLastError());
        std::swap(a, b);
        std::swap(av, bv);
    }
    if (a != keys) {
        AXGB_CUDA(cudaMemcpyAsync(keys, a, n * sizeof(K), cudaMemcpyDeviceToDevice, s));
        AXGB_CUDA(cudaMemcpyAsync(vals, av, n * sizeof(int), cudaMemcpyDeviceToDevice, s));
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

void scan_exclusive_i32_to_i64(const int *in, i64 *out, i64 n, cudaStream_t s) { scan_impl<int, i64>(in, out, n, s); }
void scan_exclusive_i32(const int *in, int *out, i64 n, cudaStream_t s) { scan_impl<int, int>(in, out, n, s); }
void radix_sort_pairs_u64(std::uint64_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s) {
    radix_impl<std::uint64_t>(keys, vals, n, key_bits, s);
}
void radix_sort_pairs_u32(std::uint32_t *keys, int *vals, i64 n, int key_bits, cudaStream_t s) {
    radix_impl<std::uint32_t>(keys, vals, n, key_bits, s);
}

}  // namespace axgb
