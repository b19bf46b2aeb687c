// Blocked, shared-memory staged split-FP32 SpMM (the fast apply path).
//
// Layout (built once per matrix on the host from the CSR):
//   * rows are taken in 32-row slices (consecutive rows, so output stores of
//     a warp stay coalesced) and slices are grouped 4 at a time into blocks
//     of source locality: with a centroid hint (matrices from
//     generate_weights), slices are visited in 3-D Morton order and each
//     block takes the 3 nearest unused slices among the next ones in that
//     order; without a hint, 4 consecutive slices;
//   * inside a block the rows are sorted by entry count (longest first), so
//     warp w holds rows of similar length and loops only to its own maximum;
//   * the block's distinct source columns are rounded out to 16-byte chunks;
//     chunk j is staged at float offset 4*j of a field's staging area, and a
//     run of up to 32 zero floats follows the chunks (padding entries read
//     it);
//   * entries are stored k-major per warp: (staging index, hi, lo), in a
//     gather schedule that spreads each step's addresses over the banks
//     (order_entries, gather_schedule.hpp).
// Kernels: one CTA per block (or per work item of a persistent launch).
// Tiles of T fields are staged into shared memory ring slots: by a producer
// warp with cp.async.cg 16-byte copies and full/empty mbarriers per slot
// (k_blk_ws, the headline kernel), by all threads with one barrier per tile
// (k_blk_chunk, and the persistent batch kernel k_blk_persist), or with one
// cp.async.bulk per run of consecutive chunks and field, completing on an
// mbarrier (k_blk_bulk). Each row warp then reduces its rows for the T fields
// with packed f32x2 compensated arithmetic (fp32x2.cuh).
#include <algorithm>
#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <thread>

#include "fp32x2.cuh"
#include "gather_schedule.hpp"
#include "internal.hpp"

namespace axgb {
namespace {

constexpr int kWarps = 4;        // warps (32-row slices) per block
constexpr int kRows = 32 * kWarps;  // rows per block
// Staging strides (floats per field) compiled into the staged kernels: a
// block takes the smaller one that holds its chunks; blocks needing more than
// the larger one go to the direct kernels.
constexpr int kUsSmall = 256 * kWarps;
constexpr int kUsLarge = 768 * kWarps;
constexpr int kMaxUS = kUsLarge;  // staging floats per field a block may use
constexpr int kMaxL = 32;        // longest row handled by the blocked kernels
constexpr int kPool = 4;         // streams the class launches are spread over
// A warp steps through its entries in whole groups of kGroup (straight-line
// code, so the scheduler overlaps the compensated steps of neighbouring
// entries) and then through the 1 .. kGroup-1 entries left up to its longest
// row; entries past a row's end are zero (weight 0 on the zero slot) and
// leave the sums unchanged.
constexpr int kGroup = 4;
const int kUsBuckets[] = {kUsSmall, kUsLarge};
// Zero floats staged after a block's chunks, one in every shared-memory bank:
// a padding read can then take a bank no entry of its gather step uses. A
// block whose chunks nearly fill its staging stride gets what is left (at
// least 4 floats): zero_run_len.
constexpr int kZeroRun = 32;
__host__ __device__ constexpr int zero_run_len(int stride, int zero) {
    return stride - zero < kZeroRun ? stride - zero : kZeroRun;
}

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

template <class F>
void parallel_for_host(i64 n, F f) {
    unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 256 || nt == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    i64 chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        i64 b = t * chunk, e = std::min(n, b + chunk);
        if (b >= e) break;
        th.emplace_back([=] { f(b, e); });
    }
    for (auto &t : th) t.join();
}

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}
// 16-byte copy of which only the first `bytes` come from global memory; the
// rest of the 16 shared-memory bytes is zero-filled.
__device__ __forceinline__ void cp_async16_part(void *smem, const void *gmem, int bytes) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(smem_u32(smem)), "l"(gmem), "r"(bytes)
                 : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}
__device__ __forceinline__ void mbar_init(std::uint64_t *bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(std::uint64_t *bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(std::uint64_t *bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, unsigned bytes, std::uint64_t *bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}
__device__ __forceinline__ unsigned long long globaltimer_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ void mbar_arrive(std::uint64_t *bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Arrive on bar once every cp.async this thread issued so far has landed (the
// barrier's expected count includes this arrival).
__device__ __forceinline__ void cp_async_mbar_arrive(std::uint64_t *bar) {
    asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}
// Wait for the phase of the given parity to complete, for at most about one
// second; false when the bound ran out.
__device__ __forceinline__ bool mbar_wait_bounded(std::uint64_t *bar, unsigned parity) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = globaltimer_ns();
    while (!mbar_try_wait(bar, parity))
        if (globaltimer_ns() - t0 > 1000000000ull) return false;
    return true;
}

// Writes the zero run (zero_run_len floats at offset zero, 16-byte aligned)
// of each of n staging areas of stride floats.
__device__ __forceinline__ void zero_runs(float *xs, int n, int stride, int zero, int tid, int nthreads) {
    const int kPer = zero_run_len(stride, zero) / 4;
    for (int q = tid; q < n * kPer; q += nthreads)
        *reinterpret_cast<float4 *>(xs + (q / kPer) * stride + zero + 4 * (q % kPer)) = make_float4(0.f, 0.f, 0.f, 0.f);
}

// Staging indices of a thread's L entries, two 16-bit values a register
// (an index is below the largest staging stride, 3072 + 4). Indexed with
// compile-time k after unrolling, so the halves are selected statically.
template <int L>
struct PackedIdx {
    unsigned v[(L + 1) / 2];
    __device__ __forceinline__ int operator[](int k) const {
        return (k & 1) ? static_cast<int>(v[k >> 1] >> 16) : static_cast<int>(v[k >> 1] & 0xffffu);
    }
    __device__ __forceinline__ void set(int k, int q) {
        if (k & 1)
            v[k >> 1] |= static_cast<unsigned>(q) << 16;
        else
            v[k >> 1] = static_cast<unsigned>(q);
    }
};

struct BlkArgs {
    const int *blocks;  // block ids of this launch
    const int *brow, *wbase, *wlen;
    const unsigned short *lidx;
    const float *hi, *lo;
    const int *cstart, *ccol;  // chunk list per block
    const int *rstart;         // runs per block (bulk variant)
    const int4 *runs;
    int us;                    // staging stride of a field (floats)
    int *status;
    i64 nbl;                   // blocks in this launch
    i64 fchunk;                // fields per work item (multiple of the stage width)
    i64 n_src;                 // source cells: the last chunk may be partial
    float *ylo;                // low parts of the outputs (hi+lo form), or null
    i64 ldylo;
};

// Work item of this CTA: (field chunk, block), chunk-major so that all CTAs
// sweep the same fields at about the same time.
__device__ __forceinline__ int item_setup(const BlkArgs &a, const float *__restrict__ &x, i64 ldx,
                                          float *__restrict__ &y, i64 ldy, i64 &nrhs, float *&ylo) {
    const i64 item = blockIdx.x;
    const i64 chunk = item / a.nbl;
    const int b = a.blocks[item - chunk * a.nbl];
    const i64 f0 = chunk * a.fchunk;
    const i64 n = nrhs - f0 < a.fchunk ? nrhs - f0 : a.fchunk;
    x += f0 * ldx;
    y += f0 * ldy;
    ylo = a.ylo ? a.ylo + f0 * a.ldylo : nullptr;
    nrhs = n;
    return b;
}

// Low parts of two outputs of a packed pair (row value s + c, c = -cn).
__device__ __forceinline__ void store_lo(float *ylo, i64 ldylo, i64 f, i64 row, F2 s, F2 cn, float ra, float rb) {
    float sa, sb, ca, cb;
    upk(s, sa, sb);
    upk(cn, ca, cb);
    ylo[f * ldylo + row] = sum_err(sa, -ca, ra);
    ylo[(f + 1) * ldylo + row] = sum_err(sb, -cb, rb);
}

// Row reduction of one staged tile of T fields (field stride US floats in
// shared memory). Per entry the packed weights (h, -lo) are formed once for
// the T/2 field pairs; per pair the compensated step is 9 FMA-pipe ops.
template <int L, int T, int US>
__device__ __forceinline__ void reduce_tile_c(const float *cur, const PackedIdx<L> &li, const float *h, const float *lw, int wl,
                                              i64 f0, i64 nrhs, i64 row, float *__restrict__ y, i64 ldy,
                                              float *__restrict__ ylo, i64 ldylo) {
    if (f0 + T <= nrhs) {
        F2 sa[T / 2], cn[T / 2];
#pragma unroll
        for (int q = 0; q < T / 2; ++q) {
            sa[q] = pk(0.f, 0.f);
            cn[q] = pk(0.f, 0.f);
        }
        auto step = [&](int k) {
            const F2 hp = pk(h[k], h[k]), ln = pk(-lw[k], -lw[k]);
            const float *p0 = cur + li[k];
#pragma unroll
            for (int q = 0; q < T / 2; ++q) cstepn(sa[q], cn[q], h[k], hp, ln, p0[(2 * q) * US], p0[(2 * q + 1) * US]);
        };
#pragma unroll
        for (int k0 = 0; k0 < L; k0 += kGroup) {
            if (k0 + kGroup <= wl) {  // warp-uniform: a whole group
#pragma unroll
                for (int k = k0; k < k0 + kGroup && k < L; ++k) step(k);
            } else if (k0 < wl) {  // the warp's last 1 .. kGroup-1 entries
#pragma unroll
                for (int k = k0; k < k0 + kGroup - 1 && k < L; ++k)
                    if (k < wl) step(k);
            }
        }
        if (row >= 0) {
#pragma unroll
            for (int q = 0; q < T / 2; ++q) {
                float ra, rb;
                upk(sub2(sa[q], cn[q]), ra, rb);
                y[(f0 + 2 * q) * ldy + row] = ra;
                y[(f0 + 2 * q + 1) * ldy + row] = rb;
                if (ylo) store_lo(ylo, ldylo, f0 + 2 * q, row, sa[q], cn[q], ra, rb);
            }
        }
    } else {
        for (int f = 0; f < T; ++f) {
            if (f0 + f >= nrhs) break;
            float s1 = 0.f, c1 = 0.f;
            const float *p0 = cur + f * US;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < wl) csum1(s1, c1, h[k], lw[k], p0[li[k]]);
            if (row >= 0) {
                const float r = __fadd_rn(s1, c1);
                y[(f0 + f) * ldy + row] = r;
                if (ylo) ylo[(f0 + f) * ldylo + row] = sum_err(s1, c1, r);
            }
        }
    }
}

// Runtime-stride version used by the bulk-copy kernel.
template <int L, int T>
__device__ __forceinline__ void reduce_tile(const float *cur, int us, const PackedIdx<L> &li, const float *h, const float *lw,
                                            int wl, i64 f0, i64 nrhs, i64 row, float *__restrict__ y, i64 ldy,
                                            float *__restrict__ ylo, i64 ldylo) {
    if (f0 + T <= nrhs) {
        F2 sa[T / 2], cn[T / 2];
#pragma unroll
        for (int q = 0; q < T / 2; ++q) {
            sa[q] = pk(0.f, 0.f);
            cn[q] = pk(0.f, 0.f);
        }
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (k < wl) {
                const F2 h2 = pk(h[k], h[k]), l2 = pk(-lw[k], -lw[k]);
                const float *p0 = cur + li[k];
#pragma unroll
                for (int q = 0; q < T / 2; ++q) cstepn(sa[q], cn[q], h[k], h2, l2, p0[(2 * q) * us], p0[(2 * q + 1) * us]);
            }
        }
        if (row >= 0) {
#pragma unroll
            for (int q = 0; q < T / 2; ++q) {
                float ra, rb;
                upk(sub2(sa[q], cn[q]), ra, rb);
                y[(f0 + 2 * q) * ldy + row] = ra;
                y[(f0 + 2 * q + 1) * ldy + row] = rb;
                if (ylo) store_lo(ylo, ldylo, f0 + 2 * q, row, sa[q], cn[q], ra, rb);
            }
        }
    } else {
        for (int f = 0; f < T; ++f) {
            if (f0 + f >= nrhs) break;
            float s1 = 0.f, c1 = 0.f;
            const float *p0 = cur + f * us;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < wl) csum1(s1, c1, h[k], lw[k], p0[li[k]]);
            if (row >= 0) {
                const float r = __fadd_rn(s1, c1);
                y[(f0 + f) * ldy + row] = r;
                if (ylo) ylo[(f0 + f) * ldylo + row] = sum_err(s1, c1, r);
            }
        }
    }
}

template <int L>
__device__ __forceinline__ void load_entries(const BlkArgs &a, int b, int zero, PackedIdx<L> &li, float *h, float *lw, int &wl,
                                             i64 &row) {
    const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31;
    row = a.brow[static_cast<i64>(b) * kRows + tid];
    wl = a.wlen[b * kWarps + w];
    const int base = a.wbase[b * kWarps + w];
#pragma unroll
    for (int k = 0; k < L; ++k) {
        if (k < wl) {
            int e = base + k * 32 + lane;
            li.set(k, a.lidx[e]);
            h[k] = a.hi[e];
            lw[k] = a.lo[e];
        } else {
            li.set(k, zero);
            h[k] = 0.f;
            lw[k] = 0.f;
        }
    }
}

// One work item: block b for the fields of x/y (nrhs of them), staged T
// fields at a time through NS shared-memory buffers of US floats per field.
template <int L, int T, int NS, int US>
__device__ __forceinline__ void blk_item(const BlkArgs &a, int b, const float *__restrict__ x, i64 ldx,
                                         float *__restrict__ y, i64 ldy, i64 nrhs, float *smem,
                                         float *__restrict__ ylo) {
    static_assert(T % 2 == 0, "fields per stage must be even");
    static_assert(NS == 2 || NS == 3, "two or three staging buffers");
    float *xs = smem;                                       // [NS][T][US]
    int *cc = reinterpret_cast<int *>(smem + NS * T * US);  // chunk columns
    const int c0 = a.cstart[b], nch = a.cstart[b + 1] - c0;
    const int zero = 4 * nch;
    for (int j = threadIdx.x; j < nch; j += kRows) cc[j] = a.ccol[c0 + j];
    PackedIdx<L> li;
    float h[L], lw[L];
    int wl;
    i64 row;
    load_entries<L>(a, b, zero, li, h, lw, wl, row);
    zero_runs(xs, NS * T, US, zero, threadIdx.x, kRows);
    __syncthreads();
    const i64 ntile = (nrhs + T - 1) / T;
    // stage(t) commits one cp.async group (empty past the end, so group
    // counting stays uniform)
    auto stage = [&](i64 t) {
        if (t < ntile) {
            float *dst = xs + (t % NS) * T * US;
            const i64 fa = t * T;
            const int nf = static_cast<int>((nrhs - fa < static_cast<i64>(T)) ? nrhs - fa : static_cast<i64>(T));
            const float *xt = x + fa * ldx;
            for (int j = threadIdx.x; j < nch; j += kRows) {
                const float *src = xt + cc[j];
                const i64 left = a.n_src - cc[j];  // the chunk of the last source cells may be partial
                if (left >= 4) {
#pragma unroll
                    for (int f = 0; f < T; ++f)
                        if (f < nf) cp_async16(dst + f * US + 4 * j, src + f * ldx);
                } else {
#pragma unroll
                    for (int f = 0; f < T; ++f)
                        if (f < nf) cp_async16_part(dst + f * US + 4 * j, src + f * ldx, static_cast<int>(4 * left));
                }
            }
        }
        cp_async_commit();
    };
#pragma unroll
    for (int q = 0; q < NS - 1; ++q) stage(q);
    for (i64 t = 0; t < ntile; ++t) {
        cp_async_wait<NS - 2>();  // tile t has landed (NS-2 newer groups may be pending)
        __syncthreads();          // ... for every thread, and tile t-1 is no longer read
        stage(t + NS - 1);        // refill the buffer tile t-1 used
        reduce_tile_c<L, T, US>(xs + (t % NS) * T * US, li, h, lw, wl, t * T, nrhs, row, y, ldy, ylo, a.ldylo);
    }
    cp_async_wait<0>();
}

template <int L, int T, int NS, int US>
__global__ void __launch_bounds__(kRows) k_blk_chunk(BlkArgs a, const float *__restrict__ x, i64 ldx,
                                                    float *__restrict__ y, i64 ldy, i64 nrhs) {
    extern __shared__ __align__(128) float smem[];
    float *ylo;
    const int b = item_setup(a, x, ldx, y, ldy, nrhs, ylo);
    blk_item<L, T, NS, US>(a, b, x, ldx, y, ldy, nrhs, smem, ylo);
}

// Warp-specialised form of the same work item. Warps 0..kWarps-1 reduce
// rows as in k_blk_chunk; warp kWarps is the producer: it stages tile t into
// ring slot t % NS with cp.async and has each of its lanes arrive on the
// slot's `full` barrier when its copies land (count 32). A row warp waits on
// `full` only, reduces, and arrives on the slot's `empty` barrier (count
// kWarps); the producer waits on `empty` before it refills the slot. Row
// warps of different lengths are thus coupled only through the NS-slot ring,
// not by a CTA-wide barrier per tile. Every wait is bounded (about 1 s); a
// wait that runs out sets a.status and ends the item.
// Resident CTAs the register allocation must allow. A CTA is five warps; a
// sub-partition's 16K registers hold 8 of them at 64 registers a thread
// (6 CTAs), 7 at 72 (5 CTAs), 5 at 102 (4 CTAs). Short rows need few
// registers, so their classes are held to the counts that two staging slots
// of 1024 floats a field also allow; the long-row classes take what they
// need.
template <int L, int NS>
constexpr int ws_min_blocks() {
#ifdef WS_MINB16
    if (L == 16 && NS == 2) return WS_MINB16;
#endif
    return L <= 8 ? 6 : L <= 12 ? 5 : L <= 20 ? 4 : 1;
}
template <int L, int T, int NS, int US>
__global__ void __launch_bounds__(kRows + 32, ws_min_blocks<L, NS>()) k_blk_ws(BlkArgs a, const float *__restrict__ x, i64 ldx,
                                                      float *__restrict__ y, i64 ldy, i64 nrhs) {
    static_assert(T % 2 == 0, "fields per stage must be even");
    static_assert(NS >= 2 && NS <= 3, "two or three ring slots");
    constexpr int kThreads = kRows + 32;
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) std::uint64_t full[NS], empty[NS];
    __shared__ volatile int abort_flag;
    float *ylo;
    const int b = item_setup(a, x, ldx, y, ldy, nrhs, ylo);
    float *xs = smem;                                       // [NS][T][US]
    int *cc = reinterpret_cast<int *>(smem + NS * T * US);  // chunk columns
    const int c0 = a.cstart[b], nch = a.cstart[b + 1] - c0;
    const int zero = 4 * nch;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int j = tid; j < nch; j += kThreads) cc[j] = a.ccol[c0 + j];
    zero_runs(xs, NS * T, US, zero, tid, kThreads);
    if (tid == 0) {
        for (int s = 0; s < NS; ++s) {
            mbar_init(&full[s], 32);
            mbar_init(&empty[s], kWarps);
        }
        abort_flag = 0;
    }
    __syncthreads();
    const i64 ntile = (nrhs + T - 1) / T;
    if (warp == kWarps) {  // producer
        for (i64 t = 0; t < ntile; ++t) {
            const int s = static_cast<int>(t % NS);
            if (t >= NS && !mbar_wait_bounded(&empty[s], static_cast<unsigned>((t / NS - 1) & 1))) {
                abort_flag = 1;
                atomicExch(a.status, 1);
                break;
            }
            if (abort_flag) break;
            float *dst = xs + s * T * US;
            const i64 fa = t * T;
            const int nf = static_cast<int>((nrhs - fa < static_cast<i64>(T)) ? nrhs - fa : static_cast<i64>(T));
            const float *xt = x + fa * ldx;
            for (int j = lane; j < nch; j += 32) {
                const float *src = xt + cc[j];
                const i64 left = a.n_src - cc[j];  // the chunk of the last source cells may be partial
                if (left >= 4) {
#pragma unroll
                    for (int f = 0; f < T; ++f)
                        if (f < nf) cp_async16(dst + f * US + 4 * j, src + f * ldx);
                } else {
#pragma unroll
                    for (int f = 0; f < T; ++f)
                        if (f < nf) cp_async16_part(dst + f * US + 4 * j, src + f * ldx, static_cast<int>(4 * left));
                }
            }
            cp_async_mbar_arrive(&full[s]);
        }
        cp_async_wait<0>();
        return;
    }
    PackedIdx<L> li;
    float h[L], lw[L];
    int wl;
    i64 row;
    load_entries<L>(a, b, zero, li, h, lw, wl, row);
    for (i64 t = 0; t < ntile; ++t) {
        const int s = static_cast<int>(t % NS);
        if (!mbar_wait_bounded(&full[s], static_cast<unsigned>((t / NS) & 1))) {
            abort_flag = 1;
            atomicExch(a.status, 1);
            break;
        }
        reduce_tile_c<L, T, US>(xs + s * T * US, li, h, lw, wl, t * T, nrhs, row, y, ldy, ylo, a.ldylo);
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[s]);
    }
}

// ─── persistent form for batches of matrices ───────────────────────────────
// One descriptor per (matrix, row-length class): the class's blocks of that
// matrix and its fields. Items (descriptor, field chunk, block) are handed
// out by an atomic counter; each CTA loops until the counter passes the
// total, so blocks of all matrices of the class share one launch.
struct BlkDesc {
    BlkArgs a;  // a.blocks / a.nbl: the class's blocks; a.fchunk: fields per item
    const float *x;
    i64 ldx;
    float *y;
    i64 ldy;
    i64 nrhs;
    i64 item_begin;
};

template <int L, int T, int NS, int US>
__global__ void __launch_bounds__(kRows) k_blk_persist(const BlkDesc *__restrict__ d, int nd, i64 total,
                                                      unsigned long long *counter) {
    extern __shared__ __align__(128) float smem[];
    __shared__ long long s_item;
    while (true) {
        if (threadIdx.x == 0) s_item = static_cast<long long>(atomicAdd(counter, 1ull));
        __syncthreads();
        const i64 it = s_item;
        __syncthreads();  // every thread has read s_item
        if (it >= total) return;
        int q = 0;
        while (q + 1 < nd && d[q + 1].item_begin <= it) ++q;
        const BlkDesc &D = d[q];
        const i64 local = it - D.item_begin;
        const i64 chunk = local / D.a.nbl;
        const int b = D.a.blocks[local - chunk * D.a.nbl];
        const i64 f0 = chunk * D.a.fchunk;
        const i64 n = D.nrhs - f0 < D.a.fchunk ? D.nrhs - f0 : D.a.fchunk;
        blk_item<L, T, NS, US>(D.a, b, D.x + f0 * D.ldx, D.ldx, D.y + f0 * D.ldy, D.ldy, n, smem, nullptr);
        __syncthreads();  // shared memory is reused by the next item
    }
}

template <int L, int T>
__global__ void __launch_bounds__(kRows) k_blk_bulk(BlkArgs a, const float *__restrict__ x, i64 ldx,
                                                   float *__restrict__ y, i64 ldy, i64 nrhs) {
    static_assert(T % 2 == 0, "fields per stage must be even");
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) std::uint64_t bar[2];
    __shared__ int abort_flag;
    const int us = a.us;
    float *xs = smem;  // [2][T][us]
    float *ylo;
    const int b = item_setup(a, x, ldx, y, ldy, nrhs, ylo);
    const int c0 = a.cstart[b], nch = a.cstart[b + 1] - c0;
    const int zero = 4 * nch;
    const int r0 = a.rstart[b], nr = a.rstart[b + 1] - r0;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    PackedIdx<L> li;
    float h[L], lw[L];
    int wl;
    i64 row;
    load_entries<L>(a, b, zero, li, h, lw, wl, row);
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    zero_runs(xs, 2 * T, us, zero, threadIdx.x, kRows);
    __syncthreads();
    const i64 ntile = (nrhs + T - 1) / T;
    auto issue = [&](i64 t, int buf) {
        if (warp != 0) return;
        const i64 fa = t * T;
        const int nf = static_cast<int>((nrhs - fa < static_cast<i64>(T)) ? nrhs - fa : static_cast<i64>(T));
        if (lane == 0) mbar_expect_tx(&bar[buf], 16u * static_cast<unsigned>(nch) * static_cast<unsigned>(nf));
        __syncwarp();
        float *dst0 = xs + buf * T * us;
        for (int q = lane; q < nr; q += 32) {
            int4 r = a.runs[r0 + q];
            for (int f = 0; f < nf; ++f)
                bulk_g2s(dst0 + f * us + r.z, x + (fa + f) * ldx + r.x, 16u * static_cast<unsigned>(r.y), &bar[buf]);
        }
    };
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    issue(0, 0);
    for (i64 t = 0; t < ntile; ++t) {
        const int buf = static_cast<int>(t & 1);
        if (t + 1 < ntile) issue(t + 1, buf ^ 1);
        const unsigned parity = static_cast<unsigned>((t >> 1) & 1);
        const unsigned long long t0 = globaltimer_ns();
        while (!mbar_try_wait(&bar[buf], parity)) {
            if (globaltimer_ns() - t0 > 1000000000ull) {  // 1 s bound
                abort_flag = 1;
                atomicExch(a.status, 1);
                break;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        reduce_tile<L, T>(xs + buf * T * us, us, li, h, lw, wl, t * T, nrhs, row, y, ldy, ylo, a.ldylo);
        __syncthreads();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
}

// Mean cap centre of each run of `per` consecutive rows (32-row slices,
// 8-row segments).
__global__ void k_slice_centroid(const DCap *cap, i64 n_rows, i64 n_slices, int per, float *out) {
    i64 s = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= n_slices) return;
    double sx = 0, sy = 0, sz = 0;
    int n = 0;
    const i64 r1 = (n_rows < s * per + per) ? n_rows : s * per + per;
    for (i64 r = s * per; r < r1; ++r) {
        sx += cap[r].x;
        sy += cap[r].y;
        sz += cap[r].z;
        ++n;
    }
    double inv = n ? 1.0 / n : 0.0;
    out[3 * s] = static_cast<float>(sx * inv);
    out[3 * s + 1] = static_cast<float>(sy * inv);
    out[3 * s + 2] = static_cast<float>(sz * inv);
}

inline unsigned spread10h(unsigned v) {
    v &= 1023u;
    v = (v | (v << 16)) & 0x030000FFu;
    v = (v | (v << 8)) & 0x0300F00Fu;
    v = (v | (v << 4)) & 0x030C30C3u;
    v = (v | (v << 2)) & 0x09249249u;
    return v;
}

// Groups of up to 4 slices: Morton visit order, each group completed with
// the nearest unused slices among the next kWindow candidates.
std::vector<std::array<int, kWarps>> group_slices(i64 nsl, const std::vector<float> &xyz) {
    std::vector<std::array<int, kWarps>> groups;
    if (xyz.size() != static_cast<size_t>(3 * nsl)) {
        for (i64 q = 0; q < nsl; q += kWarps) {
            std::array<int, kWarps> g;
            g.fill(-1);
            for (int w = 0; w < kWarps && q + w < nsl; ++w) g[w] = static_cast<int>(q + w);
            groups.push_back(g);
        }
        return groups;
    }
    std::vector<std::pair<unsigned, int>> code(nsl);
    for (i64 q = 0; q < nsl; ++q) {
        auto qz = [](float v) { return static_cast<unsigned>(std::min(1023.f, std::max(0.f, (v + 1.f) * 512.f))); };
        code[q] = {(spread10h(qz(xyz[3 * q])) << 2) | (spread10h(qz(xyz[3 * q + 1])) << 1) | spread10h(qz(xyz[3 * q + 2])),
                   static_cast<int>(q)};
    }
    std::stable_sort(code.begin(), code.end());
    std::vector<int> order(nsl);
    for (i64 q = 0; q < nsl; ++q) order[q] = code[q].second;
    std::vector<char> used(nsl, 0);
    constexpr int kWindow = 48;
    for (i64 q = 0; q < nsl; ++q) {
        int s = order[q];
        if (used[s]) continue;
        used[s] = 1;
        std::array<int, kWarps> g;
        g.fill(-1);
        g[0] = s;
        // nearest kWarps - 1 among the next kWindow unused slices in Morton order
        std::vector<std::pair<float, int>> cand;
        for (i64 r = q + 1; r < nsl && kWarps > 1 && static_cast<int>(cand.size()) < kWindow; ++r) {
            int c = order[r];
            if (used[c]) continue;
            float dx = xyz[3 * c] - xyz[3 * s], dy = xyz[3 * c + 1] - xyz[3 * s + 1], dz = xyz[3 * c + 2] - xyz[3 * s + 2];
            cand.push_back({dx * dx + dy * dy + dz * dz, c});
        }
        std::partial_sort(cand.begin(), cand.begin() + std::min<size_t>(kWarps - 1, cand.size()), cand.end());
        for (int w = 0; w < kWarps - 1 && w < static_cast<int>(cand.size()); ++w) {
            g[w + 1] = cand[w].second;
            used[cand[w].second] = 1;
        }
        groups.push_back(g);
    }
    return groups;
}

struct HostBlock {
    int rows[kRows];
    int wlen[kWarps];
    int L;                     // row-length class (multiple of 4)
    int us;                    // 4 * chunks + zero run
    int zrun;                  // zero run length (floats)
    bool staged;               // taken by the staged kernels (else by the direct ones)
    std::vector<int> ccol;     // chunk start columns
    std::vector<int4> runs;    // (col, chunks, staging offset, 0)
    std::vector<unsigned short> lidx;  // k-major per warp, concatenated warps
    std::vector<float> hi, lo;
    int wbase_rel[kWarps];
};

// Order of each row's entries in the block (written to perm) and the warps'
// gather schedules (q: staging index, e: CSR index or -1 for padding, per
// warp k-major over its wlen steps), by WarpSchedule (gather_schedule.hpp).
// Padding reads the zero run (up to kZeroRun zero floats after the chunks,
// one a bank). A padding step of a row is exact (weight 0 on a +0 value
// leaves both sums unchanged), so every split-FP32 layout computes the same
// bits from perm. Blocks the staged kernels do not take (rows longer than
// kMaxL, or more staging than kMaxUS) keep each row's CSR order (schedule =
// false).
void order_entries(const HostBlock &H, const std::vector<int> &rp, const std::vector<int> &col,
                   const std::vector<int> &cols, std::vector<int> &perm, std::vector<int> &q_out,
                   std::vector<int> &e_out, WarpSchedule &S, bool schedule) {
    const int zero = 4 * static_cast<int>(cols.size());
    q_out.clear();
    e_out.clear();
    if (!schedule) {
        for (int w = 0; w < kWarps; ++w)
            for (int lane = 0; lane < 32; ++lane) {
                const int r = H.rows[32 * w + lane];
                if (r >= 0)
                    for (int k = rp[r]; k < rp[r + 1]; ++k) perm[k] = k;
            }
        return;
    }
    S.left.assign(zero + H.zrun, 0);
    for (int w = 0; w < kWarps; ++w) {
        for (int lane = 0; lane < 32; ++lane) {
            const int r = H.rows[32 * w + lane];
            S.cand[lane].clear();
            if (r < 0) continue;
            for (int k = rp[r]; k < rp[r + 1]; ++k) {
                const int c = col[k];
                const int pos =
                    static_cast<int>(std::lower_bound(cols.begin(), cols.end(), c >> 2) - cols.begin());
                S.cand[lane].push_back({k, 4 * pos + (c & 3)});
            }
        }
        AXGB_REQUIRE(S.run(H.wlen[w], zero, H.zrun, q_out, e_out),
                     "blocked layout: gather schedule left entries unplaced");
        for (int lane = 0; lane < 32; ++lane) {
            const int r = H.rows[32 * w + lane];
            if (r < 0) continue;
            for (size_t j = 0; j < S.placed[lane].size(); ++j) perm[rp[r] + j] = S.placed[lane][j];
        }
    }
}

}  // namespace

void slice_centroids(const MeshView &dst, Matrix &m, cudaStream_t s) {
    const i64 nsl = (m.n_dst + 31) / 32, nsg = (m.n_dst + 7) / 8;
    if (nsl == 0 || !dst.cap) return;
    DBuf<float> d(3 * nsl), d8(3 * nsg);
    k_slice_centroid<<<nblk(nsl, 256), 256, 0, s>>>(dst.cap, m.n_dst, nsl, 32, d.p);
    k_slice_centroid<<<nblk(nsg, 256), 256, 0, s>>>(dst.cap, m.n_dst, nsg, 8, d8.p);
    AXGB_CUDA(cudaGetLastError());
    m.slice_xyz.resize(3 * nsl);
    m.seg_xyz.resize(3 * nsg);
    AXGB_CUDA(cudaMemcpyAsync(m.slice_xyz.data(), d.p, sizeof(float) * 3 * nsl, cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaMemcpyAsync(m.seg_xyz.data(), d8.p, sizeof(float) * 3 * nsg, cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaStreamSynchronize(s));
}

// Source renumbering: new index = rank of first use when the rows are read
// in order (unused cells last, in their own order). Adopted when it cuts the
// 16-byte chunks the 128-row groups of consecutive rows touch by more than
// 1.5x; then col is rewritten in place and the renumbering uploaded.
void plan_source_order(Matrix &m, const std::vector<int> &rp, std::vector<int> &col, cudaStream_t s) {
    const i64 n = m.n_dst, nnz = m.nnz, ns = m.n_src;
    m.src_renum = false;
    if (nnz == 0 || ns == 0) return;
    std::vector<int> rank(ns, -1);
    int next = 0;
    for (i64 e = 0; e < nnz; ++e)
        if (rank[col[e]] < 0) rank[col[e]] = next++;
    for (i64 c = 0; c < ns; ++c)
        if (rank[c] < 0) rank[c] = next++;
    i64 ch0 = 0, ch1 = 0;
    std::vector<int> a, b;
    for (i64 r0 = 0; r0 < n; r0 += kRows) {
        const i64 e0 = rp[r0], e1 = rp[std::min<i64>(n, r0 + kRows)];
        a.clear();
        b.clear();
        for (i64 e = e0; e < e1; ++e) {
            a.push_back(col[e] >> 2);
            b.push_back(rank[col[e]] >> 2);
        }
        std::sort(a.begin(), a.end());
        std::sort(b.begin(), b.end());
        ch0 += std::unique(a.begin(), a.end()) - a.begin();
        ch1 += std::unique(b.begin(), b.end()) - b.begin();
    }
    if (ch0 <= ch1 + ch1 / 2) return;
    std::vector<int> inv(ns);
    for (i64 c = 0; c < ns; ++c) inv[rank[c]] = static_cast<int>(c);
    for (i64 e = 0; e < nnz; ++e) col[e] = rank[col[e]];
    m.src_inv.upload_vec(inv, s);
    m.split_col.upload_vec(col, s);
    m.src_renum = true;
}

void build_blocked(Matrix &m, cudaStream_t s) {
    Blocked &B = m.blocked;
    if (B.built) return;
    const i64 n = m.n_dst, nnz = m.nnz;
    const i64 nsl = (n + 31) / 32;
    std::vector<int> rp(n + 1), col(std::max<i64>(1, nnz));
    std::vector<double> val(std::max<i64>(1, nnz));
    AXGB_CUDA(cudaMemcpy(rp.data(), m.row_ptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (nnz) {
        AXGB_CUDA(cudaMemcpy(col.data(), m.col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
        AXGB_CUDA(cudaMemcpy(val.data(), m.val.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
    }
    plan_source_order(m, rp, col, s);  // columns below are in the split layouts' numbering
    auto groups = group_slices(nsl, m.slice_xyz);
    const i64 nb = static_cast<i64>(groups.size());
    std::vector<HostBlock> hb(nb);
    std::vector<int> perm(std::max<i64>(1, nnz));
    parallel_for_host(nb, [&](i64 b0, i64 b1) {
        std::vector<std::pair<int, int>> rl;
        std::vector<int> cols, sq, se;
        WarpSchedule scratch;
        for (i64 b = b0; b < b1; ++b) {
            HostBlock &H = hb[b];
            rl.clear();
            for (int g : groups[b])
                if (g >= 0)
                    for (i64 r = static_cast<i64>(g) * 32; r < std::min<i64>(n, static_cast<i64>(g) * 32 + 32); ++r)
                        rl.push_back({-(rp[r + 1] - rp[r]), static_cast<int>(r)});
            std::stable_sort(rl.begin(), rl.end());
            for (int t = 0; t < kRows; ++t) H.rows[t] = t < static_cast<int>(rl.size()) ? rl[t].second : -1;
            cols.clear();
            for (auto &pr : rl)
                for (int k = rp[pr.second]; k < rp[pr.second + 1]; ++k) cols.push_back(col[k] >> 2);
            std::sort(cols.begin(), cols.end());
            cols.erase(std::unique(cols.begin(), cols.end()), cols.end());
            H.ccol.resize(cols.size());
            for (size_t j = 0; j < cols.size(); ++j) H.ccol[j] = cols[j] * 4;
            {
                const int z = 4 * static_cast<int>(cols.size());
                int bucket = kUsBuckets[0];
                for (int u : kUsBuckets)
                    if (z + 4 <= u) {
                        bucket = u;
                        break;
                    }
                H.zrun = z + 4 <= kMaxUS ? zero_run_len(bucket, z) : 4;
                H.us = z + H.zrun;
            }
            H.runs.clear();
            for (size_t j = 0; j < cols.size();) {
                size_t j1 = j + 1;
                while (j1 < cols.size() && cols[j1] == cols[j1 - 1] + 1) ++j1;
                H.runs.push_back(make_int4(cols[j] * 4, static_cast<int>(j1 - j), static_cast<int>(4 * j), 0));
                j = j1;
            }
            int maxlen = 0;
            for (int w = 0; w < kWarps; ++w) {
                int mx = 0;
                for (int t = 32 * w; t < 32 * w + 32; ++t)
                    if (H.rows[t] >= 0) mx = std::max(mx, rp[H.rows[t] + 1] - rp[H.rows[t]]);
                H.wlen[w] = mx;
                maxlen = std::max(maxlen, mx);
            }
            H.L = std::max(4, (maxlen + 3) / 4 * 4);
            H.staged = maxlen <= kMaxL && H.us <= kMaxUS;
            order_entries(H, rp, col, cols, perm, sq, se, scratch, H.staged);
            if (!H.staged)  // no entries stored: the direct kernels take these slices
                for (int w = 0; w < kWarps; ++w) H.wlen[w] = 0;
            H.lidx.resize(sq.size());
            H.hi.resize(sq.size());
            H.lo.resize(sq.size());
            for (size_t i = 0; i < sq.size(); ++i) {
                const int e = se[i];
                H.lidx[i] = static_cast<unsigned short>(sq[i]);
                H.hi[i] = e >= 0 ? static_cast<float>(val[e]) : 0.f;
                H.lo[i] = e >= 0 ? static_cast<float>(val[e] - static_cast<double>(H.hi[i])) : 0.f;
            }
            int off = 0;
            for (int w = 0; w < kWarps; ++w) {
                H.wbase_rel[w] = off;
                off += 32 * H.wlen[w];
            }
        }
    });
    // classes and flattening
    std::vector<int> brow(nb * kRows), wbase(nb * kWarps), wlen(nb * kWarps), cstart(nb + 1, 0), rstart(nb + 1, 0);
    std::vector<int> ccol;
    std::vector<int4> runs;
    std::vector<unsigned short> lidx;
    std::vector<float> hi, lo;
    std::map<std::pair<int, int>, std::vector<int>> cls;
    std::vector<int> fb;
    for (i64 b = 0; b < nb; ++b) {
        HostBlock &H = hb[b];
        const int ebase = static_cast<int>(lidx.size());
        for (int t = 0; t < kRows; ++t) brow[b * kRows + t] = H.rows[t];
        for (int w = 0; w < kWarps; ++w) {
            wbase[b * kWarps + w] = ebase + H.wbase_rel[w];
            wlen[b * kWarps + w] = H.wlen[w];
        }
        cstart[b] = static_cast<int>(ccol.size());
        ccol.insert(ccol.end(), H.ccol.begin(), H.ccol.end());
        rstart[b] = static_cast<int>(runs.size());
        runs.insert(runs.end(), H.runs.begin(), H.runs.end());
        lidx.insert(lidx.end(), H.lidx.begin(), H.lidx.end());
        hi.insert(hi.end(), H.hi.begin(), H.hi.end());
        lo.insert(lo.end(), H.lo.begin(), H.lo.end());
        if (H.staged) {
            int ub = 0;
            while (kUsBuckets[ub] < H.us) ++ub;
            cls[{H.L, kUsBuckets[ub]}].push_back(static_cast<int>(b));
        } else {
            for (int g : groups[b])
                if (g >= 0) fb.push_back(g);
        }
        std::vector<int>().swap(H.ccol);
        std::vector<unsigned short>().swap(H.lidx);
        std::vector<float>().swap(H.hi);
        std::vector<float>().swap(H.lo);
    }
    cstart[nb] = static_cast<int>(ccol.size());
    rstart[nb] = static_cast<int>(runs.size());
    AXGB_REQUIRE(lidx.size() < (size_t(1) << 31), "blocked layout: too many entries");
    std::vector<int> ids;
    B.launches.clear();
    for (auto &kv : cls) {
        Blocked::Launch l;
        l.L = kv.first.first;
        l.us = kv.first.second;
        l.begin = static_cast<i64>(ids.size());
        l.n = static_cast<i64>(kv.second.size());
        ids.insert(ids.end(), kv.second.begin(), kv.second.end());
        B.launches.push_back(l);
    }
    B.order.resize(B.launches.size());
    for (size_t q = 0; q < B.order.size(); ++q) B.order[q] = static_cast<int>(q);
    std::stable_sort(B.order.begin(), B.order.end(),
                     [&](int p1, int p2) { return B.launches[p1].n > B.launches[p2].n; });
    B.n_blocks = nb;
    B.n_src = m.n_src;
    B.h_us.resize(nb);
    for (i64 b = 0; b < nb; ++b) B.h_us[b] = hb[b].us;
    B.h_block_ids = ids;
    B.brow.upload_vec(brow, s);
    B.wbase.upload_vec(wbase, s);
    B.wlen.upload_vec(wlen, s);
    B.cstart.upload_vec(cstart, s);
    B.ccol.upload_vec(ccol, s);
    B.rstart.upload_vec(rstart, s);
    B.runs.upload_vec(runs, s);
    B.lidx.upload_vec(lidx, s);
    B.hi.upload_vec(hi, s);
    B.lo.upload_vec(lo, s);
    B.block_ids.upload_vec(ids, s);
    B.fallback_slices.upload_vec(fb, s);
    m.split_perm.upload_vec(perm, s);
    B.n_fallback = static_cast<i64>(fb.size());
    if (!B.status.p) {
        B.status.alloc(1);
        B.status.zero(s);
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
    B.built = true;
}

bool blocked_eligible(const Matrix &m, const void *x, i64 ldx, bool bulk) {
    // 16-byte aligned field starts; the bulk copies also need whole chunks
    return (reinterpret_cast<std::uintptr_t>(x) % 16 == 0) && (ldx % 4 == 0) && (!bulk || m.n_src % 4 == 0);
}

int blocked_launches(const Matrix &m) {
    return static_cast<int>(m.blocked.launches.size()) + (m.blocked.n_fallback > 0 ? 1 : 0);
}

namespace {

template <int L, int T, int NS, int US>
void launch_chunk_us(const BlkArgs &a, i64 grid, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    size_t bytes = sizeof(float) * static_cast<size_t>(US) * NS * T + sizeof(int) * static_cast<size_t>(US / 4);
    AXGB_CUDA(cudaFuncSetAttribute(k_blk_chunk<L, T, NS, US>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(bytes)));
    k_blk_chunk<L, T, NS, US><<<static_cast<unsigned>(grid), kRows, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

// Staging stride buckets compiled in: kUsSmall and kUsLarge floats per field.
template <int L, int T>
void launch_chunk(const BlkArgs &a, int us, int ns, i64 grid, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs,
                  cudaStream_t s) {
    if (us <= kUsSmall) {
        if (ns >= 3)
            launch_chunk_us<L, T, 3, kUsSmall>(a, grid, x, ldx, y, ldy, nrhs, s);
        else
            launch_chunk_us<L, T, 2, kUsSmall>(a, grid, x, ldx, y, ldy, nrhs, s);
    } else {
        launch_chunk_us<L, (T > 4 ? 4 : T), 2, kUsLarge>(a, grid, x, ldx, y, ldy, nrhs, s);
    }
}

template <int L, int T, int NS, int US>
void launch_ws_us(const BlkArgs &a, i64 grid, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    size_t bytes = sizeof(float) * static_cast<size_t>(US) * NS * T + sizeof(int) * static_cast<size_t>(US / 4);
    AXGB_CUDA(cudaFuncSetAttribute(k_blk_ws<L, T, NS, US>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(bytes)));
    k_blk_ws<L, T, NS, US><<<static_cast<unsigned>(grid), kRows + 32, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

// Ring depth with the most resident CTAs: three slots unless two let more
// CTAs fit (registers, not staging memory, often bound the count). Cached
// per instantiation.
template <int L, int T>
int ws_auto_stages() {
    static int ns = 0;
    if (ns) return ns;
    constexpr size_t b2 = sizeof(float) * kUsSmall * 2 * T + sizeof(int) * (kUsSmall / 4);
    constexpr size_t b3 = sizeof(float) * kUsSmall * 3 * T + sizeof(int) * (kUsSmall / 4);
    AXGB_CUDA(cudaFuncSetAttribute(k_blk_ws<L, T, 2, kUsSmall>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(b2)));
    AXGB_CUDA(cudaFuncSetAttribute(k_blk_ws<L, T, 3, kUsSmall>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                   static_cast<int>(b3)));
    int o2 = 0, o3 = 0;
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o2, k_blk_ws<L, T, 2, kUsSmall>, kRows + 32, b2));
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o3, k_blk_ws<L, T, 3, kUsSmall>, kRows + 32, b3));
    ns = o3 >= o2 ? 3 : 2;
    return ns;
}

template <int L, int T>
void launch_ws(const BlkArgs &a, int us, int ns, i64 grid, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs,
               cudaStream_t s) {
    if (us <= kUsSmall) {
        if (ns == 0) ns = ws_auto_stages<L, T>();
        if (ns >= 3)
            launch_ws_us<L, T, 3, kUsSmall>(a, grid, x, ldx, y, ldy, nrhs, s);
        else
            launch_ws_us<L, T, 2, kUsSmall>(a, grid, x, ldx, y, ldy, nrhs, s);
    } else {
        launch_ws_us<L, T, 2, kUsLarge>(a, grid, x, ldx, y, ldy, nrhs, s);
    }
}

template <int L, int T>
void launch_one(const Blocked &B, const Blocked::Launch &l, int kind, int ns, const float *x, i64 ldx, float *y,
                i64 ldy, i64 nrhs, i64 fchunk, cudaStream_t s, float *ylo, i64 ldylo) {
    const bool bulk = kind == 2;
    BlkArgs a{};
    a.ylo = ylo;
    a.ldylo = ldylo;
    a.nbl = l.n;
    a.fchunk = (fchunk <= 0 || fchunk >= nrhs) ? nrhs : (fchunk + T - 1) / T * T;
    const i64 grid = l.n * ((nrhs + a.fchunk - 1) / a.fchunk);
    a.blocks = B.block_ids.p + l.begin;
    a.brow = B.brow.p;
    a.wbase = B.wbase.p;
    a.wlen = B.wlen.p;
    a.lidx = B.lidx.p;
    a.hi = B.hi.p;
    a.lo = B.lo.p;
    a.cstart = B.cstart.p;
    a.ccol = B.ccol.p;
    a.rstart = B.rstart.p;
    a.runs = B.runs.p;
    a.us = l.us;
    a.status = B.status.p;
    a.n_src = B.n_src;
    if (kind == 3) {
        if constexpr (T == 4) launch_ws<L, T>(a, l.us, ns, grid, x, ldx, y, ldy, nrhs, s);  // four fields per stage only
    } else if (bulk) {
        size_t bytes = sizeof(float) * static_cast<size_t>(l.us) * 2 * T;
        AXGB_CUDA(cudaFuncSetAttribute(k_blk_bulk<L, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       static_cast<int>(bytes)));
        k_blk_bulk<L, T><<<static_cast<unsigned>(grid), kRows, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
    } else {
        launch_chunk<L, T>(a, l.us, ns, grid, x, ldx, y, ldy, nrhs, s);
    }
}

template <int T>
void launch_class(const Blocked &B, const Blocked::Launch &l, int kind, int ns, const float *x, i64 ldx, float *y,
                  i64 ldy, i64 nrhs, i64 fchunk, cudaStream_t s, float *ylo, i64 ldylo) {
    {
        if (l.n == 0) return;
        // T = 8 staging of the largest buckets would exceed shared memory: use 4 there
        const bool big = static_cast<size_t>(l.us) * 2 * T * sizeof(float) > 200 * 1024;
        if (T == 8 && big) {
            switch (l.L) {
                case 4: launch_one<4, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 8: launch_one<8, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 12: launch_one<12, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 16: launch_one<16, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 20: launch_one<20, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 24: launch_one<24, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                case 28: launch_one<28, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
                default: launch_one<32, 4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            }
            return;
        }
        switch (l.L) {
            case 4: launch_one<4, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 8: launch_one<8, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 12: launch_one<12, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 16: launch_one<16, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 20: launch_one<20, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 24: launch_one<24, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            case 28: launch_one<28, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
            default: launch_one<32, T>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, s, ylo, ldylo); break;
        }
    }
}

}  // namespace

// ─── batches ────────────────────────────────────────────────────────────────
namespace {

constexpr int kBatchT = 4, kBatchNS = 2;
constexpr i64 kBatchFChunk = 32;  // fields per work item
// Short-row blocks (at most 8 entries a row) whose staging needs at most
// kUsTiny floats a field (a coarse source under a fine destination) run in a
// batch with that stride and 8 fields per stage: 16 KB of staging instead of
// 32 KB, so more CTAs fit, and twice the work per tile.
constexpr int kUsTiny = 256, kTinyT = 8, kTinyMaxL = 8;
constexpr i64 kTinyFChunk = 64;  // fields per work item there (32 measured 6% slower on the 17-pair batch)

BlkArgs blk_args(const Blocked &B, const Blocked::Launch &l, i64 n_src) {
    BlkArgs a{};
    a.n_src = n_src;
    a.nbl = l.n;
    a.blocks = B.block_ids.p + l.begin;
    a.brow = B.brow.p;
    a.wbase = B.wbase.p;
    a.wlen = B.wlen.p;
    a.lidx = B.lidx.p;
    a.hi = B.hi.p;
    a.lo = B.lo.p;
    a.cstart = B.cstart.p;
    a.ccol = B.ccol.p;
    a.rstart = B.rstart.p;
    a.runs = B.runs.p;
    a.us = l.us;
    a.status = B.status.p;
    return a;
}

template <int L, int US, int T = kBatchT>
void persist_launch(const BlkDesc *d, int nd, i64 total, unsigned long long *counter, cudaStream_t s) {
    constexpr size_t bytes = sizeof(float) * US * kBatchNS * T + sizeof(int) * (US / 4);
    auto k = k_blk_persist<L, T, kBatchNS, US>;
    AXGB_CUDA(cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    int dev = 0, sms = 0, per = 0;
    AXGB_CUDA(cudaGetDevice(&dev));
    AXGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k, kRows, bytes));
    const i64 grid = std::min<i64>(total, static_cast<i64>(sms) * std::max(1, per));
    k<<<static_cast<unsigned>(grid), kRows, bytes, s>>>(d, nd, total, counter);
}

template <int US>
void persist_dispatch(int L, const BlkDesc *d, int nd, i64 total, unsigned long long *counter, cudaStream_t s) {
    switch (L) {
        case 4: persist_launch<4, US>(d, nd, total, counter, s); break;
        case 8: persist_launch<8, US>(d, nd, total, counter, s); break;
        case 12: persist_launch<12, US>(d, nd, total, counter, s); break;
        case 16: persist_launch<16, US>(d, nd, total, counter, s); break;
        case 20: persist_launch<20, US>(d, nd, total, counter, s); break;
        case 24: persist_launch<24, US>(d, nd, total, counter, s); break;
        case 28: persist_launch<28, US>(d, nd, total, counter, s); break;
        default: persist_launch<32, US>(d, nd, total, counter, s); break;
    }
}

}  // namespace

struct BlkBatch {
    struct Part {
        int mat, launch;
        std::vector<int> ids;  // the launch's blocks in this group (empty: all of them)
    };
    struct Group {
        int L = 0, us = 0;
        std::vector<Part> parts;
        std::vector<BlkDesc> desc;
        DBuf<BlkDesc> d_desc;
        DBuf<int> d_ids;  // concatenated block subsets of the parts that have one
        DBuf<unsigned long long> counter;
        i64 total = 0;
    };
    std::vector<Matrix *> mats;
    std::vector<i64> nrhs;
    std::vector<Group> groups;
};

std::shared_ptr<BlkBatch> blk_batch_create(const std::vector<Matrix *> &mats, const std::vector<i64> &nrhs,
                                           const std::vector<char> &use) {
    auto bb = std::make_shared<BlkBatch>();
    bb->mats = mats;
    bb->nrhs = nrhs;
    std::map<std::pair<int, int>, int> gi;
    auto add = [&](int L, int us, BlkBatch::Part part) {
        auto key = std::make_pair(L, us);
        auto it = gi.find(key);
        if (it == gi.end()) {
            it = gi.emplace(key, static_cast<int>(bb->groups.size())).first;
            bb->groups.emplace_back();
            bb->groups.back().L = L;
            bb->groups.back().us = us;
        }
        bb->groups[it->second].parts.push_back(std::move(part));
    };
    for (size_t q = 0; q < mats.size(); ++q) {
        if (!use[q] || nrhs[q] <= 0) continue;
        const Blocked &B = mats[q]->blocked;
        for (size_t li = 0; li < B.launches.size(); ++li) {
            const Blocked::Launch &l = B.launches[li];
            if (l.n == 0) continue;
            if (l.L <= kTinyMaxL && l.us == kUsSmall && !B.h_block_ids.empty()) {
                std::vector<int> tiny, rest;
                for (i64 k = l.begin; k < l.begin + l.n; ++k) {
                    const int b = B.h_block_ids[k];
                    (B.h_us[b] <= kUsTiny ? tiny : rest).push_back(b);
                }
                if (!tiny.empty() && !rest.empty()) {
                    add(l.L, kUsTiny, {static_cast<int>(q), static_cast<int>(li), std::move(tiny)});
                    add(l.L, l.us, {static_cast<int>(q), static_cast<int>(li), std::move(rest)});
                    continue;
                }
                if (!tiny.empty()) {
                    add(l.L, kUsTiny, {static_cast<int>(q), static_cast<int>(li), {}});
                    continue;
                }
            }
            add(l.L, l.us, {static_cast<int>(q), static_cast<int>(li), {}});
        }
    }
    for (auto &g : bb->groups) {
        g.d_desc.alloc(g.parts.size());
        g.counter.alloc(1);
        g.desc.resize(g.parts.size());
        std::vector<int> ids;
        std::vector<i64> off(g.parts.size(), -1);
        for (size_t i = 0; i < g.parts.size(); ++i)
            if (!g.parts[i].ids.empty()) {
                off[i] = static_cast<i64>(ids.size());
                ids.insert(ids.end(), g.parts[i].ids.begin(), g.parts[i].ids.end());
            }
        g.d_ids.upload_vec(ids);
        i64 items = 0;
        for (size_t i = 0; i < g.parts.size(); ++i) {
            const int q = g.parts[i].mat;
            const Blocked &B = mats[q]->blocked;
            BlkDesc &D = g.desc[i];
            D.a = blk_args(B, B.launches[g.parts[i].launch], mats[q]->n_src);
            if (off[i] >= 0) {  // a subset of the launch's blocks
                D.a.blocks = g.d_ids.p + off[i];
                D.a.nbl = static_cast<i64>(g.parts[i].ids.size());
            }
            D.a.us = g.us;
            D.a.fchunk = std::min<i64>(g.us <= kUsTiny ? kTinyFChunk : kBatchFChunk, nrhs[q]);
            D.nrhs = nrhs[q];
            D.item_begin = items;
            items += D.a.nbl * ((nrhs[q] + D.a.fchunk - 1) / D.a.fchunk);
        }
        g.total = items;
    }
    AXGB_CUDA(cudaDeviceSynchronize());  // the block subsets are uploaded before any launch reads them
    return bb;
}

void blk_batch_set_fields(BlkBatch &bb, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy,
                          cudaStream_t s) {
    for (auto &g : bb.groups) {
        for (size_t i = 0; i < g.parts.size(); ++i) {
            const int q = g.parts[i].mat;
            g.desc[i].x = x[q];
            g.desc[i].ldx = ldx[q];
            g.desc[i].y = y[q];
            g.desc[i].ldy = ldy[q];
        }
        AXGB_CUDA(cudaMemcpyAsync(g.d_desc.p, g.desc.data(), sizeof(BlkDesc) * g.desc.size(), cudaMemcpyHostToDevice,
                                  s));
    }
}

// Class groups with the most items first, spread round-robin over the
// given streams (each group has its own work counter, so they may run
// concurrently; a persistent launch's tail then overlaps the next one).
void blk_batch_launch(BlkBatch &bb, const cudaStream_t *streams, int n_streams) {
    std::vector<int> order;
    for (size_t q = 0; q < bb.groups.size(); ++q)
        if (bb.groups[q].total > 0) order.push_back(static_cast<int>(q));
    std::stable_sort(order.begin(), order.end(),
                     [&](int a, int b) { return bb.groups[a].total > bb.groups[b].total; });
    for (size_t i = 0; i < order.size(); ++i) {
        auto &g = bb.groups[order[i]];
        cudaStream_t s = streams[i % n_streams];
        AXGB_CUDA(cudaMemsetAsync(g.counter.p, 0, sizeof(unsigned long long), s));
        if (g.us <= kUsTiny) {
            if (g.L <= 4)
                persist_launch<4, kUsTiny, kTinyT>(g.d_desc.p, static_cast<int>(g.desc.size()), g.total, g.counter.p, s);
            else
                persist_launch<8, kUsTiny, kTinyT>(g.d_desc.p, static_cast<int>(g.desc.size()), g.total, g.counter.p, s);
        } else if (g.us <= kUsSmall)
            persist_dispatch<kUsSmall>(g.L, g.d_desc.p, static_cast<int>(g.desc.size()), g.total, g.counter.p, s);
        else
            persist_dispatch<kUsLarge>(g.L, g.d_desc.p, static_cast<int>(g.desc.size()), g.total, g.counter.p, s);
    }
    AXGB_CUDA(cudaGetLastError());
}

void apply_blocked(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, int kind, int T, int ns,
                   i64 fchunk, cudaStream_t s, float *ylo, i64 ldylo) {
    Blocked &B = m.blocked;
    // Classes run concurrently on a small stream pool (fork/join through
    // events on the caller's stream, so the call stays stream-ordered and
    // capturable); the largest classes are issued first.
    std::lock_guard<std::mutex> lk(B.pool_mu);
    if (B.pool.empty()) {
        B.pool.resize(kPool);
        B.join.resize(kPool);
        for (int q = 0; q < kPool; ++q) {
            AXGB_CUDA(cudaStreamCreateWithFlags(&B.pool[q], cudaStreamNonBlocking));
            AXGB_CUDA(cudaEventCreateWithFlags(&B.join[q], cudaEventDisableTiming));
        }
        AXGB_CUDA(cudaEventCreateWithFlags(&B.fork, cudaEventDisableTiming));
    }
    AXGB_CUDA(cudaEventRecord(B.fork, s));
    const int used = static_cast<int>(std::min<size_t>(kPool, B.order.size()));
    for (int q = 0; q < used; ++q) AXGB_CUDA(cudaStreamWaitEvent(B.pool[q], B.fork, 0));
    for (size_t i = 0; i < B.order.size(); ++i) {
        const Blocked::Launch &l = B.launches[B.order[i]];
        cudaStream_t st = B.pool[i % kPool];
        if (T >= 8)
            launch_class<8>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, st, ylo, ldylo);
        else if (T >= 4)
            launch_class<4>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, st, ylo, ldylo);
        else
            launch_class<2>(B, l, kind, ns, x, ldx, y, ldy, nrhs, fchunk, st, ylo, ldylo);
    }
    for (int q = 0; q < used; ++q) {
        AXGB_CUDA(cudaEventRecord(B.join[q], B.pool[q]));
        AXGB_CUDA(cudaStreamWaitEvent(s, B.join[q], 0));
    }
    AXGB_CUDA(cudaGetLastError());
}


// ─── segmented layout: lane = field ────────────────────────────────────────
namespace {

constexpr int kSegRows = 8;            // rows per segment: one 32-byte sector of a field's outputs
constexpr int kSegW = 4;               // segments per group = consumer warps of a CTA
constexpr int kSegF = 32;              // fields per tile, one per lane
constexpr int kSegLd = kSegF + 1;      // floats per staged cell (the extra float spreads cells over banks)
constexpr int kSegUs[] = {160, 256};   // staged-cell buckets (launches)
static_assert(kSegW == kWarps, "segment groups reuse the slice grouping of four");

struct SegArgs {
    const int4 *grp, *slot;
    const uint4 *pairs;
    const int *cellmap, *gids;
    const unsigned *eoff;
    const float4 *ew;
    int *status;
    float *ylo;
    i64 ldylo;
    int max_ent;  // entry pairs of the largest group (shared-memory copy of a group's entries)
};

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

// One group (CTA) for all fields. Warp kSegW is the producer: for tile t (32
// fields) it copies field f of staged cell i to xs[slot][i][f] with 4-byte
// cp.async (lanes = consecutive staged cells, so the global side reads runs
// of the field and the shared side writes 33-float rows without conflicts)
// and arrives on the slot's `full` barrier as its copies land. Warp w < kSegW
// owns segment w of the group: per tile, lane = field, it sums the
// segment's row pairs entry by entry (both cells read conflict-free: the 32
// lanes read one 132-byte row), releases the slot, and writes the segment's
// 8 rows x 32 fields through a transpose buffer, 4 fields x 8 rows (four
// 32-byte sectors) per store. Bounded waits, as k_blk_ws.
template <int NS, int US>
__global__ void __launch_bounds__((kSegW + 1) * 32) k_seg(SegArgs a, const float *__restrict__ x, i64 ldx,
                                                          float *__restrict__ y, i64 ldy, i64 nrhs) {
    constexpr int kThreads = (kSegW + 1) * 32;
    constexpr int kOb = kSegRows + 1;  // transpose buffer row (field) stride
    extern __shared__ __align__(128) float smem[];
    float4 *ews = reinterpret_cast<float4 *>(smem);                           // [max_ent] the group's weights
    unsigned *eos = reinterpret_cast<unsigned *>(ews + a.max_ent);            // [max_ent] and cell offsets
    float *xs = reinterpret_cast<float *>(eos + a.max_ent);                   // [NS][US + 1][kSegLd]
    float *ob = xs + NS * (US + 1) * kSegLd;                                  // [kSegW][kSegF][kOb]
    int *cm = reinterpret_cast<int *>(ob + kSegW * kSegF * kOb);              // [US]
    __shared__ __align__(8) std::uint64_t full[NS], empty[NS];
    __shared__ volatile int abort_flag;
    const int g = a.gids[blockIdx.x];
    const int4 gd = a.grp[g];
    const int nc = gd.y;  // staged cells; slot nc is the zero cell
    const int e0 = gd.z, ne = gd.w;  // the group's entry pairs
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    for (int i = tid; i < nc; i += kThreads) cm[i] = a.cellmap[gd.x + i];
    for (int i = tid; i < ne; i += kThreads) {
        ews[i] = a.ew[e0 + i];
        eos[i] = a.eoff[e0 + i];
    }
    for (int q = tid; q < NS * kSegLd; q += kThreads)
        xs[(q / kSegLd) * (US + 1) * kSegLd + nc * kSegLd + q % kSegLd] = 0.f;
    if (tid == 0) {
        for (int st = 0; st < NS; ++st) {
            mbar_init(&full[st], 32);
            mbar_init(&empty[st], kSegW);
        }
        abort_flag = 0;
    }
    __syncthreads();
    const i64 ntile = (nrhs + kSegF - 1) / kSegF;
    if (warp == kSegW) {  // producer
        for (i64 t = 0; t < ntile; ++t) {
            const int st = static_cast<int>(t % NS);
            if (t >= NS && !mbar_wait_bounded(&empty[st], static_cast<unsigned>((t / NS - 1) & 1))) {
                abort_flag = 1;
                atomicExch(a.status, 1);
                break;
            }
            if (abort_flag) break;
            const i64 f0 = t * kSegF;
            const int nf = static_cast<int>(nrhs - f0 < kSegF ? nrhs - f0 : kSegF);
            const float *xt = x + f0 * ldx;
            float *dst = xs + st * (US + 1) * kSegLd;
            for (int i = lane; i < nc; i += 32) {
                const float *src = xt + cm[i];
                float *d = dst + i * kSegLd;
#pragma unroll 8
                for (int f = 0; f < nf; ++f) cp_async4(d + f, src + f * ldx);
            }
            cp_async_mbar_arrive(&full[st]);
        }
        cp_async_wait<0>();
        return;
    }
    const int4 sl = a.slot[static_cast<i64>(g) * kSegW + warp];
    const uint4 pr4 = a.pairs[static_cast<i64>(g) * kSegW + warp];
    const unsigned prs[4] = {pr4.x, pr4.y, pr4.z, pr4.w};
    float *obw = ob + warp * kSegF * kOb;
    const int r = lane & 7;
    const bool store_r = ((sl.z >> r) & 1) != 0;
    const i64 row = static_cast<i64>(sl.x) * kSegRows + r;
    for (i64 t = 0; t < ntile; ++t) {
        const int st = static_cast<int>(t % NS);
        if (!mbar_wait_bounded(&full[st], static_cast<unsigned>((t / NS) & 1))) {
            abort_flag = 1;
            atomicExch(a.status, 1);
            break;
        }
        const float *xl = xs + st * (US + 1) * kSegLd + lane;
        F2 acc[4], cnn[4];
        int e = sl.y - e0;
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const int len = static_cast<int>((prs[p] >> 8) & 63u);
            F2 s2 = pk(0.f, 0.f), c2 = pk(0.f, 0.f);
#pragma unroll 4
            for (int k = 0; k < len; ++k) {
                const unsigned u = eos[e + k];
                const float4 w = ews[e + k];
                cstep_pair(s2, c2, w, xl[u & 0xffffu], xl[u >> 16]);
            }
            e += len;
            acc[p] = s2;
            cnn[p] = c2;
        }
        __syncwarp();
        if (lane == 0) mbar_arrive(&empty[st]);  // the slot is no longer read by this warp
        const i64 f0 = t * kSegF;
        const int nf = static_cast<int>(nrhs - f0 < kSegF ? nrhs - f0 : kSegF);
#pragma unroll
        for (int p = 0; p < 4; ++p) {
            const unsigned pr = prs[p];
            if (!(pr & 128u)) continue;
            float ya, yb;
            upk(sub2(acc[p], cnn[p]), ya, yb);
            obw[lane * kOb + (pr & 7u)] = ya;
            if (pr & 64u) obw[lane * kOb + ((pr >> 3) & 7u)] = yb;
        }
        __syncwarp();
#pragma unroll
        for (int fb = 0; fb < kSegF / 4; ++fb) {
            const int f = 4 * fb + (lane >> 3);
            if (f < nf && store_r) y[(f0 + f) * ldy + row] = obw[f * kOb + r];
        }
        if (a.ylo) {  // low parts of the same outputs, through the same buffer
            __syncwarp();
#pragma unroll
            for (int p = 0; p < 4; ++p) {
                const unsigned pr = prs[p];
                if (!(pr & 128u)) continue;
                float ya, yb, sa, sb, ca, cb;
                upk(sub2(acc[p], cnn[p]), ya, yb);
                upk(acc[p], sa, sb);
                upk(cnn[p], ca, cb);
                obw[lane * kOb + (pr & 7u)] = sum_err(sa, -ca, ya);
                if (pr & 64u) obw[lane * kOb + ((pr >> 3) & 7u)] = sum_err(sb, -cb, yb);
            }
            __syncwarp();
#pragma unroll
            for (int fb = 0; fb < kSegF / 4; ++fb) {
                const int f = 4 * fb + (lane >> 3);
                if (f < nf && store_r) a.ylo[(f0 + f) * a.ldylo + row] = obw[f * kOb + r];
            }
        }
        __syncwarp();
    }
}

// Rows of at most 32 entries outside the groups: warp per (row, 32 fields),
// lane = field, entries in the layout's order (csum1).
__global__ void __launch_bounds__(256) k_seg_rows(const int *__restrict__ rows, const int *__restrict__ ptr,
                                                  const int *__restrict__ col, const float *__restrict__ hi,
                                                  const float *__restrict__ lo, i64 n, const float *__restrict__ x,
                                                  i64 ldx, float *__restrict__ y, i64 ldy, i64 nrhs, float *ylo,
                                                  i64 ldylo) {
    const i64 w = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const i64 i = w % n, fc = w / n;
    const i64 f = fc * 32 + (threadIdx.x & 31);
    if (fc * 32 >= nrhs || f >= nrhs) return;
    const int b = ptr[i], e = ptr[i + 1];
    const float *xf = x + f * ldx;
    float s = 0.f, c = 0.f;
    for (int k = b; k < e; ++k) csum1(s, c, hi[k], lo[k], __ldg(xf + col[k]));
    const float r = __fadd_rn(s, c);
    y[f * ldy + rows[i]] = r;
    if (ylo) ylo[f * ldylo + rows[i]] = sum_err(s, c, r);
}

template <int NS, int US>
void launch_seg_us(const SegArgs &a, i64 grid, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs,
                   cudaStream_t s) {
    const size_t bytes = sizeof(float) * (static_cast<size_t>(NS) * (US + 1) * kSegLd + kSegW * kSegF * (kSegRows + 1)) +
                         (sizeof(float4) + sizeof(unsigned)) * static_cast<size_t>(a.max_ent) + sizeof(int) * US;
    AXGB_CUDA(cudaFuncSetAttribute(k_seg<NS, US>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    k_seg<NS, US><<<static_cast<unsigned>(grid), (kSegW + 1) * 32, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

struct HostGroup {
    int segs[kSegW];
    int mask[kSegW];
    unsigned pr[kSegW][4];
    std::vector<int> cells;
    std::vector<unsigned> eoff;
    std::vector<float4> ew;
    int slot_ent[kSegW];  // entry pairs of each slot (relative)
    bool fallback = false;
    std::vector<int> fb_rows;
};

}  // namespace

void build_segmented(Matrix &m, cudaStream_t s) {
    Segmented &G = m.seg;
    if (G.built) return;
    build_blocked(m, s);  // the split entry order (split_perm)
    const i64 n = m.n_dst, nnz = m.nnz;
    std::vector<int> rp(n + 1), col(std::max<i64>(1, nnz)), perm(std::max<i64>(1, nnz));
    std::vector<double> val(std::max<i64>(1, nnz));
    AXGB_CUDA(cudaMemcpy(rp.data(), m.row_ptr.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost));
    if (nnz) {
        AXGB_CUDA(cudaMemcpy(col.data(), m.col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
        AXGB_CUDA(cudaMemcpy(val.data(), m.val.p, sizeof(double) * nnz, cudaMemcpyDeviceToHost));
        AXGB_CUDA(cudaMemcpy(perm.data(), m.split_perm.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    }
    const i64 nsg = (n + kSegRows - 1) / kSegRows;
    auto groups = group_slices(nsg, m.seg_xyz);  // four nearby segments per group (consecutive without a hint)
    const i64 ng = static_cast<i64>(groups.size());
    const int usmax = kSegUs[sizeof(kSegUs) / sizeof(kSegUs[0]) - 1];
    std::vector<HostGroup> hg(ng);
    auto split = [&](int q, float &h, float &l) {
        h = static_cast<float>(val[q]);
        l = static_cast<float>(val[q] - static_cast<double>(h));
    };
    parallel_for_host(ng, [&](i64 g0, i64 g1) {
        std::vector<int> rows;
        for (i64 g = g0; g < g1; ++g) {
            HostGroup &H = hg[g];
            H.cells.clear();
            for (int w = 0; w < kSegW; ++w) {
                H.segs[w] = groups[g][w];
                H.mask[w] = 0;
                for (int p = 0; p < 4; ++p) H.pr[w][p] = 0;
                H.slot_ent[w] = 0;
                const int sg = groups[g][w];
                if (sg < 0) continue;
                for (int r = 0; r < kSegRows; ++r) {
                    const i64 row = static_cast<i64>(sg) * kSegRows + r;
                    if (row >= n || rp[row + 1] - rp[row] > 32) continue;
                    for (int q = rp[row]; q < rp[row + 1]; ++q) H.cells.push_back(col[q]);
                }
            }
            std::sort(H.cells.begin(), H.cells.end());
            H.cells.erase(std::unique(H.cells.begin(), H.cells.end()), H.cells.end());
            const int nc = static_cast<int>(H.cells.size());
            if (nc > usmax) {  // too many staged cells: the group's rows go to the fallback kernel
                H.fallback = true;
                for (int w = 0; w < kSegW; ++w) {
                    const int sg = groups[g][w];
                    if (sg < 0) continue;
                    for (int r = 0; r < kSegRows; ++r) {
                        const i64 row = static_cast<i64>(sg) * kSegRows + r;
                        if (row < n && rp[row + 1] - rp[row] <= 32) H.fb_rows.push_back(static_cast<int>(row));
                    }
                }
                H.cells.clear();
                continue;
            }
            auto pos = [&](int c) {
                return static_cast<unsigned>(std::lower_bound(H.cells.begin(), H.cells.end(), c) - H.cells.begin());
            };
            for (int w = 0; w < kSegW; ++w) {
                const int sg = groups[g][w];
                if (sg < 0) continue;
                rows.clear();
                for (int r = 0; r < kSegRows; ++r) {
                    const i64 row = static_cast<i64>(sg) * kSegRows + r;
                    if (row < n && rp[row + 1] - rp[row] <= 32) rows.push_back(r);
                }
                std::stable_sort(rows.begin(), rows.end(), [&](int ra, int rb) {
                    const i64 a0 = static_cast<i64>(sg) * kSegRows + ra, b0 = static_cast<i64>(sg) * kSegRows + rb;
                    return rp[a0 + 1] - rp[a0] > rp[b0 + 1] - rp[b0];
                });
                const int before = static_cast<int>(H.eoff.size());
                for (size_t p = 0; p < rows.size(); p += 2) {
                    const int ra = rows[p], rb = p + 1 < rows.size() ? rows[p + 1] : -1;
                    const i64 ra0 = static_cast<i64>(sg) * kSegRows + ra;
                    const int la = rp[ra0 + 1] - rp[ra0];
                    const i64 rb0 = rb >= 0 ? static_cast<i64>(sg) * kSegRows + rb : -1;
                    const int lb = rb >= 0 ? rp[rb0 + 1] - rp[rb0] : 0;
                    H.mask[w] |= 1 << ra;
                    if (rb >= 0) H.mask[w] |= 1 << rb;
                    H.pr[w][p / 2] = static_cast<unsigned>(ra) | (static_cast<unsigned>(rb >= 0 ? rb : 0) << 3) |
                                     (rb >= 0 ? 64u : 0u) | 128u | (static_cast<unsigned>(la) << 8);
                    for (int k = 0; k < la; ++k) {
                        const int qa = perm[rp[ra0] + k];
                        unsigned ua = pos(col[qa]) * kSegLd, ub = static_cast<unsigned>(nc) * kSegLd;
                        float ha, la_, hb = 0.f, lb_ = 0.f;
                        split(qa, ha, la_);
                        if (k < lb) {
                            const int qb = perm[rp[rb0] + k];
                            ub = pos(col[qb]) * kSegLd;
                            split(qb, hb, lb_);
                        }
                        H.eoff.push_back(ua | (ub << 16));
                        H.ew.push_back(make_float4(ha, hb, -la_, -lb_));
                    }
                }
                H.slot_ent[w] = static_cast<int>(H.eoff.size()) - before;
            }
        }
    });
    // flatten
    std::vector<int4> grp(ng), slot(ng * kSegW);
    std::vector<uint4> pairs(ng * kSegW);
    std::vector<int> cellmap, fb_rows;
    std::vector<unsigned> eoff;
    std::vector<float4> ew;
    std::vector<std::vector<int>> bucket(sizeof(kSegUs) / sizeof(kSegUs[0]));
    for (i64 g = 0; g < ng; ++g) {
        HostGroup &H = hg[g];
        grp[g] = make_int4(static_cast<int>(cellmap.size()), static_cast<int>(H.cells.size()),
                           static_cast<int>(eoff.size()), static_cast<int>(H.eoff.size()));
        if (!H.fallback) G.max_ent = std::max(G.max_ent, static_cast<int>(H.eoff.size()));
        int ent = static_cast<int>(eoff.size());
        for (int w = 0; w < kSegW; ++w) {
            slot[g * kSegW + w] = make_int4(H.fallback ? -1 : H.segs[w], ent, H.fallback ? 0 : H.mask[w], 0);
            pairs[g * kSegW + w] = make_uint4(H.pr[w][0], H.pr[w][1], H.pr[w][2], H.pr[w][3]);
            ent += H.slot_ent[w];
        }
        if (H.fallback) {
            fb_rows.insert(fb_rows.end(), H.fb_rows.begin(), H.fb_rows.end());
            continue;
        }
        cellmap.insert(cellmap.end(), H.cells.begin(), H.cells.end());
        eoff.insert(eoff.end(), H.eoff.begin(), H.eoff.end());
        ew.insert(ew.end(), H.ew.begin(), H.ew.end());
        int b = 0;
        while (kSegUs[b] < static_cast<int>(H.cells.size())) ++b;
        bucket[b].push_back(static_cast<int>(g));
        std::vector<int>().swap(H.cells);
        std::vector<unsigned>().swap(H.eoff);
        std::vector<float4>().swap(H.ew);
    }
    std::vector<int> gids;
    G.launches.clear();
    G.max_ent = std::max(G.max_ent, 1);
    for (size_t b = 0; b < bucket.size(); ++b) {
        if (bucket[b].empty()) continue;
        G.launches.push_back({kSegUs[b], static_cast<i64>(gids.size()), static_cast<i64>(bucket[b].size())});
        gids.insert(gids.end(), bucket[b].begin(), bucket[b].end());
    }
    // fallback short rows and long rows, row-contiguous in the split order (original numbering)
    auto rowlist = [&](const std::vector<int> &rl, DBuf<int> &drow, DBuf<int> &dptr, DBuf<int> &dcol,
                       DBuf<float> &dhi, DBuf<float> &dlo) {
        std::vector<int> ptr(1, 0), c;
        std::vector<float> h, l;
        for (int r : rl) {
            for (int k = rp[r]; k < rp[r + 1]; ++k) {
                const int q = perm[k];
                float hh, ll;
                split(q, hh, ll);
                c.push_back(col[q]);
                h.push_back(hh);
                l.push_back(ll);
            }
            ptr.push_back(static_cast<int>(c.size()));
        }
        drow.upload_vec(rl, s);
        dptr.upload_vec(ptr, s);
        dcol.upload_vec(c, s);
        dhi.upload_vec(h, s);
        dlo.upload_vec(l, s);
    };
    std::vector<int> long_rows;
    for (i64 r = 0; r < n; ++r)
        if (rp[r + 1] - rp[r] > 32) long_rows.push_back(static_cast<int>(r));
    rowlist(fb_rows, G.fb_row, G.fb_ptr, G.fb_col, G.fb_hi, G.fb_lo);
    rowlist(long_rows, G.l_row, G.l_ptr, G.l_col, G.l_hi, G.l_lo);
    G.n_fb = static_cast<i64>(fb_rows.size());
    G.n_long = static_cast<i64>(long_rows.size());
    G.grp.upload_vec(grp, s);
    G.slot.upload_vec(slot, s);
    G.pairs.upload_vec(pairs, s);
    G.cellmap.upload_vec(cellmap, s);
    G.gids.upload_vec(gids, s);
    G.eoff.upload_vec(eoff, s);
    G.ew.upload_vec(ew, s);
    if (!G.status.p) {
        G.status.alloc(1);
        G.status.zero(s);
    }
    G.n_groups = ng;
    AXGB_CUDA(cudaStreamSynchronize(s));
    G.built = true;
}

void apply_segmented(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s, float *ylo,
                     i64 ldylo, int ns) {
    Segmented &G = m.seg;
    if (nrhs <= 0) return;
    std::lock_guard<std::mutex> lk(G.pool_mu);
    const int nl = static_cast<int>(G.launches.size()) + (G.n_fb > 0 ? 1 : 0) + (G.n_long > 0 ? 1 : 0);
    if (G.pool.empty()) {
        G.pool.resize(3);
        G.join.resize(3);
        for (int q = 0; q < 3; ++q) {
            AXGB_CUDA(cudaStreamCreateWithFlags(&G.pool[q], cudaStreamNonBlocking));
            AXGB_CUDA(cudaEventCreateWithFlags(&G.join[q], cudaEventDisableTiming));
        }
        AXGB_CUDA(cudaEventCreateWithFlags(&G.fork, cudaEventDisableTiming));
    }
    const int used = std::min(3, nl);
    AXGB_CUDA(cudaEventRecord(G.fork, s));
    for (int q = 0; q < used; ++q) AXGB_CUDA(cudaStreamWaitEvent(G.pool[q], G.fork, 0));
    int q = 0;
    SegArgs a{G.grp.p, G.slot.p, G.pairs.p, G.cellmap.p, nullptr, G.eoff.p, G.ew.p, G.status.p, ylo, ldylo,
              G.max_ent};
    // the largest bucket first: it holds the groups with the most work
    for (int li = static_cast<int>(G.launches.size()) - 1; li >= 0; --li) {
        const Segmented::Launch &l = G.launches[li];
        a.gids = G.gids.p + l.begin;
        cudaStream_t st = G.pool[q++ % 3];
        if (l.usmax <= kSegUs[0]) {
            if (ns >= 3)
                launch_seg_us<3, kSegUs[0]>(a, l.n, x, ldx, y, ldy, nrhs, st);
            else
                launch_seg_us<2, kSegUs[0]>(a, l.n, x, ldx, y, ldy, nrhs, st);
        } else {
            if (ns >= 3)
                launch_seg_us<3, kSegUs[1]>(a, l.n, x, ldx, y, ldy, nrhs, st);
            else
                launch_seg_us<2, kSegUs[1]>(a, l.n, x, ldx, y, ldy, nrhs, st);
        }
    }
    if (G.n_fb > 0) {
        const i64 warps = G.n_fb * ((nrhs + 31) / 32);
        k_seg_rows<<<nblk(warps * 32, 256), 256, 0, G.pool[q++ % 3]>>>(G.fb_row.p, G.fb_ptr.p, G.fb_col.p, G.fb_hi.p,
                                                                      G.fb_lo.p, G.n_fb, x, ldx, y, ldy, nrhs, ylo,
                                                                      ldylo);
    }
    if (G.n_long > 0)
        launch_long_rows(G.l_row.p, G.l_ptr.p, G.l_col.p, G.l_hi.p, G.l_lo.p, G.n_long, x, ldx, y, ldy, nrhs,
                         G.pool[q++ % 3], ylo, ldylo);
    AXGB_CUDA(cudaGetLastError());
    for (int k = 0; k < used; ++k) {
        AXGB_CUDA(cudaEventRecord(G.join[k], G.pool[k]));
        AXGB_CUDA(cudaStreamWaitEvent(s, G.join[k], 0));
    }
}

}  // namespace axgb
