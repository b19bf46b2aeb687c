// Sparse weight apply on the device: y[f] = S x[f] for fields f < nrhs,
// fields laid out [f][cell] (the LayoutLeft (n_cells, n_vars) of
// batch_apply, libs/axis/include/axis/solver/apply.hpp:275-343).
//
// Layout: 32-row sliced ELL built once per matrix from the CSR. One warp
// owns one slice (one row per lane): it loads its row's entries (column,
// FP64 weight or FP32 hi+lo pair) once into registers, then streams the
// fields of its work item through them, so the matrix is read once per
// item while the gathers of x are the only per-field traffic. Slices are
// grouped by length class (<=8, <=16, <=32, <=64 entries) so each class
// runs a kernel with a fixed register array; longer slices take a kernel
// that re-reads its entries from global memory.
//
// Split FP32 path: weights w = hi + lo (hi = fp32(w), lo = fp32(w - hi));
// per entry the product hi*x is split exactly (fma), lo*x is added to the
// error term, and the running sum is carried with Knuth's TwoSum, so each
// output is the compensated sum rounded once to FP32. Two fields are
// processed together with packed f32x2 instructions.
//
// Work items are (field tile, slice), tile-major: all warps sweep the same
// tile of fields at once, so the source values they gather stay in L2
// between neighbouring slices. The tile width and the number of fields per
// thread iteration are the tuning knobs (see the autotuner in api.cpp).
#include <algorithm>

#include "internal.hpp"

namespace axgb {

struct Batch {
    struct Desc {
        const int *base, *len, *rlen, *col;
        const float *hi, *lo;
        i64 n_rows, n_slices;
        const float *x;
        i64 ldx;
        float *y;
        i64 ldy;
        i64 nrhs;
        i64 tile;
        i64 n_tiles;
        i64 item_begin;  // first global item of this matrix
    };
    std::vector<std::shared_ptr<Matrix>> mats;
    std::vector<i64> nrhs;
    std::vector<Desc> desc;
    DBuf<Desc> d_desc;
    DBuf<unsigned long long> counter;
    i64 total_items = 0;
    int blocks = 0;
    // graph per stream, replayed while descriptors are updated in place
    std::map<cudaStream_t, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
    std::vector<const void *> last_ptrs;
    std::mutex mu;
    ~Batch() {
        for (auto &g : graphs) {
            cudaGraphExecDestroy(g.second.second);
            cudaGraphDestroy(g.second.first);
        }
    }
};

namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// ─── packed f32x2 helpers ──────────────────────────────────────────────────

struct F2 {
    unsigned long long v;
};
__device__ __forceinline__ F2 pk(float a, float b) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(a), "f"(b));
    return r;
}
__device__ __forceinline__ void upk(F2 r, float &a, float &b) { asm("mov.b64 {%0, %1}, %2;" : "=f"(a), "=f"(b) : "l"(r.v)); }
__device__ __forceinline__ F2 add2(F2 a, F2 b) {
    F2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 sub2(F2 a, F2 b) {
    F2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 mul2(F2 a, F2 b) {
    F2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ F2 fma2(F2 a, F2 b, F2 c) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}

// One compensated step for one field: s + c accumulates (hi + lo) * x.
__device__ __forceinline__ void csum1(float &s, float &c, float h, float l, float x) {
    float p = __fmul_rn(h, x);
    float pe = __fmaf_rn(h, x, -p);
    float q = __fmaf_rn(l, x, pe);
    float t = __fadd_rn(s, p);
    float bp = __fsub_rn(t, s);
    float e = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
    s = t;
    c = __fadd_rn(c, __fadd_rn(e, q));
}

// Same for two fields at once; hn = -hi (so mul gives -p exactly).
__device__ __forceinline__ void csum2(F2 &s, F2 &c, F2 h, F2 hn, F2 l, F2 x) {
    F2 pn = mul2(hn, x);
    F2 pe = fma2(h, x, pn);
    F2 q = fma2(l, x, pe);
    F2 t = sub2(s, pn);
    F2 bp = sub2(t, s);
    F2 a2 = sub2(s, sub2(t, bp));
    F2 a3 = add2(pn, bp);
    F2 e = sub2(a2, a3);
    s = t;
    c = add2(c, add2(e, q));
}

// Same arithmetic as csum2 (bitwise identical results) but without a
// negated-weight register pair: the product error is formed with -x and
// the compensation is carried negated (cn = -c); the row value is s - cn.
__device__ __forceinline__ void cstep2(F2 &s, F2 &cn, F2 h, F2 l, F2 x, F2 mone) {
    F2 nx = mul2(x, mone);
    F2 p = mul2(h, x);
    F2 pen = fma2(h, nx, p);  // p - h*x = -(product error), exact
    F2 t = add2(s, p);
    F2 bp = sub2(t, s);
    F2 a2 = sub2(s, sub2(t, bp));
    F2 a3 = sub2(p, bp);
    F2 e = add2(a2, a3);      // TwoSum error
    F2 u1 = fma2(l, nx, pen); // -(lo*x + product error)
    cn = add2(cn, sub2(u1, e));
    s = t;
}

struct SellArgs {
    const int *ids;
    i64 n_ids;
    const int *base, *len, *rlen, *col;
    const float *hi, *lo;
    const double *w64;
    i64 n_rows;
};

__device__ __forceinline__ float ldg_f(const float *p) { return __ldg(p); }

// ─── split-FP32 kernel ─────────────────────────────────────────────────────
// L > 0: entries cached in registers (slice length <= L).
// L == 0: entries re-read from global memory (long slices).
template <int L, int U>
__global__ void __launch_bounds__(256) k_split(SellArgs a, const float *__restrict__ x, i64 ldx, float *__restrict__ y,
                                               i64 ldy, i64 nrhs, i64 tile) {
    const int lane = threadIdx.x & 31;
    const i64 item = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const i64 n_tiles = (nrhs + tile - 1) / tile;
    if (item >= n_tiles * a.n_ids) return;
    const i64 t = item / a.n_ids;
    const int sid = a.ids[item - t * a.n_ids];
    const i64 row = static_cast<i64>(sid) * 32 + lane;
    const int base = a.base[sid];
    const int rl = a.rlen[static_cast<i64>(sid) * 32 + lane];
    const i64 f0 = t * tile, f1 = min(f0 + tile, nrhs);
    const bool store = row < a.n_rows;
    if constexpr (L > 0) {
        int c[L];
        float h[L], lw[L];
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (k < rl) {
                int e = base + k * 32 + lane;
                c[k] = a.col[e];
                h[k] = a.hi[e];
                lw[k] = a.lo[e];
            } else {
                c[k] = 0;
                h[k] = 0.f;
                lw[k] = 0.f;
            }
        }
        i64 f = f0;
        if constexpr (U >= 2) {
            F2 hp[L], hn[L], lp[L];
#pragma unroll
            for (int k = 0; k < L; ++k) {
                hp[k] = pk(h[k], h[k]);
                hn[k] = pk(-h[k], -h[k]);
                lp[k] = pk(lw[k], lw[k]);
            }
            for (; f + U <= f1; f += U) {
                F2 s[U / 2], cc[U / 2];
#pragma unroll
                for (int u = 0; u < U / 2; ++u) {
                    s[u] = pk(0.f, 0.f);
                    cc[u] = pk(0.f, 0.f);
                }
                const float *xf = x + f * ldx;
#pragma unroll
                for (int k = 0; k < L; ++k) {
                    if (k < rl) {
#pragma unroll
                        for (int u = 0; u < U / 2; ++u) {
                            float xa = ldg_f(xf + (2 * u) * ldx + c[k]);
                            float xb = ldg_f(xf + (2 * u + 1) * ldx + c[k]);
                            csum2(s[u], cc[u], hp[k], hn[k], lp[k], pk(xa, xb));
                        }
                    }
                }
                if (store) {
#pragma unroll
                    for (int u = 0; u < U / 2; ++u) {
                        F2 r = add2(s[u], cc[u]);
                        float ra, rb;
                        upk(r, ra, rb);
                        y[(f + 2 * u) * ldy + row] = ra;
                        y[(f + 2 * u + 1) * ldy + row] = rb;
                    }
                }
            }
        }
        for (; f < f1; ++f) {
            float s = 0.f, cc = 0.f;
            const float *xf = x + f * ldx;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < rl) csum1(s, cc, h[k], lw[k], ldg_f(xf + c[k]));
            if (store) y[f * ldy + row] = __fadd_rn(s, cc);
        }
    } else {
        for (i64 f = f0; f < f1; ++f) {
            float s = 0.f, cc = 0.f;
            const float *xf = x + f * ldx;
            for (int k = 0; k < rl; ++k) {
                int e = base + k * 32 + lane;
                csum1(s, cc, a.hi[e], a.lo[e], ldg_f(xf + a.col[e]));
            }
            if (store) y[f * ldy + row] = __fadd_rn(s, cc);
        }
    }
}

// ─── FP64 kernel ───────────────────────────────────────────────────────────
template <int L, int U>
__global__ void __launch_bounds__(256) k_f64(SellArgs a, const double *__restrict__ x, i64 ldx, double *__restrict__ y,
                                             i64 ldy, i64 nrhs, i64 tile) {
    const int lane = threadIdx.x & 31;
    const i64 item = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const i64 n_tiles = (nrhs + tile - 1) / tile;
    if (item >= n_tiles * a.n_ids) return;
    const i64 t = item / a.n_ids;
    const int sid = a.ids[item - t * a.n_ids];
    const i64 row = static_cast<i64>(sid) * 32 + lane;
    const int base = a.base[sid];
    const int rl = a.rlen[static_cast<i64>(sid) * 32 + lane];
    const i64 f0 = t * tile, f1 = min(f0 + tile, nrhs);
    const bool store = row < a.n_rows;
    if constexpr (L > 0) {
        int c[L];
        double w[L];
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (k < rl) {
                int e = base + k * 32 + lane;
                c[k] = a.col[e];
                w[k] = a.w64[e];
            } else {
                c[k] = 0;
                w[k] = 0.0;
            }
        }
        i64 f = f0;
        for (; f + U <= f1; f += U) {
            double s[U];
#pragma unroll
            for (int u = 0; u < U; ++u) s[u] = 0.0;
            const double *xf = x + f * ldx;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < rl) {
#pragma unroll
                    for (int u = 0; u < U; ++u) s[u] = fma(w[k], __ldg(xf + u * ldx + c[k]), s[u]);
                }
            if (store) {
#pragma unroll
                for (int u = 0; u < U; ++u) y[(f + u) * ldy + row] = s[u];
            }
        }
        for (; f < f1; ++f) {
            double s = 0.0;
            const double *xf = x + f * ldx;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < rl) s = fma(w[k], __ldg(xf + c[k]), s);
            if (store) y[f * ldy + row] = s;
        }
    } else {
        for (i64 f = f0; f < f1; ++f) {
            double s = 0.0;
            const double *xf = x + f * ldx;
            for (int k = 0; k < rl; ++k) {
                int e = base + k * 32 + lane;
                s = fma(a.w64[e], __ldg(xf + a.col[e]), s);
            }
            if (store) y[f * ldy + row] = s;
        }
    }
}

// ─── layout build ──────────────────────────────────────────────────────────

__global__ void k_slice_len(const int *rp, i64 n_rows, i64 n_slices, int *len) {
    i64 s = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (s >= n_slices) return;
    int m = 0;
    for (int q = 0; q < 32; ++q) {
        i64 r = s * 32 + q;
        if (r < n_rows) m = max(m, rp[r + 1] - rp[r]);
    }
    len[s] = m * 32;  // entries of the slice; scanned into base
}

__global__ void k_sell_fill(const int *rp, const int *ccol, const double *val, i64 n_rows, i64 n_slices,
                            const int *base, const int *slen32, int *rlen, int *col, float *hi, float *lo,
                            double *w64) {
    i64 r = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n_slices * 32) return;
    i64 s = r >> 5;
    int lane = static_cast<int>(r & 31);
    int L = slen32[s] / 32;
    int b = base[s];
    int n = 0, r0 = 0;
    if (r < n_rows) {
        r0 = rp[r];
        n = rp[r + 1] - r0;
    }
    rlen[r] = n;
    int last = n > 0 ? ccol[r0 + n - 1] : 0;
    for (int k = 0; k < L; ++k) {
        int e = b + k * 32 + lane;
        if (k < n) {
            double w = val[r0 + k];
            col[e] = ccol[r0 + k];
            if (hi) {
                float h = __double2float_rn(w);
                hi[e] = h;
                lo[e] = __double2float_rn(w - static_cast<double>(h));
            }
            if (w64) w64[e] = w;
        } else {
            col[e] = last;
            if (hi) {
                hi[e] = 0.f;
                lo[e] = 0.f;
            }
            if (w64) w64[e] = 0.0;
        }
    }
}

void build_sell(Matrix &m, int fmt, cudaStream_t s) {
    Sell &S = fmt == 0 ? m.sell64 : m.sell32;
    if (S.built) return;
    const i64 n_rows = m.n_dst;
    const i64 n_slices = (n_rows + 31) / 32;
    DBuf<int> slen32(n_slices), base(n_slices + 1);
    if (n_slices > 0) {
        k_slice_len<<<nblk(n_slices, 256), 256, 0, s>>>(m.row_ptr.p, n_rows, n_slices, slen32.p);
        AXGB_CUDA(cudaGetLastError());
    }
    scan_exclusive_i32(slen32.p, base.p, n_slices, s);
    int total = 0;
    AXGB_CUDA(cudaMemcpy(&total, base.p + n_slices, sizeof(int), cudaMemcpyDeviceToHost));
    S.n_slices = n_slices;
    S.n_entries = total;
    S.col.alloc(total);
    S.len.alloc(n_slices);
    S.base = std::move(base);
    DBuf<int> rlen(n_slices * 32);
    if (fmt == 1) {
        S.hi.alloc(total);
        S.lo.alloc(total);
    } else {
        S.w64.alloc(total);
    }
    if (n_slices > 0) {
        k_sell_fill<<<nblk(n_slices * 32, 256), 256, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, n_rows, n_slices,
                                                            S.base.p, slen32.p, rlen.p, S.col.p,
                                                            fmt == 1 ? S.hi.p : nullptr, fmt == 1 ? S.lo.p : nullptr,
                                                            fmt == 0 ? S.w64.p : nullptr);
        AXGB_CUDA(cudaGetLastError());
    }
    // length classes on the host
    std::vector<int> h_len(n_slices);
    if (n_slices) AXGB_CUDA(cudaMemcpy(h_len.data(), slen32.p, sizeof(int) * n_slices, cudaMemcpyDeviceToHost));
    const int bounds[5] = {8, 16, 32, 64, 1 << 30};
    std::vector<std::vector<int>> cls(5);
    for (i64 q = 0; q < n_slices; ++q) {
        int L = h_len[q] / 32;
        int c = 0;
        while (L > bounds[c]) ++c;
        cls[c].push_back(static_cast<int>(q));
    }
    std::vector<int> ids;
    S.class_begin.assign(6, 0);
    S.class_maxlen.assign(5, 0);
    for (int c = 0; c < 5; ++c) {
        S.class_begin[c] = static_cast<i64>(ids.size());
        for (int q : cls[c]) S.class_maxlen[c] = std::max(S.class_maxlen[c], h_len[q] / 32);
        ids.insert(ids.end(), cls[c].begin(), cls[c].end());
    }
    S.class_begin[5] = static_cast<i64>(ids.size());
    S.class_ids.upload(ids.data(), ids.size(), s);
    S.h_slice_len.resize(n_slices);
    for (i64 q = 0; q < n_slices; ++q) S.h_slice_len[q] = h_len[q] / 32;
    // keep row lengths in the len buffer's companion: store rlen in 'len' slot
    S.len = std::move(rlen);
    AXGB_CUDA(cudaStreamSynchronize(s));
    S.built = true;
}

SellArgs sell_args(const Matrix &m, const Sell &S, int cls) {
    SellArgs a;
    a.ids = S.class_ids.p + S.class_begin[cls];
    a.n_ids = S.class_begin[cls + 1] - S.class_begin[cls];
    a.base = S.base.p;
    a.len = nullptr;
    a.rlen = S.len.p;
    a.col = S.col.p;
    a.hi = S.hi.p;
    a.lo = S.lo.p;
    a.w64 = S.w64.p;
    a.n_rows = m.n_dst;
    return a;
}

template <int L>
void launch_split(const SellArgs &a, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, i64 tile, int U,
                  cudaStream_t s) {
    i64 items = ((nrhs + tile - 1) / tile) * a.n_ids;
    if (items == 0) return;
    unsigned blocks = nblk(items * 32, 256);
    if (U >= 4)
        k_split<L, 4><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
    else if (U >= 2)
        k_split<L, 2><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
    else
        k_split<L, 1><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
}

template <int L>
void launch_f64(const SellArgs &a, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, i64 tile, cudaStream_t s) {
    i64 items = ((nrhs + tile - 1) / tile) * a.n_ids;
    if (items == 0) return;
    unsigned blocks = nblk(items * 32, 256);
    if (nrhs >= 2)
        k_f64<L, 2><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
    else
        k_f64<L, 1><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
}

// ─── conservation ──────────────────────────────────────────────────────────

template <class T>
__global__ void k_integral(const T *f, const double *area, const double *frac, i64 n, int mode, double *partial) {
    // mode 0: sum f*area*frac; 1: sum over frac != 0 of f*area (DstArea)
    __shared__ double sh[256];
    double acc = 0.0;
    for (i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<i64>(gridDim.x) * blockDim.x) {
        double v = static_cast<double>(f[i]);
        if (mode == 0)
            acc += v * area[i] * frac[i];
        else if (frac[i] != 0.0)
            acc += v * area[i];
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = 128; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

template <class T>
double integral(const T *f, const double *area, const double *frac, i64 n, int mode, cudaStream_t s) {
    const int blocks = 1024;
    DBuf<double> part(blocks);
    k_integral<T><<<blocks, 256, 0, s>>>(f, area, frac, n, mode, part.p);
    AXGB_CUDA(cudaGetLastError());
    std::vector<double> h(blocks);
    AXGB_CUDA(cudaMemcpyAsync(h.data(), part.p, sizeof(double) * blocks, cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaStreamSynchronize(s));
    double acc = 0.0;
    for (double v : h) acc += v;
    return acc;
}

// ─── staged split-FP32 kernel ──────────────────────────────────────────────
// One CTA owns a block of 128 rows (4 slices). The block's unique source
// columns are staged per field into shared memory with cp.async (coalesced:
// the column list is sorted), double-buffered over tiles of T fields, and
// each thread reduces its row from shared memory with its entries (16-bit
// local column, hi, lo) held in registers.

constexpr int kSR = 128;            // rows per staged block
constexpr int kStagedMaxU = 2048;   // unique columns a block may stage (139 KB of smem at T = 8)

__device__ __forceinline__ void cp_async4(void *smem, const void *gmem) {
    unsigned sa = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;" ::"n"(N) : "memory");
}

// Slice of warp w in staged block b (-1 = none).
__device__ __forceinline__ int block_slice(const int4 *bs, int b, int w) {
    int4 v = bs[b];
    return w == 0 ? v.x : (w == 1 ? v.y : (w == 2 ? v.z : v.w));
}

struct StagedArgs {
    const int4 *bslices;
    const int *blocks;
    i64 n_blocks;
    const int *base, *rlen;
    const unsigned short *lidx;
    const float *hi, *lo;
    const int *ucol, *ustart, *ucount;
    i64 n_rows, n_slices;
    int ustride;
};

template <int L, int T>
__global__ void __launch_bounds__(kSR) k_staged(StagedArgs a, const float *__restrict__ x, i64 ldx,
                                               float *__restrict__ y, i64 ldy, i64 nrhs) {
    extern __shared__ __align__(16) float smem[];
    const int US = a.ustride;
    int *ucs = reinterpret_cast<int *>(smem);
    float *xs = smem + US;  // [2][T][US]
    const int b = a.blocks[blockIdx.x];
    const int U = a.ucount[b];
    const int *ug = a.ucol + a.ustart[b];
    for (int u = threadIdx.x; u < U; u += kSR) ucs[u] = ug[u];
    const int lane = threadIdx.x & 31;
    const i64 sid = block_slice(a.bslices, b, threadIdx.x >> 5);
    const i64 row = sid * 32 + lane;
    int rl = 0, base = 0;
    if (sid >= 0) {
        base = a.base[sid];
        rl = a.rlen[row];
    }
    int li[L];
    float h[L], lw[L];
#pragma unroll
    for (int k = 0; k < L; ++k) {
        if (k < rl) {
            int e = base + k * 32 + lane;
            li[k] = a.lidx[e];
            h[k] = a.hi[e];
            lw[k] = a.lo[e];
        } else {
            li[k] = 0;
            h[k] = 0.f;
            lw[k] = 0.f;
        }
    }
    const bool store = sid >= 0 && row < a.n_rows;
    __syncthreads();
    const i64 ntile = (nrhs + T - 1) / T;
    auto stage = [&](i64 t, float *dst) {
#pragma unroll
        for (int f = 0; f < T; ++f) {
            i64 fg = t * T + f;
            if (fg < nrhs) {
                const float *xf = x + fg * ldx;
                for (int u = threadIdx.x; u < U; u += kSR) cp_async4(dst + f * US + u, xf + ucs[u]);
            }
        }
        cp_async_commit();
    };
    stage(0, xs);
    for (i64 t = 0; t < ntile; ++t) {
        const float *cur = xs + (t & 1) * T * US;
        if (t + 1 < ntile) {
            stage(t + 1, xs + ((t + 1) & 1) * T * US);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const i64 f0 = t * T;
#pragma unroll
        for (int f = 0; f < T; f += 2) {
            if (f0 + f + 1 < nrhs) {
                F2 sa = pk(0.f, 0.f), ca = pk(0.f, 0.f);
                const float *c0 = cur + f * US, *c1 = cur + (f + 1) * US;
#pragma unroll
                for (int k = 0; k < L; ++k)
                    if (k < rl) csum2(sa, ca, pk(h[k], h[k]), pk(-h[k], -h[k]), pk(lw[k], lw[k]), pk(c0[li[k]], c1[li[k]]));
                if (store) {
                    float ra, rb;
                    upk(add2(sa, ca), ra, rb);
                    y[(f0 + f) * ldy + row] = ra;
                    y[(f0 + f + 1) * ldy + row] = rb;
                }
            } else if (f0 + f < nrhs) {
                float s1 = 0.f, c1 = 0.f;
                const float *c0 = cur + f * US;
#pragma unroll
                for (int k = 0; k < L; ++k)
                    if (k < rl) csum1(s1, c1, h[k], lw[k], c0[li[k]]);
                if (store) y[(f0 + f) * ldy + row] = __fadd_rn(s1, c1);
            }
        }
        __syncthreads();
    }
}

__global__ void k_entry_rows(const int *rp, i64 n_rows, int *erow) {
    i64 r = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n_rows) return;
    for (int k = rp[r]; k < rp[r + 1]; ++k) erow[k] = static_cast<int>(r);
}

__global__ void k_block_keys(const int *erow, const int *col, const int *blk_of_slice, i64 nnz, std::uint64_t *key,
                             int *val) {
    i64 e = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (e >= nnz) return;
    key[e] = (static_cast<std::uint64_t>(blk_of_slice[erow[e] >> 5]) << 32) | static_cast<unsigned>(col[e]);
    val[e] = static_cast<int>(e);
}

__global__ void k_unique_flags(const std::uint64_t *key, i64 n, int *flag) {
    i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    flag[i] = (i == 0 || key[i] != key[i - 1]) ? 1 : 0;
}

__global__ void k_unique_emit(const std::uint64_t *key, const int *flag, const i64 *pos, i64 n, int *ucol, int *ucount) {
    i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n || !flag[i]) return;
    ucol[pos[i]] = static_cast<int>(key[i] & 0xffffffffu);
    atomicAdd(&ucount[key[i] >> 32], 1);
}

__global__ void k_entry_lidx(const std::uint64_t *key, const int *val, const int *flag, const i64 *pos,
                             const int *ustart, i64 n, unsigned short *lidx_csr) {
    i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n) return;
    i64 uid = pos[i] + flag[i] - 1;
    lidx_csr[val[i]] = static_cast<unsigned short>(uid - ustart[key[i] >> 32]);
}

__global__ void k_sell_lidx(const int *rp, i64 n_rows, i64 n_slices, const int *base, const int *rlen,
                            const unsigned short *lidx_csr, unsigned short *slidx) {
    i64 r = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n_slices * 32) return;
    i64 s = r >> 5;
    int lane = static_cast<int>(r & 31);
    int L = (base[s + 1] - base[s]) / 32;
    int n = rlen[r];
    int r0 = r < n_rows ? rp[r] : 0;
    for (int k = 0; k < L; ++k) slidx[base[s] + k * 32 + lane] = k < n ? lidx_csr[r0 + k] : 0;
}

void build_staged(Matrix &m, cudaStream_t s) {
    Staged &G = m.staged;
    if (G.built) return;
    build_sell(m, 1, s);
    const Sell &S = m.sell32;
    const i64 n_rows = m.n_dst, nnz = m.nnz;
    // Blocks of 4 slices grouped by source locality: slices sorted by the
    // median source column of their entries, then taken 4 at a time, so a
    // block's rows share source cells and consecutive blocks are neighbours.
    const i64 nsl = S.n_slices;
    std::vector<int> hrp(n_rows + 1), hcol(std::max<i64>(1, nnz));
    AXGB_CUDA(cudaMemcpy(hrp.data(), m.row_ptr.p, sizeof(int) * (n_rows + 1), cudaMemcpyDeviceToHost));
    if (nnz) AXGB_CUDA(cudaMemcpy(hcol.data(), m.col.p, sizeof(int) * nnz, cudaMemcpyDeviceToHost));
    std::vector<long long> skey(nsl);
    for (i64 q = 0; q < nsl; ++q) {
        int a0 = hrp[q * 32], a1 = hrp[std::min<i64>((q + 1) * 32, n_rows)];
        if (a1 == a0) {
            skey[q] = (1ll << 40) + q;  // empty slices last
            continue;
        }
        std::vector<int> c(hcol.begin() + a0, hcol.begin() + a1);
        std::nth_element(c.begin(), c.begin() + c.size() / 2, c.end());
        skey[q] = (static_cast<long long>(c[c.size() / 2]) << 20) + (q & 0xfffff);
    }
    std::vector<int> order(nsl);
    for (i64 q = 0; q < nsl; ++q) order[q] = static_cast<int>(q);
    std::stable_sort(order.begin(), order.end(), [&](int x1, int x2) { return skey[x1] < skey[x2]; });
    const i64 nb = (nsl + 3) / 4;
    G.n_blocks = nb;
    G.h_bslices.assign(nb, make_int4(-1, -1, -1, -1));
    std::vector<int> blk_of_slice(std::max<i64>(1, nsl));
    for (i64 q = 0; q < nsl; ++q) {
        i64 b = q / 4;
        int *slot = &G.h_bslices[b].x;
        slot[q % 4] = order[q];
        blk_of_slice[order[q]] = static_cast<int>(b);
    }
    G.bslices.upload(G.h_bslices.data(), std::max<size_t>(1, G.h_bslices.size()), s);
    G.blk_of_slice.upload(blk_of_slice.data(), blk_of_slice.size(), s);
    const int *d_blk_p = G.blk_of_slice.p;
    G.ucount.alloc(nb);
    G.ucount.zero(s);
    G.ustart.alloc(nb + 1);
    G.lidx.alloc(S.n_entries);
    DBuf<unsigned short> lidx_csr(nnz);
    i64 n_unique = 0;
    if (nnz > 0) {
        DBuf<int> erow(nnz), val(nnz), flag(nnz);
        DBuf<std::uint64_t> key(nnz);
        DBuf<i64> pos(nnz + 1);
        k_entry_rows<<<nblk(n_rows, 256), 256, 0, s>>>(m.row_ptr.p, n_rows, erow.p);
        k_block_keys<<<nblk(nnz, 256), 256, 0, s>>>(erow.p, m.col.p, d_blk_p, nnz, key.p, val.p);
        AXGB_CUDA(cudaGetLastError());
        int bits = 32;
        while (bits < 64 && (static_cast<unsigned long long>(nb) >> (bits - 32)) > 0) ++bits;
        radix_sort_pairs_u64(key.p, val.p, nnz, bits, s);
        k_unique_flags<<<nblk(nnz, 256), 256, 0, s>>>(key.p, nnz, flag.p);
        scan_exclusive_i32_to_i64(flag.p, pos.p, nnz, s);
        AXGB_CUDA(cudaMemcpy(&n_unique, pos.p + nnz, sizeof(i64), cudaMemcpyDeviceToHost));
        G.ucol.alloc(n_unique);
        k_unique_emit<<<nblk(nnz, 256), 256, 0, s>>>(key.p, flag.p, pos.p, nnz, G.ucol.p, G.ucount.p);
        scan_exclusive_i32(G.ucount.p, G.ustart.p, nb, s);
        k_entry_lidx<<<nblk(nnz, 256), 256, 0, s>>>(key.p, val.p, flag.p, pos.p, G.ustart.p, nnz, lidx_csr.p);
        AXGB_CUDA(cudaGetLastError());
    } else {
        G.ucol.alloc(1);
        scan_exclusive_i32(G.ucount.p, G.ustart.p, nb, s);
    }
    if (S.n_slices > 0) {
        k_sell_lidx<<<nblk(S.n_slices * 32, 256), 256, 0, s>>>(m.row_ptr.p, n_rows, S.n_slices, S.base.p, S.len.p,
                                                              lidx_csr.p, G.lidx.p);
        AXGB_CUDA(cudaGetLastError());
    }
    // classes on the host
    std::vector<int> hc(nb);
    if (nb) AXGB_CUDA(cudaMemcpy(hc.data(), G.ucount.p, sizeof(int) * nb, cudaMemcpyDeviceToHost));
    std::vector<std::vector<int>> cls(3);
    std::vector<int> fb;
    G.class_umax.assign(3, 0);
    for (i64 b = 0; b < nb; ++b) {
        int L = 0;
        const int *bsl = &G.h_bslices[b].x;
        for (int w = 0; w < 4; ++w)
            if (bsl[w] >= 0) L = std::max(L, S.h_slice_len[bsl[w]]);
        int c = L <= 8 ? 0 : (L <= 16 ? 1 : (L <= 32 ? 2 : 3));
        if (c < 3 && hc[b] <= kStagedMaxU) {
            cls[c].push_back(static_cast<int>(b));
            G.class_umax[c] = std::max(G.class_umax[c], hc[b]);
        } else {
            for (int w = 0; w < 4; ++w)
                if (bsl[w] >= 0) fb.push_back(bsl[w]);
        }
    }
    std::vector<int> ids;
    G.class_begin.assign(4, 0);
    for (int c = 0; c < 3; ++c) {
        G.class_begin[c] = static_cast<i64>(ids.size());
        ids.insert(ids.end(), cls[c].begin(), cls[c].end());
    }
    G.class_begin[3] = static_cast<i64>(ids.size());
    G.block_ids.upload(ids.data(), ids.size(), s);
    G.fallback_slices.upload(fb.data(), fb.size(), s);
    G.n_fallback = static_cast<i64>(fb.size());
    AXGB_CUDA(cudaStreamSynchronize(s));
    G.built = true;
}

template <int L, int T>
void launch_staged(const Matrix &m, int cls, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    const Staged &G = m.staged;
    const Sell &S = m.sell32;
    i64 nb = G.class_begin[cls + 1] - G.class_begin[cls];
    if (nb == 0) return;
    StagedArgs a;
    a.bslices = G.bslices.p;
    a.blocks = G.block_ids.p + G.class_begin[cls];
    a.n_blocks = nb;
    a.base = S.base.p;
    a.rlen = S.len.p;
    a.lidx = G.lidx.p;
    a.hi = S.hi.p;
    a.lo = S.lo.p;
    a.ucol = G.ucol.p;
    a.ustart = G.ustart.p;
    a.ucount = G.ucount.p;
    a.n_rows = m.n_dst;
    a.n_slices = S.n_slices;
    a.ustride = (std::max(G.class_umax[cls], 1) + 31) / 32 * 32;
    size_t bytes = sizeof(float) * static_cast<size_t>(a.ustride) * (1 + 2 * T);
    AXGB_CUDA(cudaFuncSetAttribute(k_staged<L, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    k_staged<L, T><<<static_cast<unsigned>(nb), kSR, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

template <int T>
void apply_staged_T(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    launch_staged<8, T>(m, 0, x, ldx, y, ldy, nrhs, s);
    launch_staged<16, T>(m, 1, x, ldx, y, ldy, nrhs, s);
    launch_staged<32, T>(m, 2, x, ldx, y, ldy, nrhs, s);
}

// ─── bulk-staged split-FP32 kernel ─────────────────────────────────────────
// Same blocking as k_staged, but the block's source values are fetched as
// contiguous runs (rounded out to 16-byte chunks) with cp.async.bulk on the
// TMA engine, one copy per (run, field), completion counted on an mbarrier
// per buffer. Padding entries of a row point at a zero slot at the end of
// each field's staging area, so the row loop is branch-free; rows are
// grouped in length classes of 4. Requires x 16-byte aligned, ld_x and
// n_src multiples of 4 (so no rounded copy leaves a field's row).

constexpr int kBulkMaxUS = 3072;  // staged floats per field per block (196 KB of smem at T = 8)

__device__ __forceinline__ unsigned smem_u32(const void *p) {
    return static_cast<unsigned>(__cvta_generic_to_shared(p));
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

struct BulkArgs {
    const int4 *bslices;
    const int *blocks;
    i64 n_blocks;
    const int *base, *rlen;
    const unsigned short *lidx;  // staging-area index per sliced-ELL entry (zero slot for padding)
    const float *hi, *lo;
    const int *rstart;  // runs of block b: [rstart[b], rstart[b+1])
    const int4 *runs;   // (global col of the first chunk, chunks, staging offset, 0)
    const int *bus;     // staging floats per field of block b (incl. the 4-float zero slot)
    i64 n_rows, n_slices;
    int us_max;          // stride of a field's staging area in this launch
    int *status;         // device status word (1 = a bounded wait timed out)
};

template <int L, int T>
__global__ void __launch_bounds__(kSR) k_bulk(BulkArgs a, const float *__restrict__ x, i64 ldx,
                                             float *__restrict__ y, i64 ldy, i64 nrhs) {
    extern __shared__ __align__(128) float smem[];
    __shared__ __align__(8) std::uint64_t bar[2];
    __shared__ int abort_flag;
    const int US = a.us_max;
    float *xs = smem;  // [2][T][US]
    const int b = a.blocks[blockIdx.x];
    const int r0 = a.rstart[b], nr = a.rstart[b + 1] - r0;
    const int zero = a.bus[b] - 4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const i64 sid = block_slice(a.bslices, b, warp);
    const i64 row = sid * 32 + lane;
    int rl = 0, base = 0;
    if (sid >= 0) {
        base = a.base[sid];
        rl = a.rlen[row];
    }
    int li[L];
    F2 hp[L], hn[L], lp[L];
#pragma unroll
    for (int k = 0; k < L; ++k) {
        float h = 0.f, l = 0.f;
        int q = zero;
        if (k < rl) {
            int e = base + k * 32 + lane;
            q = a.lidx[e];
            h = a.hi[e];
            l = a.lo[e];
        }
        li[k] = q;
        hp[k] = pk(h, h);
        hn[k] = pk(-h, -h);
        lp[k] = pk(l, l);
    }
    const bool store = sid >= 0 && row < a.n_rows;
    if (threadIdx.x == 0) {
        mbar_init(&bar[0], 1);
        mbar_init(&bar[1], 1);
        abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    // zero slots of both buffers (never written by the bulk copies)
    for (int q = threadIdx.x; q < 2 * T; q += kSR) {
        float4 *zp = reinterpret_cast<float4 *>(xs + q * US + zero);
        *zp = make_float4(0.f, 0.f, 0.f, 0.f);
    }
    __syncthreads();
    const i64 ntile = (nrhs + T - 1) / T;
    auto issue = [&](i64 t, int buf) {
        if (warp != 0) return;
        const i64 fa = t * T;
        const int nf = static_cast<int>((nrhs - fa < static_cast<i64>(T) ? nrhs - fa : static_cast<i64>(T)));
        if (lane == 0) {
            unsigned bytes = nr > 0 ? 16u * static_cast<unsigned>(a.runs[r0].w) : 0u;
            mbar_expect_tx(&bar[buf], bytes * static_cast<unsigned>(nf));
        }
        __syncwarp();
        float *dst0 = xs + buf * T * US;
        for (int q = lane; q < nr; q += 32) {
            int4 r = a.runs[r0 + q];
            for (int f = 0; f < nf; ++f)
                bulk_g2s(dst0 + f * US + r.z, x + (fa + f) * ldx + r.x, 16u * static_cast<unsigned>(r.y), &bar[buf]);
        }
    };
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    issue(0, 0);
    for (i64 t = 0; t < ntile; ++t) {
        const int buf = static_cast<int>(t & 1);
        if (t + 1 < ntile) issue(t + 1, buf ^ 1);
        // bounded wait for this tile's copies
        const unsigned parity = static_cast<unsigned>((t >> 1) & 1);
        const unsigned long long t0 = globaltimer_ns();
        while (!mbar_try_wait(&bar[buf], parity)) {
            if (globaltimer_ns() - t0 > 1000000000ull) {
                abort_flag = 1;
                atomicExch(a.status, 1);
                break;
            }
        }
        __syncthreads();
        if (abort_flag) break;
        const float *cur = xs + buf * T * US;
        const i64 f0 = t * T;
#pragma unroll
        for (int f = 0; f < T; f += 2) {
            if (f0 + f + 1 < nrhs) {
                F2 sa = pk(0.f, 0.f), ca = pk(0.f, 0.f);
                const float *c0 = cur + f * US, *c1 = cur + (f + 1) * US;
#pragma unroll
                for (int k = 0; k < L; ++k) csum2(sa, ca, hp[k], hn[k], lp[k], pk(c0[li[k]], c1[li[k]]));
                if (store) {
                    float ra, rb;
                    upk(add2(sa, ca), ra, rb);
                    y[(f0 + f) * ldy + row] = ra;
                    y[(f0 + f + 1) * ldy + row] = rb;
                }
            } else if (f0 + f < nrhs) {
                float s1 = 0.f, c1 = 0.f;
                const float *c0 = cur + f * US;
#pragma unroll
                for (int k = 0; k < L; ++k) {
                    float hh, dummy, ll;
                    upk(hp[k], hh, dummy);
                    upk(lp[k], ll, dummy);
                    csum1(s1, c1, hh, ll, c0[li[k]]);
                }
                if (store) y[(f0 + f) * ldy + row] = __fadd_rn(s1, c1);
            }
        }
        __syncthreads();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
}

// Chunked variant: the same staging layout and branch-free row loop as
// k_bulk, but the 16-byte chunks are copied by all threads with
// cp.async.cg (one instruction per chunk and field), double-buffered with
// cp.async groups.
struct ChunkArgs {
    const int4 *bslices;
    const int *blocks;
    i64 n_blocks;
    const int *base, *rlen;
    const unsigned short *lidx;
    const float *hi, *lo;
    const int *cstart;  // chunks of block b: [cstart[b], cstart[b+1])
    const int *ccol;    // global column of each chunk (multiple of 4)
    i64 n_rows, n_slices;
    int us_max;
};

__device__ __forceinline__ void cp_async16(void *smem, const void *gmem) {
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(smem)), "l"(gmem) : "memory");
}

template <int L, int T>
__global__ void __launch_bounds__(kSR) k_chunk(ChunkArgs a, const float *__restrict__ x, i64 ldx,
                                              float *__restrict__ y, i64 ldy, i64 nrhs) {
    static_assert(T % 2 == 0, "fields per stage must be even");
    extern __shared__ __align__(128) float smem[];
    const int US = a.us_max;
    float *xs = smem;  // [2][T][US]
    const int b = a.blocks[blockIdx.x];
    const int c0 = a.cstart[b], nch = a.cstart[b + 1] - c0;
    const int zero = 4 * nch;
    const int lane = threadIdx.x & 31;
    const i64 sid = block_slice(a.bslices, b, threadIdx.x >> 5);
    const i64 row = sid * 32 + lane;
    int rl = 0, base = 0;
    if (sid >= 0) {
        base = a.base[sid];
        rl = a.rlen[row];
    }
    int li[L];
    float h[L], lw[L];
#pragma unroll
    for (int k = 0; k < L; ++k) {
        float hv = 0.f, lv = 0.f;
        int q = zero;
        if (k < rl) {
            int e = base + k * 32 + lane;
            q = a.lidx[e];
            hv = a.hi[e];
            lv = a.lo[e];
        }
        li[k] = q;
        h[k] = hv;
        lw[k] = lv;
    }
    const bool store = sid >= 0 && row < a.n_rows;
    for (int q = threadIdx.x; q < 2 * T; q += kSR)
        *reinterpret_cast<float4 *>(xs + q * US + zero) = make_float4(0.f, 0.f, 0.f, 0.f);
    const i64 ntile = (nrhs + T - 1) / T;
    auto stage = [&](i64 t, float *dst) {
        const i64 fa = t * T;
        const int nf = static_cast<int>((nrhs - fa < static_cast<i64>(T)) ? nrhs - fa : static_cast<i64>(T));
        for (int j = threadIdx.x; j < nch; j += kSR) {
            const int g = a.ccol[c0 + j];
            const float *src = x + fa * ldx + g;
#pragma unroll
            for (int f = 0; f < T; ++f)
                if (f < nf) cp_async16(dst + f * US + 4 * j, src + f * ldx);
        }
        cp_async_commit();
    };
    const F2 mone = pk(-1.f, -1.f);
    stage(0, xs);
    for (i64 t = 0; t < ntile; ++t) {
        const float *cur = xs + (t & 1) * T * US;
        if (t + 1 < ntile) {
            stage(t + 1, xs + ((t + 1) & 1) * T * US);
            cp_async_wait<1>();
        } else {
            cp_async_wait<0>();
        }
        __syncthreads();
        const i64 f0 = t * T;
        if (f0 + T <= nrhs) {
            F2 sa[T / 2], cn[T / 2];
#pragma unroll
            for (int q = 0; q < T / 2; ++q) {
                sa[q] = pk(0.f, 0.f);
                cn[q] = pk(0.f, 0.f);
            }
#pragma unroll
            for (int k = 0; k < L; ++k) {
                const F2 h2 = pk(h[k], h[k]), l2 = pk(lw[k], lw[k]);
                const float *pk0 = cur + li[k];
#pragma unroll
                for (int q = 0; q < T / 2; ++q)
                    cstep2(sa[q], cn[q], h2, l2, pk(pk0[(2 * q) * US], pk0[(2 * q + 1) * US]), mone);
            }
            if (store) {
#pragma unroll
                for (int q = 0; q < T / 2; ++q) {
                    float ra, rb;
                    upk(sub2(sa[q], cn[q]), ra, rb);
                    y[(f0 + 2 * q) * ldy + row] = ra;
                    y[(f0 + 2 * q + 1) * ldy + row] = rb;
                }
            }
        } else {
            for (int f = 0; f < T; ++f) {
                if (f0 + f >= nrhs) break;
                float s1 = 0.f, c1 = 0.f;
                const float *p0 = cur + f * US;
#pragma unroll
                for (int k = 0; k < L; ++k) csum1(s1, c1, h[k], lw[k], p0[li[k]]);
                if (store) y[(f0 + f) * ldy + row] = __fadd_rn(s1, c1);
            }
        }
        __syncthreads();
    }
}

template <int L, int T>
void launch_chunk(Matrix &m, int cls, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    const Bulk &B = m.bulk;
    const Sell &S = m.sell32;
    i64 nb = B.class_begin[cls + 1] - B.class_begin[cls];
    if (nb == 0) return;
    ChunkArgs a;
    a.bslices = m.staged.bslices.p;
    a.blocks = B.block_ids.p + B.class_begin[cls];
    a.n_blocks = nb;
    a.base = S.base.p;
    a.rlen = S.len.p;
    a.lidx = B.lidx.p;
    a.hi = S.hi.p;
    a.lo = S.lo.p;
    a.cstart = B.cstart.p;
    a.ccol = B.ccol.p;
    a.n_rows = m.n_dst;
    a.n_slices = S.n_slices;
    a.us_max = (B.class_usmax[cls] + 31) / 32 * 32;
    size_t bytes = sizeof(float) * static_cast<size_t>(a.us_max) * 2 * T;
    AXGB_CUDA(cudaFuncSetAttribute(k_chunk<L, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    k_chunk<L, T><<<static_cast<unsigned>(nb), kSR, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

template <int T>
void apply_chunk_T(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    launch_chunk<4, T>(m, 0, x, ldx, y, ldy, nrhs, s);
    launch_chunk<8, T>(m, 1, x, ldx, y, ldy, nrhs, s);
    launch_chunk<12, T>(m, 2, x, ldx, y, ldy, nrhs, s);
    launch_chunk<16, T>(m, 3, x, ldx, y, ldy, nrhs, s);
    launch_chunk<20, T>(m, 4, x, ldx, y, ldy, nrhs, s);
    launch_chunk<24, T>(m, 5, x, ldx, y, ldy, nrhs, s);
    launch_chunk<28, T>(m, 6, x, ldx, y, ldy, nrhs, s);
    launch_chunk<32, T>(m, 7, x, ldx, y, ldy, nrhs, s);
}

__global__ void k_bulk_lidx(const int *rp, i64 n_rows, i64 n_slices, const int *base, const int *rlen,
                            const unsigned short *lidx_sell, const int *ustart, const int *remap, const int *bus,
                            const unsigned char *staged_ok, const int *blk_of_slice, unsigned short *out) {
    i64 r = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (r >= n_slices * 32) return;
    i64 s = r >> 5;
    int lane = static_cast<int>(r & 31);
    i64 b = blk_of_slice[s];
    int L = (base[s + 1] - base[s]) / 32;
    int n = rlen[r];
    bool ok = staged_ok[b] != 0;
    for (int k = 0; k < L; ++k) {
        int e = base[s] + k * 32 + lane;
        int v = 0;
        if (ok) v = k < n ? remap[ustart[b] + lidx_sell[e]] : bus[b] - 4;
        out[e] = static_cast<unsigned short>(v);
    }
}

void build_bulk(Matrix &m, cudaStream_t s) {
    Bulk &B = m.bulk;
    if (B.built) return;
    build_staged(m, s);
    const Staged &G = m.staged;
    const Sell &S = m.sell32;
    const i64 nb = G.n_blocks;
    std::vector<int> ustart(nb + 1), ucount(nb);
    std::vector<int> ucol(std::max<size_t>(1, G.ucol.n));
    if (nb) {
        AXGB_CUDA(cudaMemcpy(ustart.data(), G.ustart.p, sizeof(int) * (nb + 1), cudaMemcpyDeviceToHost));
        AXGB_CUDA(cudaMemcpy(ucount.data(), G.ucount.p, sizeof(int) * nb, cudaMemcpyDeviceToHost));
        AXGB_CUDA(cudaMemcpy(ucol.data(), G.ucol.p, sizeof(int) * G.ucol.n, cudaMemcpyDeviceToHost));
    }
    const i64 n_unique = nb ? ustart[nb] : 0;
    std::vector<int> remap(std::max<i64>(1, n_unique));
    std::vector<std::vector<int4>> runs(nb);
    std::vector<int> bus(nb, 4);
    // runs of consecutive columns, rounded out to 16-byte chunks; runs whose
    // chunks touch or are one chunk apart are merged
    for (i64 b = 0; b < nb; ++b) {
        const int *c = ucol.data() + ustart[b];
        const int n = ucount[b];
        int off = 0;
        int q = 0;
        while (q < n) {
            int g4 = c[q] & ~3;
            int end4 = (c[q] | 3) + 1;
            int q1 = q + 1;
            while (q1 < n && (c[q1] & ~3) <= end4 + 4) {
                end4 = std::max(end4, (c[q1] | 3) + 1);
                ++q1;
            }
            int chunks = (end4 - g4) / 4;
            runs[b].push_back(make_int4(g4, chunks, off, 0));
            for (int t = q; t < q1; ++t) remap[ustart[b] + t] = off + (c[t] - g4);
            off += 4 * chunks;
            q = q1;
        }
        bus[b] = off + 4;  // + zero slot
        if (!runs[b].empty()) runs[b][0].w = off / 4;  // total chunks of the block
    }
    // classes: (row length class in steps of 4) x fits-in-smem
    std::vector<unsigned char> ok(nb, 0);
    const int nclass = 8;
    std::vector<std::vector<int>> cls(nclass);
    B.class_usmax.assign(nclass, 0);
    std::vector<int> rstart(nb + 1, 0);
    std::vector<int4> allruns;
    for (i64 b = 0; b < nb; ++b) {
        int L = 0;
        const int *bsl = &G.h_bslices[b].x;
        for (int w = 0; w < 4; ++w)
            if (bsl[w] >= 0) L = std::max(L, S.h_slice_len[bsl[w]]);
        int c = L <= 4 ? 0 : (L + 3) / 4 - 1;
        rstart[b] = static_cast<int>(allruns.size());
        allruns.insert(allruns.end(), runs[b].begin(), runs[b].end());
        if (c < nclass && bus[b] <= kBulkMaxUS) {
            ok[b] = 1;
            cls[c].push_back(static_cast<int>(b));
            B.class_usmax[c] = std::max(B.class_usmax[c], bus[b]);
        }
    }
    rstart[nb] = static_cast<int>(allruns.size());
    std::vector<int> ids, fb;
    B.class_begin.assign(nclass + 1, 0);
    for (int c = 0; c < nclass; ++c) {
        B.class_begin[c] = static_cast<i64>(ids.size());
        ids.insert(ids.end(), cls[c].begin(), cls[c].end());
    }
    B.class_begin[nclass] = static_cast<i64>(ids.size());
    for (i64 b = 0; b < nb; ++b)
        if (!ok[b]) {
            const int *bsl = &G.h_bslices[b].x;
            for (int w = 0; w < 4; ++w)
                if (bsl[w] >= 0) fb.push_back(bsl[w]);
        }
    B.block_ids.upload(ids.data(), ids.size(), s);
    B.fallback_slices.upload(fb.data(), fb.size(), s);
    B.n_fallback = static_cast<i64>(fb.size());
    B.rstart.upload(rstart.data(), rstart.size(), s);
    // flattened 16-byte chunk list (chunk j of a block stages at offset 4*j)
    std::vector<int> cstart(nb + 1, 0), ccol;
    for (i64 b = 0; b < nb; ++b) {
        cstart[b] = static_cast<int>(ccol.size());
        for (const int4 &r : runs[b])
            for (int j = 0; j < r.y; ++j) ccol.push_back(r.x + 4 * j);
    }
    cstart[nb] = static_cast<int>(ccol.size());
    B.cstart.upload(cstart.data(), cstart.size(), s);
    B.ccol.upload(ccol.data(), std::max<size_t>(1, ccol.size()), s);
    B.runs.upload(allruns.data(), std::max<size_t>(1, allruns.size()), s);
    B.bus.upload(bus.data(), std::max<size_t>(1, bus.size()), s);
    DBuf<int> d_remap;
    d_remap.upload(remap.data(), remap.size(), s);
    DBuf<unsigned char> d_ok;
    d_ok.upload(ok.data(), std::max<size_t>(1, ok.size()), s);
    B.lidx.alloc(S.n_entries);
    if (S.n_slices > 0) {
        k_bulk_lidx<<<nblk(S.n_slices * 32, 256), 256, 0, s>>>(m.row_ptr.p, m.n_dst, S.n_slices, S.base.p, S.len.p,
                                                              G.lidx.p, G.ustart.p, d_remap.p, B.bus.p, d_ok.p,
                                                              G.blk_of_slice.p, B.lidx.p);
        AXGB_CUDA(cudaGetLastError());
    }
    if (!B.status.p) {
        B.status.alloc(1);
        B.status.zero(s);
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
    B.built = true;
}

template <int L, int T>
void launch_bulk(Matrix &m, int cls, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    const Bulk &B = m.bulk;
    const Sell &S = m.sell32;
    i64 nb = B.class_begin[cls + 1] - B.class_begin[cls];
    if (nb == 0) return;
    BulkArgs a;
    a.bslices = m.staged.bslices.p;
    a.blocks = B.block_ids.p + B.class_begin[cls];
    a.n_blocks = nb;
    a.base = S.base.p;
    a.rlen = S.len.p;
    a.lidx = B.lidx.p;
    a.hi = S.hi.p;
    a.lo = S.lo.p;
    a.rstart = B.rstart.p;
    a.runs = B.runs.p;
    a.bus = B.bus.p;
    a.n_rows = m.n_dst;
    a.n_slices = S.n_slices;
    a.us_max = (B.class_usmax[cls] + 31) / 32 * 32;
    a.status = B.status.p;
    size_t bytes = sizeof(float) * static_cast<size_t>(a.us_max) * 2 * T;
    AXGB_CUDA(cudaFuncSetAttribute(k_bulk<L, T>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(bytes)));
    k_bulk<L, T><<<static_cast<unsigned>(nb), kSR, bytes, s>>>(a, x, ldx, y, ldy, nrhs);
}

template <int T>
void apply_bulk_T(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    launch_bulk<4, T>(m, 0, x, ldx, y, ldy, nrhs, s);
    launch_bulk<8, T>(m, 1, x, ldx, y, ldy, nrhs, s);
    launch_bulk<12, T>(m, 2, x, ldx, y, ldy, nrhs, s);
    launch_bulk<16, T>(m, 3, x, ldx, y, ldy, nrhs, s);
    launch_bulk<20, T>(m, 4, x, ldx, y, ldy, nrhs, s);
    launch_bulk<24, T>(m, 5, x, ldx, y, ldy, nrhs, s);
    launch_bulk<28, T>(m, 6, x, ldx, y, ldy, nrhs, s);
    launch_bulk<32, T>(m, 7, x, ldx, y, ldy, nrhs, s);
}

bool bulk_eligible(const Matrix &m, const float *x, i64 ldx) {
    return (reinterpret_cast<std::uintptr_t>(x) % 16 == 0) && (ldx % 4 == 0) && (m.n_src % 4 == 0);
}

// ─── persistent batch kernel ───────────────────────────────────────────────
// Items of all matrices are handed out by one atomic counter (no waiting):
// item -> (matrix, tile, slice). Entries of up to 32 per row are cached in
// registers; longer rows are read from global memory.
__global__ void __launch_bounds__(256) k_batch(const Batch::Desc *__restrict__ desc, int n_desc, i64 total,
                                               unsigned long long *counter) {
    const int lane = threadIdx.x & 31;
    while (true) {
        unsigned long long it = 0;
        if (lane == 0) it = atomicAdd(counter, 1ull);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (static_cast<i64>(it) >= total) return;
        int m = 0;
        while (m + 1 < n_desc && desc[m + 1].item_begin <= static_cast<i64>(it)) ++m;
        const Batch::Desc &d = desc[m];
        i64 local = static_cast<i64>(it) - d.item_begin;
        i64 t = local / d.n_slices;
        i64 sid = local - t * d.n_slices;
        i64 row = sid * 32 + lane;
        int base = d.base[sid];
        int rl = d.rlen[sid * 32 + lane];
        i64 f0 = t * d.tile, f1 = min(f0 + d.tile, d.nrhs);
        bool store = row < d.n_rows;
        constexpr int L = 32;
        int c[L];
        float h[L], lw[L];
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (k < rl) {
                int e = base + k * 32 + lane;
                c[k] = d.col[e];
                h[k] = d.hi[e];
                lw[k] = d.lo[e];
            } else {
                c[k] = 0;
                h[k] = 0.f;
                lw[k] = 0.f;
            }
        }
        for (i64 f = f0; f < f1; ++f) {
            float s = 0.f, cc = 0.f;
            const float *xf = d.x + f * d.ldx;
#pragma unroll
            for (int k = 0; k < L; ++k)
                if (k < rl) csum1(s, cc, h[k], lw[k], __ldg(xf + c[k]));
            for (int k = L; k < rl; ++k) {
                int e = base + k * 32 + lane;
                csum1(s, cc, d.hi[e], d.lo[e], __ldg(xf + d.col[e]));
            }
            if (store) d.y[f * d.ldy + row] = __fadd_rn(s, cc);
        }
    }
}

}  // namespace

void matrix_prepare(Matrix &m, int format, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(m.mu);
    if (format == 3) {
        build_bulk(m, s);
        const Bulk &B = m.bulk;
        int launches = B.n_fallback > 0 ? 1 : 0;
        for (size_t c = 0; c + 1 < B.class_begin.size(); ++c)
            if (B.class_begin[c + 1] > B.class_begin[c]) ++launches;
        m.stats[6] = launches;
        return;
    }
    if (format == 2) {
        build_staged(m, s);
        const Staged &G = m.staged;
        int launches = G.n_fallback > 0 ? 1 : 0;
        for (int c = 0; c < 3; ++c)
            if (G.class_begin[c + 1] > G.class_begin[c]) ++launches;
        m.stats[7] = launches;
        return;
    }
    build_sell(m, format == 0 ? 0 : 1, s);
    if (format == 1) {
        const Sell &S = m.sell32;
        int launches = 0;
        for (int c = 0; c < 5; ++c)
            if (S.class_begin[c + 1] > S.class_begin[c]) ++launches;
        m.stats[5] = launches;
    }
}

void apply_split(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                 cudaStream_t s) {
    if (nrhs <= 0) return;
    if ((p.variant == 2 || p.variant == 3) && bulk_eligible(m, x, ldx)) {
        if (!m.bulk.built) matrix_prepare(m, 3, s);
        if (p.variant == 3) {
            if (p.unroll >= 8)
                apply_bulk_T<8>(m, x, ldx, y, ldy, nrhs, s);
            else if (p.unroll >= 4)
                apply_bulk_T<4>(m, x, ldx, y, ldy, nrhs, s);
            else
                apply_bulk_T<2>(m, x, ldx, y, ldy, nrhs, s);
        } else {
            if (p.unroll >= 8)
                apply_chunk_T<8>(m, x, ldx, y, ldy, nrhs, s);
            else if (p.unroll >= 4)
                apply_chunk_T<4>(m, x, ldx, y, ldy, nrhs, s);
            else
                apply_chunk_T<2>(m, x, ldx, y, ldy, nrhs, s);
        }
        const Bulk &B = m.bulk;
        if (B.n_fallback > 0) {
            SellArgs a = sell_args(m, m.sell32, 4);
            a.ids = B.fallback_slices.p;
            a.n_ids = B.n_fallback;
            launch_split<0>(a, x, ldx, y, ldy, nrhs, nrhs, 1, s);
        }
        AXGB_CUDA(cudaGetLastError());
        return;
    }
    if (p.variant >= 1) {
        if (!m.staged.built) matrix_prepare(m, 2, s);
        if (p.unroll >= 8)
            apply_staged_T<8>(m, x, ldx, y, ldy, nrhs, s);
        else if (p.unroll >= 4)
            apply_staged_T<4>(m, x, ldx, y, ldy, nrhs, s);
        else
            apply_staged_T<2>(m, x, ldx, y, ldy, nrhs, s);
        const Staged &G = m.staged;
        if (G.n_fallback > 0) {
            SellArgs a = sell_args(m, m.sell32, 4);
            a.ids = G.fallback_slices.p;
            a.n_ids = G.n_fallback;
            launch_split<0>(a, x, ldx, y, ldy, nrhs, nrhs, 1, s);
        }
        AXGB_CUDA(cudaGetLastError());
        return;
    }
    if (!m.sell32.built) matrix_prepare(m, 1, s);
    const Sell &S = m.sell32;
    i64 tile = (p.fields_per_pass <= 0 || p.fields_per_pass > nrhs) ? nrhs : p.fields_per_pass;
    const int unroll = p.unroll;
    launch_split<8>(sell_args(m, S, 0), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<16>(sell_args(m, S, 1), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<32>(sell_args(m, S, 2), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<64>(sell_args(m, S, 3), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<0>(sell_args(m, S, 4), x, ldx, y, ldy, nrhs, tile, unroll, s);
    AXGB_CUDA(cudaGetLastError());
}

void apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    if (!m.sell64.built) matrix_prepare(m, 0, s);
    const Sell &S = m.sell64;
    i64 tile = nrhs;
    if (tile <= 0) return;
    launch_f64<8>(sell_args(m, S, 0), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<16>(sell_args(m, S, 1), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<32>(sell_args(m, S, 2), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<64>(sell_args(m, S, 3), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<0>(sell_args(m, S, 4), x, ldx, y, ldy, nrhs, tile, s);
    AXGB_CUDA(cudaGetLastError());
}

void conservation(Matrix &m, const void *src, const void *dst, bool f32, int norm_type, double *out, cudaStream_t s) {
    double si, di;
    if (f32) {
        si = integral(static_cast<const float *>(src), m.area_a.p, m.frac_a.p, m.n_src, 0, s);
        di = integral(static_cast<const float *>(dst), m.area_b.p, m.frac_b.p, m.n_dst, norm_type == 0 ? 1 : 0, s);
    } else {
        si = integral(static_cast<const double *>(src), m.area_a.p, m.frac_a.p, m.n_src, 0, s);
        di = integral(static_cast<const double *>(dst), m.area_b.p, m.frac_b.p, m.n_dst, norm_type == 0 ? 1 : 0, s);
    }
    double ae = std::abs(si - di);
    double den = std::max({std::abs(si), std::abs(di), 2.220446049250313e-16});
    out[0] = si;
    out[1] = di;
    out[2] = ae;
    out[3] = ae / den;
}

std::shared_ptr<Batch> batch_create(const std::vector<std::shared_ptr<Matrix>> &mats, const std::vector<i64> &nrhs) {
    auto b = std::make_shared<Batch>();
    b->mats = mats;
    b->nrhs = nrhs;
    i64 items = 0;
    for (size_t q = 0; q < mats.size(); ++q) {
        Matrix &m = *mats[q];
        matrix_prepare(m, 1, 0);
        Batch::Desc d{};
        d.base = m.sell32.base.p;
        d.len = nullptr;
        d.rlen = m.sell32.len.p;
        d.col = m.sell32.col.p;
        d.hi = m.sell32.hi.p;
        d.lo = m.sell32.lo.p;
        d.n_rows = m.n_dst;
        d.n_slices = m.sell32.n_slices;
        d.nrhs = nrhs[q];
        d.tile = std::max<i64>(1, std::min<i64>(nrhs[q], 8));
        d.n_tiles = (nrhs[q] + d.tile - 1) / d.tile;
        d.item_begin = items;
        items += d.n_tiles * d.n_slices;
        b->desc.push_back(d);
    }
    b->total_items = items;
    b->d_desc.alloc(std::max<size_t>(1, b->desc.size()));
    b->counter.alloc(1);
    int dev = 0, sms = 0;
    AXGB_CUDA(cudaGetDevice(&dev));
    AXGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch, 256, 0));
    b->blocks = std::max(1, sms * std::max(1, per_sm));
    return b;
}

void batch_apply(Batch &b, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(b.mu);
    const size_t k = b.desc.size();
    std::vector<const void *> ptrs;
    for (size_t q = 0; q < k; ++q) {
        AXGB_REQUIRE(ldx[q] >= b.mats[q]->n_src && ldy[q] >= b.mats[q]->n_dst, "batch_apply: leading dimension");
        ptrs.push_back(x[q]);
        ptrs.push_back(y[q]);
        ptrs.push_back(reinterpret_cast<const void *>(ldx[q]));
        ptrs.push_back(reinterpret_cast<const void *>(ldy[q]));
    }
    if (ptrs != b.last_ptrs) {
        for (size_t q = 0; q < k; ++q) {
            b.desc[q].x = x[q];
            b.desc[q].ldx = ldx[q];
            b.desc[q].y = y[q];
            b.desc[q].ldy = ldy[q];
        }
        // stream-ordered update of the descriptors the graph reads
        AXGB_CUDA(cudaMemcpyAsync(b.d_desc.p, b.desc.data(), sizeof(Batch::Desc) * k, cudaMemcpyHostToDevice, s));
        AXGB_CUDA(cudaStreamSynchronize(s));
        b.last_ptrs = ptrs;
    }
    if (b.total_items == 0) return;
    auto it = b.graphs.find(s);
    if (it == b.graphs.end()) {
        cudaStream_t cap = s;
        bool own = false;
        if (cap == 0) {  // legacy stream cannot be captured: capture on a private stream
            AXGB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        cudaGraph_t g;
        cudaGraphExec_t ge;
        AXGB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        cudaMemsetAsync(b.counter.p, 0, sizeof(unsigned long long), cap);
        k_batch<<<b.blocks, 256, 0, cap>>>(b.d_desc.p, static_cast<int>(k), b.total_items, b.counter.p);
        AXGB_CUDA(cudaStreamEndCapture(cap, &g));
        AXGB_CUDA(cudaGraphInstantiate(&ge, g, 0));
        if (own) AXGB_CUDA(cudaStreamDestroy(cap));
        it = b.graphs.emplace(s, std::make_pair(g, ge)).first;
    }
    AXGB_CUDA(cudaGraphLaunch(it->second.second, s));
}

}  // namespace axgb
