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

#include "fp32x2.cuh"
#include "internal.hpp"

namespace axgb {

// Arguments of the source gather of a batch member (renumbered sources).
struct GatherDesc {
    const float *x;
    i64 ldx;
    const int *inv;
    i64 n, nrhs;
    float *xr;
    i64 ldr;
};

struct Batch {
    // One descriptor per (matrix, kind): mode 0 covers the slices whose rows
    // have at most 32 entries (lane per row, items = field tile x slice);
    // mode 1 the rows of at most 32 entries of the other slices (lane per
    // field, items = 32-field chunk x row); mode 2 the rows of more than 32
    // entries (lane per leaf, items = 8-field chunk x row).
    struct Desc {
        const int *base, *len, *rlen, *col;
        const float *hi, *lo;
        const int *lrow, *lptr, *lcol;  // mode 2: row-contiguous long rows
        const float *lhi, *llo;
        const int *ids;  // slice ids (modes 0, 1)
        i64 n_ids;       // slices (modes 0, 1) or long rows (mode 2)
        int mode;
        int mat;  // index of the matrix in the batch
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
    // descriptors: the slice items (mode 0) first, then the row items
    // (modes 1, 2); each group has its own persistent kernel and counter
    std::vector<Desc> desc;
    DBuf<Desc> d_desc;
    DBuf<unsigned long long> counter;  // [0]: slice items, [1]: row items
    i64 total_items = 0;               // both groups
    i64 total_slice_items = 0, total_row_items = 0;
    int n_slice_desc = 0;
    int blocks_slices = 0, blocks_rows = 0;
    // matrices whose fields take the persistent staged kernels (blocked
    // layout) in the current plan, and that plan
    std::vector<char> use;
    bool planned = false;
    std::shared_ptr<BlkBatch> blk;
    // members with renumbered sources: fields gathered into xr first
    std::vector<DBuf<float>> xr;
    std::vector<GatherDesc> gdesc;
    DBuf<GatherDesc> d_gdesc;
    // graph per stream, replayed while descriptors are updated in place
    std::map<cudaStream_t, std::pair<cudaGraph_t, cudaGraphExec_t>> graphs;
    std::vector<const void *> last_ptrs;
    // Every graph shares the work counters, descriptors and gather scratch
    // above, so a call on another stream than the previous call's first waits
    // for the previous call's work (event `done`, recorded after each launch).
    cudaEvent_t done = nullptr;
    cudaStream_t last_stream = nullptr;
    bool launched = false;
    // side streams and events of the captured fork/join (kernels of the graph
    // that may run concurrently)
    static constexpr int kSide = 5;
    cudaStream_t side[kSide] = {};
    cudaEvent_t fork = nullptr, join[kSide] = {};
    std::mutex mu;
    ~Batch() {
        for (auto &g : graphs) {
            cudaGraphExecDestroy(g.second.second);
            cudaGraphDestroy(g.second.first);
        }
        if (done) cudaEventDestroy(done);
        for (int q = 0; q < kSide; ++q) {
            if (side[q]) cudaStreamDestroy(side[q]);
            if (join[q]) cudaEventDestroy(join[q]);
        }
        if (fork) cudaEventDestroy(fork);
    }
};

namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

struct SellArgs {
    const int *ids;
    i64 n_ids;
    const int *base, *len, *rlen, *col;
    const float *hi, *lo;
    const double *w64;
    i64 n_rows;
    float *ylo;  // split kernels: low parts of the outputs (hi+lo form), or null
    i64 ldylo;
};

__device__ __forceinline__ float ldg_f(const float *p) { return __ldg(p); }

// ─── split-FP32 kernel ─────────────────────────────────────────────────────
// Lane per row for slices whose rows have at most L <= 32 entries, entries
// cached in registers (longer rows: k_split_rows).
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
    static_assert(L > 0 && L <= 32, "lane-per-row kernels cache at most 32 entries");
    {
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
            F2 hp[L], lp[L];
#pragma unroll
            for (int k = 0; k < L; ++k) {
                hp[k] = pk(h[k], h[k]);
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
                            csum2(s[u], cc[u], h[k], hp[k], lp[k], xa, xb);
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
                        if (a.ylo) {
                            float sa, sb, ca, cb;
                            upk(s[u], sa, sb);
                            upk(cc[u], ca, cb);
                            a.ylo[(f + 2 * u) * a.ldylo + row] = sum_err(sa, ca, ra);
                            a.ylo[(f + 2 * u + 1) * a.ldylo + row] = sum_err(sb, cb, rb);
                        }
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
            if (store) {
                const float r = __fadd_rn(s, cc);
                y[f * ldy + row] = r;
                if (a.ylo) a.ylo[f * a.ldylo + row] = sum_err(s, cc, r);
            }
        }
    }
}

// ─── FP64 kernel ───────────────────────────────────────────────────────────
// Lane per row, slices of rows with at most L <= 32 entries (longer rows:
// k_f64_rows); s = fma(w, x, s) in entry order.
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
    static_assert(L > 0 && L <= 32, "lane-per-row kernels cache at most 32 entries");
    {
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
    }
}

// ─── long rows ─────────────────────────────────────────────────────────────
// Slices in the long classes (some row has more than 32 entries; coarse
// destination cells over a fine source, e.g. polar cells over a lat-lon
// source) run in two launches:
//   k_split_rows: rows of at most 32 entries of those slices, one warp per
//                 (row, 32 fields), lane = field, entry order;
//   k_split_long: rows of more than 32 entries, one warp per (row, F
//                 fields), lane = leaf of the order in fp32x2.cuh, the F
//                 fields carried side by side, entries read row-contiguous
//                 (Sell::lcol/lhi/llo), shuffle butterfly at the end.
// Entry k of row p of slice sid sits at base[sid] + 32k + p.
__device__ __forceinline__ bool row_item(const SellArgs &a, i64 nrhs, i64 &row, int &sid, int &p, i64 &f) {
    const int lane = threadIdx.x & 31;
    const i64 w = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const i64 per = a.n_ids * 32;
    if (w >= per * ((nrhs + 31) / 32)) return false;
    const i64 fc = w / per;
    const i64 q = w - fc * per;
    sid = a.ids[q >> 5];
    p = static_cast<int>(q & 31);
    row = static_cast<i64>(sid) * 32 + p;
    f = fc * 32 + lane;
    return row < a.n_rows && f < nrhs;
}

__global__ void __launch_bounds__(256) k_split_rows(SellArgs a, const float *__restrict__ x, i64 ldx,
                                                    float *__restrict__ y, i64 ldy, i64 nrhs) {
    i64 row, f;
    int sid, p;
    if (!row_item(a, nrhs, row, sid, p, f)) return;
    const int n = a.rlen[row];
    if (n > 32) return;  // k_split_long
    const int e0 = a.base[sid] + p;
    const float *xf = x + f * ldx;
    float s = 0.f, c = 0.f;
    for (int k = 0; k < n; ++k) {
        const int e = e0 + 32 * k;
        csum1(s, c, a.hi[e], a.lo[e], ldg_f(xf + a.col[e]));
    }
    const float r = __fadd_rn(s, c);
    y[f * ldy + row] = r;
    if (a.ylo) a.ylo[f * a.ldylo + row] = sum_err(s, c, r);
}

__global__ void __launch_bounds__(256) k_f64_rows(SellArgs a, const double *__restrict__ x, i64 ldx,
                                                  double *__restrict__ y, i64 ldy, i64 nrhs) {
    i64 row, f;
    int sid, p;
    if (!row_item(a, nrhs, row, sid, p, f)) return;
    const int n = a.rlen[row];
    if (n > 32) return;  // k_f64_long
    const int e0 = a.base[sid] + p;
    const double *xf = x + f * ldx;
    double s = 0.0;
    for (int k = 0; k < n; ++k) {
        const int e = e0 + 32 * k;
        s = fma(a.w64[e], __ldg(xf + a.col[e]), s);
    }
    y[f * ldy + row] = s;
}

constexpr i64 kFusedMaxF64 = 2;  // FP64 applies of at most this many fields take the fused kernel
constexpr int kFusedK = 4;        // entries a row of the fused kernels loads before gathering

struct LongRows {
    const int *row, *ptr, *col;
    const float *hi, *lo;
    const double *w64;
    i64 n;
    float *ylo;  // split: low parts of the outputs (hi+lo form), or null
    i64 ldylo;
};
constexpr int kLongF = 8;  // fields per warp in the long-row kernels
constexpr int kLongQ1 = 8;  // entries a lane loads ahead in a single-field long row
constexpr int kBatchLongF = 4;  // fields per long-row item of the persistent batch kernel (k_batch<true>)

// Warp w: long row w % n, fields [F*(w / n), ...). Lane j sums entries
// j, j+32, ... of the row for each of the F fields (leaves), then a
// butterfly over lane offsets 1..16 combines the leaves; lane f stores
// field f.
template <int F = kLongF>
__device__ __forceinline__ void split_long_row(const LongRows &L, i64 w, const float *x, i64 ldx, float *y,
                                               i64 ldy, i64 nrhs) {
    const int lane = threadIdx.x & 31;
    const i64 i = w % L.n, fc = w / L.n;
    const i64 row = L.row[i];
    const int b = L.ptr[i], n = L.ptr[i + 1] - b;
    const i64 f0 = fc * F;
    const int nf = static_cast<int>(nrhs - f0 < F ? nrhs - f0 : F);
    float s[F], c[F];
#pragma unroll
    for (int f = 0; f < F; ++f) {
        s[f] = 0.f;
        c[f] = 0.f;
    }
    // four of the leaf's entries per step (kLongQ1 for a single field): their
    // loads are issued together (memory-level parallelism for rows of
    // hundreds of entries), then summed in order, as one entry per step would
    int k = lane;
    if (nf == 1) {  // warp-uniform
        for (; k + 32 * (kLongQ1 - 1) < n; k += 32 * kLongQ1) {
            int cq[kLongQ1];
            float hq[kLongQ1], lq[kLongQ1], xq[kLongQ1];
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) {
                cq[q] = L.col[b + k + 32 * q];
                hq[q] = L.hi[b + k + 32 * q];
                lq[q] = L.lo[b + k + 32 * q];
            }
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) xq[q] = ldg_f(x + f0 * ldx + cq[q]);
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) csum1(s[0], c[0], hq[q], lq[q], xq[q]);
        }
    }
    for (; k + 96 < n; k += 128) {
        int cq[4];
        float hq[4], lq[4], xq[4][F];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cq[q] = L.col[b + k + 32 * q];
            hq[q] = L.hi[b + k + 32 * q];
            lq[q] = L.lo[b + k + 32 * q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int f = 0; f < F; ++f) xq[q][f] = f < nf ? ldg_f(x + (f0 + f) * ldx + cq[q]) : 0.f;
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int f = 0; f < F; ++f)
                if (f < nf) csum1(s[f], c[f], hq[q], lq[q], xq[q][f]);
    }
    for (; k < n; k += 32) {
        const int col = L.col[b + k];
        const float h = L.hi[b + k], l = L.lo[b + k];
#pragma unroll
        for (int f = 0; f < F; ++f)
            if (f < nf) csum1(s[f], c[f], h, l, ldg_f(x + (f0 + f) * ldx + col));
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
        if (f < nf) {  // warp-uniform
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const float s2 = __shfl_xor_sync(0xffffffffu, s[f], off);
                const float c2 = __shfl_xor_sync(0xffffffffu, c[f], off);
                lcombine(s[f], c[f], s2, c2);
            }
            if (lane == f) {
                const float r = __fadd_rn(s[f], c[f]);
                y[(f0 + f) * ldy + row] = r;
                if (L.ylo) L.ylo[(f0 + f) * L.ldylo + row] = sum_err(s[f], c[f], r);
            }
        }
    }
}

__global__ void __launch_bounds__(256) k_split_long(LongRows L, const float *__restrict__ x, i64 ldx,
                                                    float *__restrict__ y, i64 ldy, i64 nrhs) {
    const i64 w = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (w >= L.n * ((nrhs + kLongF - 1) / kLongF)) return;
    split_long_row(L, w, x, ldx, y, ldy, nrhs);
}

// FP64 form of split_long_row: leaves summed with fma in entry order, then
// the butterfly with plain additions.
template <int F = kLongF>
__device__ __forceinline__ void f64_long_row(const LongRows &L, i64 w, const double *x, i64 ldx, double *y,
                                             i64 ldy, i64 nrhs) {
    const int lane = threadIdx.x & 31;
    const i64 i = w % L.n, fc = w / L.n;
    const i64 row = L.row[i];
    const int b = L.ptr[i], n = L.ptr[i + 1] - b;
    const i64 f0 = fc * F;
    const int nf = static_cast<int>(nrhs - f0 < F ? nrhs - f0 : F);
    double s[F];
#pragma unroll
    for (int f = 0; f < F; ++f) s[f] = 0.0;
    int k = lane;
    if (nf == 1) {  // kLongQ1 entries' loads in flight for a single field, as split_long_row
        for (; k + 32 * (kLongQ1 - 1) < n; k += 32 * kLongQ1) {
            int cq[kLongQ1];
            double wq[kLongQ1], xq[kLongQ1];
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) {
                cq[q] = L.col[b + k + 32 * q];
                wq[q] = L.w64[b + k + 32 * q];
            }
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) xq[q] = __ldg(x + f0 * ldx + cq[q]);
#pragma unroll
            for (int q = 0; q < kLongQ1; ++q) s[0] = fma(wq[q], xq[q], s[0]);
        }
    }
    for (; k + 96 < n; k += 128) {  // four entries' loads in flight, summed in order
        int cq[4];
        double wq[4], xq[4][F];
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            cq[q] = L.col[b + k + 32 * q];
            wq[q] = L.w64[b + k + 32 * q];
        }
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int f = 0; f < F; ++f) xq[q][f] = f < nf ? __ldg(x + (f0 + f) * ldx + cq[q]) : 0.0;
#pragma unroll
        for (int q = 0; q < 4; ++q)
#pragma unroll
            for (int f = 0; f < F; ++f)
                if (f < nf) s[f] = fma(wq[q], xq[q][f], s[f]);
    }
    for (; k < n; k += 32) {
        const int col = L.col[b + k];
        const double wv = L.w64[b + k];
#pragma unroll
        for (int f = 0; f < F; ++f)
            if (f < nf) s[f] = fma(wv, __ldg(x + (f0 + f) * ldx + col), s[f]);
    }
#pragma unroll
    for (int f = 0; f < F; ++f) {
        if (f < nf) {
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) s[f] = s[f] + __shfl_xor_sync(0xffffffffu, s[f], off);
            if (lane == f) y[(f0 + f) * ldy + row] = s[f];
        }
    }
}

__global__ void __launch_bounds__(256) k_f64_long(LongRows L, const double *__restrict__ x, i64 ldx,
                                                  double *__restrict__ y, i64 ldy, i64 nrhs) {
    const i64 w = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (w >= L.n * ((nrhs + kLongF - 1) / kLongF)) return;
    f64_long_row(L, w, x, ldx, y, ldy, nrhs);
}

// ─── few fields: one launch over the whole matrix ────────────────────────
// Warps [0, n_slices): lane per row of one slice, rows of at most 32 entries,
// each entry read from the sliced layout per field (nothing cached: with
// one or two fields there is nothing to reuse); warps [n_slices, n_slices +
// n_lrows): one row of more than 32 entries each, for all fields, 8 at a time
// (split_long_row / f64_long_row). Same summation order as the class
// kernels, so the same bits, in one launch instead of one per class.
// F: fields a long-row warp carries (the call's field count, at most
// kLongF); few fields need few registers, so more warps fit.
template <int F>
__global__ void __launch_bounds__(256, F <= 2 ? 4 : 2) k_split_fused(SellArgs a, LongRows L, i64 n_slices,
                                                                   const float *__restrict__ x, i64 ldx,
                                                                   float *__restrict__ y, i64 ldy, i64 nrhs) {
    const int lane = threadIdx.x & 31;
    const i64 wg = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    // the long rows' warps come first in the grid: each is a long chain of
    // dependent loads, and starting them with the first wave overlaps them
    // with the short rows instead of leaving them as the tail
    if (wg < L.n) {
        for (i64 fc = 0; fc * F < nrhs; ++fc) split_long_row<F>(L, fc * L.n + wg, x, ldx, y, ldy, nrhs);
        return;
    }
    const i64 w = wg - L.n;
    if (w < n_slices) {
        const i64 row = w * 32 + lane;
        if (row >= a.n_rows) return;
        const int n = a.rlen[row];
        if (n > 32) return;  // a long row: its own warp above
        const int e0 = a.base[w] + lane;
        for (i64 f = 0; f < nrhs; ++f) {
            const float *xf = x + f * ldx;
            float s = 0.f, c = 0.f;
            // kFusedK entries at a time: their loads, then their gathers, then
            // the compensated steps in entry order (two memory round trips a
            // chunk instead of two an entry)
            for (int k0 = 0; k0 < n; k0 += kFusedK) {
                int cl[kFusedK];
                float hv[kFusedK], lv[kFusedK], xv[kFusedK];
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) {
                        const int e = e0 + 32 * (k0 + j);
                        cl[j] = a.col[e];
                        hv[j] = a.hi[e];
                        lv[j] = a.lo[e];
                    }
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) xv[j] = ldg_f(xf + cl[j]);
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) csum1(s, c, hv[j], lv[j], xv[j]);
            }
            const float r = __fadd_rn(s, c);
            y[f * ldy + row] = r;
            if (a.ylo) a.ylo[f * a.ldylo + row] = sum_err(s, c, r);
        }
    }
}

template <int F>
__global__ void __launch_bounds__(256, F <= 2 ? 4 : 2) k_f64_fused(SellArgs a, LongRows L, i64 n_slices,
                                                                 const double *__restrict__ x, i64 ldx,
                                                                 double *__restrict__ y, i64 ldy, i64 nrhs) {
    const int lane = threadIdx.x & 31;
    const i64 wg = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (wg < L.n) {  // long rows first, as k_split_fused
        for (i64 fc = 0; fc * F < nrhs; ++fc) f64_long_row<F>(L, fc * L.n + wg, x, ldx, y, ldy, nrhs);
        return;
    }
    const i64 w = wg - L.n;
    if (w < n_slices) {
        const i64 row = w * 32 + lane;
        if (row >= a.n_rows) return;
        const int n = a.rlen[row];
        if (n > 32) return;
        const int e0 = a.base[w] + lane;
        for (i64 f = 0; f < nrhs; ++f) {
            const double *xf = x + f * ldx;
            double s = 0.0;
            for (int k0 = 0; k0 < n; k0 += kFusedK) {  // as k_split_fused
                int cl[kFusedK];
                double wv[kFusedK], xv[kFusedK];
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) {
                        const int e = e0 + 32 * (k0 + j);
                        cl[j] = a.col[e];
                        wv[j] = a.w64[e];
                    }
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) xv[j] = __ldg(xf + cl[j]);
#pragma unroll
                for (int j = 0; j < kFusedK; ++j)
                    if (k0 + j < n) s = fma(wv[j], xv[j], s);
            }
            y[f * ldy + row] = s;
        }
    }
}

// Row-contiguous copy of the long rows' entries (in the layout's order).
__global__ void k_long_fill(const int *rp, const int *ccol, const double *val, const int *perm, const int *lrow,
                            const int *lptr, i64 n_lrows, int *lcol, float *lhi, float *llo, double *lw64) {
    const i64 i = blockIdx.x;
    if (i >= n_lrows) return;
    const int r = lrow[i], r0 = rp[r], b = lptr[i], n = lptr[i + 1] - b;
    for (int k = threadIdx.x; k < n; k += blockDim.x) {
        const int src = perm ? perm[r0 + k] : r0 + k;
        const double w = val[src];
        lcol[b + k] = ccol[src];
        if (lhi) {
            const float h = __double2float_rn(w);
            lhi[b + k] = h;
            llo[b + k] = __double2float_rn(w - static_cast<double>(h));
        }
        if (lw64) lw64[b + k] = w;
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

// perm (optional): CSR index of the k-th entry of each row (split layouts).
__global__ void k_sell_fill(const int *rp, const int *ccol, const double *val, const int *perm, i64 n_rows,
                            i64 n_slices, const int *base, const int *slen32, int *rlen, int *col, float *hi,
                            float *lo, double *w64) {
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
            const int src = perm ? perm[r0 + k] : r0 + k;
            double w = val[src];
            col[e] = ccol[src];
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
        const int *perm = (fmt == 1 && m.split_perm.p) ? m.split_perm.p : nullptr;
        const int *ccol = (fmt == 1 && m.src_renum) ? m.split_col.p : m.col.p;
        k_sell_fill<<<nblk(n_slices * 32, 256), 256, 0, s>>>(m.row_ptr.p, ccol, m.val.p, perm, n_rows, n_slices,
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
    // rows of more than 32 entries, row-contiguous
    {
        std::vector<int> rp(n_rows + 1);
        AXGB_CUDA(cudaMemcpy(rp.data(), m.row_ptr.p, sizeof(int) * (n_rows + 1), cudaMemcpyDeviceToHost));
        std::vector<int> lrow, lptr(1, 0);
        for (i64 r = 0; r < n_rows; ++r)
            if (rp[r + 1] - rp[r] > 32) {
                lrow.push_back(static_cast<int>(r));
                lptr.push_back(lptr.back() + rp[r + 1] - rp[r]);
            }
        S.n_lrows = static_cast<i64>(lrow.size());
        S.lrow.upload_vec(lrow, s);
        S.lptr.upload_vec(lptr, s);
        const size_t ne = std::max<size_t>(1, lptr.back());
        S.lcol.alloc(ne);
        if (fmt == 1) {
            S.lhi.alloc(ne);
            S.llo.alloc(ne);
        } else {
            S.lw64.alloc(ne);
        }
        if (S.n_lrows > 0) {
            const int *perm = (fmt == 1 && m.split_perm.p) ? m.split_perm.p : nullptr;
            const int *ccol = (fmt == 1 && m.src_renum) ? m.split_col.p : m.col.p;
            k_long_fill<<<static_cast<unsigned>(S.n_lrows), 128, 0, s>>>(
                m.row_ptr.p, ccol, m.val.p, perm, S.lrow.p, S.lptr.p, S.n_lrows, S.lcol.p,
                fmt == 1 ? S.lhi.p : nullptr, fmt == 1 ? S.llo.p : nullptr, fmt == 0 ? S.lw64.p : nullptr);
            AXGB_CUDA(cudaGetLastError());
        }
    }
    S.class_ids.upload(ids.data(), ids.size(), s);
    S.h_slice_len.resize(n_slices);
    for (i64 q = 0; q < n_slices; ++q) S.h_slice_len[q] = h_len[q] / 32;
    // keep row lengths in the len buffer's companion: store rlen in 'len' slot
    S.len = std::move(rlen);
    AXGB_CUDA(cudaStreamSynchronize(s));
    S.built = true;
}

SellArgs sell_args(const Matrix &m, const Sell &S, int cls, float *ylo = nullptr, i64 ldylo = 0) {
    SellArgs a{};
    a.ylo = ylo;
    a.ldylo = ldylo;
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

LongRows long_rows(const Sell &S) {
    LongRows L{};
    L.row = S.lrow.p;
    L.ptr = S.lptr.p;
    L.col = S.lcol.p;
    L.hi = S.lhi.p;
    L.lo = S.llo.p;
    L.w64 = S.lw64.p;
    L.n = S.n_lrows;
    return L;
}

// Slices of the long classes: their short rows (k_*_rows), then every row
// of more than 32 entries (k_*_long).
void launch_split_rows(const SellArgs &a, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    if (a.n_ids == 0 || nrhs == 0) return;
    const i64 warps = a.n_ids * 32 * ((nrhs + 31) / 32);
    k_split_rows<<<nblk(warps * 32, 256), 256, 0, s>>>(a, x, ldx, y, ldy, nrhs);
}
void launch_split_long(const Sell &S, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s,
                       float *ylo = nullptr, i64 ldylo = 0) {
    if (S.n_lrows == 0 || nrhs == 0) return;
    const i64 warps = S.n_lrows * ((nrhs + kLongF - 1) / kLongF);
    LongRows L = long_rows(S);
    L.ylo = ylo;
    L.ldylo = ldylo;
    k_split_long<<<nblk(warps * 32, 256), 256, 0, s>>>(L, x, ldx, y, ldy, nrhs);
}
void launch_f64_rows(const SellArgs &a, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    if (a.n_ids == 0 || nrhs == 0) return;
    const i64 warps = a.n_ids * 32 * ((nrhs + 31) / 32);
    k_f64_rows<<<nblk(warps * 32, 256), 256, 0, s>>>(a, x, ldx, y, ldy, nrhs);
}
void launch_f64_long(const Sell &S, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    if (S.n_lrows == 0 || nrhs == 0) return;
    const i64 warps = S.n_lrows * ((nrhs + kLongF - 1) / kLongF);
    k_f64_long<<<nblk(warps * 32, 256), 256, 0, s>>>(long_rows(S), x, ldx, y, ldy, nrhs);
}
}  // namespace

// Rows of more than 32 entries given row-contiguous (the segmented layout's
// own copy, original source numbering): k_split_long, same summation order.
void launch_long_rows(const int *row, const int *ptr, const int *col, const float *hi, const float *lo, i64 n,
                      const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, cudaStream_t s, float *ylo, i64 ldylo) {
    if (n == 0 || nrhs == 0) return;
    LongRows L{};
    L.row = row;
    L.ptr = ptr;
    L.col = col;
    L.hi = hi;
    L.lo = lo;
    L.n = n;
    L.ylo = ylo;
    L.ldylo = ldylo;
    const i64 warps = n * ((nrhs + kLongF - 1) / kLongF);
    k_split_long<<<nblk(warps * 32, 256), 256, 0, s>>>(L, x, ldx, y, ldy, nrhs);
}

namespace {

// One launch for the whole matrix (few fields): warp per slice, then warp per long row.
void launch_split_fused(const Matrix &m, const Sell &S, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs,
                        cudaStream_t s, float *ylo, i64 ldylo) {
    const i64 warps = S.n_slices + S.n_lrows;
    if (warps == 0 || nrhs == 0) return;
    LongRows L = long_rows(S);
    L.ylo = ylo;
    L.ldylo = ldylo;
    const SellArgs a = sell_args(m, S, 0, ylo, ldylo);
    const unsigned g = nblk(warps * 32, 256);
    if (nrhs == 1)
        k_split_fused<1><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
    else if (nrhs == 2)
        k_split_fused<2><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
    else if (nrhs <= 4)
        k_split_fused<4><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
    else
        k_split_fused<kLongF><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
}
void launch_f64_fused(const Matrix &m, const Sell &S, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs,
                      cudaStream_t s) {
    const i64 warps = S.n_slices + S.n_lrows;
    if (warps == 0 || nrhs == 0) return;
    const SellArgs a = sell_args(m, S, 0);
    const LongRows L = long_rows(S);
    const unsigned g = nblk(warps * 32, 256);
    if (nrhs == 1)
        k_f64_fused<1><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
    else if (nrhs == 2)
        k_f64_fused<2><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
    else
        k_f64_fused<kLongF><<<g, 256, 0, s>>>(a, L, S.n_slices, x, ldx, y, ldy, nrhs);
}

template <int L>
void launch_f64(const SellArgs &a, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, i64 tile, cudaStream_t s) {
    i64 items = ((nrhs + tile - 1) / tile) * a.n_ids;
    if (items == 0) return;
    unsigned blocks = nblk(items * 32, 256);
    if (nrhs >= 4)  // four independent FMA chains and their gathers in flight a thread (eight measured slower)
        k_f64<L, 4><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
    else if (nrhs >= 2)
        k_f64<L, 2><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
    else
        k_f64<L, 1><<<blocks, 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, tile);
}

// ─── NaN-aware and masked FP64 applies ────────────────────────────────────
// nan_batch_apply of include/axis/solver/apply.hpp:359-437 on the FP64
// sliced-ELL layout (each row's entries in CSR order), lane per row: per row
// the total weight, per field the weighted sum and the valid weight, with
// unfused multiply and add in entry order, so the NaN decisions and the
// values match the reference loop bit for bit. 0 < L <= 32: entries cached
// in registers; L == 0: rows of any length, entries re-read per field.
__device__ __forceinline__ double nan_result(double total, double wsum, double valid, double na_thres) {
    if (valid == 0.0 || total == 0.0) return __longlong_as_double(0x7ff8000000000000ll);
    const double frac = __ddiv_rn(valid, total);
    return frac < __dsub_rn(__dsub_rn(1.0, na_thres), 1e-6) ? __longlong_as_double(0x7ff8000000000000ll)
                                                            : __ddiv_rn(wsum, valid);
}

template <int L>
__global__ void __launch_bounds__(256) k_nan_sell(SellArgs a, const double *__restrict__ x, i64 ldx,
                                                  double *__restrict__ y, i64 ldy, i64 nrhs, double na_thres) {
    const int lane = threadIdx.x & 31;
    const i64 item = (static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    if (item >= a.n_ids) return;
    const int sid = a.ids[item];
    const i64 row = static_cast<i64>(sid) * 32 + lane;
    if (row >= a.n_rows) return;
    const int base = a.base[sid] + lane, rl = a.rlen[row];
    if constexpr (L > 0) {
        int c[L];
        double w[L];
        double total = 0.0;
#pragma unroll
        for (int k = 0; k < L; ++k) {
            if (k < rl) {
                c[k] = a.col[base + 32 * k];
                w[k] = a.w64[base + 32 * k];
                total = __dadd_rn(total, w[k]);
            }
        }
        for (i64 v = 0; v < nrhs; ++v) {
            const double *xv = x + v * ldx;
            double wsum = 0.0, valid = 0.0;
#pragma unroll
            for (int k = 0; k < L; ++k) {
                if (k < rl) {
                    const double xk = __ldg(xv + c[k]);
                    if (!isnan(xk)) {
                        wsum = __dadd_rn(wsum, __dmul_rn(w[k], xk));
                        valid = __dadd_rn(valid, w[k]);
                    }
                }
            }
            y[v * ldy + row] = nan_result(total, wsum, valid, na_thres);
        }
    } else {
        // rows of any length (the long classes): fields over gridDim.y, the
        // loads of 8 entries issued ahead of their in-order accumulation
        double total = 0.0;
        for (int k = 0; k < rl; ++k) total = __dadd_rn(total, a.w64[base + 32 * k]);
        for (i64 v = blockIdx.y; v < nrhs; v += gridDim.y) {
            const double *xv = x + v * ldx;
            double wsum = 0.0, valid = 0.0;
            for (int k0 = 0; k0 < rl; k0 += 8) {
                double wk[8], xk[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (k0 + u < rl) {
                        wk[u] = a.w64[base + 32 * (k0 + u)];
                        xk[u] = __ldg(xv + a.col[base + 32 * (k0 + u)]);
                    }
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    if (k0 + u < rl && !isnan(xk[u])) {
                        wsum = __dadd_rn(wsum, __dmul_rn(wk[u], xk[u]));
                        valid = __dadd_rn(valid, wk[u]);
                    }
                }
            }
            y[v * ldy + row] = nan_result(total, wsum, valid, na_thres);
        }
    }
}

// Masked apply of include/axis/solver/apply.hpp:458-532: rows with mask 0
// are not written; the others get the row sum in CSR order.
__global__ void k_masked_apply(const int *__restrict__ rp, const int *__restrict__ col,
                               const double *__restrict__ val, i64 n_dst, const double *__restrict__ x,
                               const int *__restrict__ mask, double *__restrict__ y) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst || (mask && mask[j] == 0)) return;
    double s = 0.0;
    for (int k = rp[j]; k < rp[j + 1]; ++k) s = __dadd_rn(s, __dmul_rn(val[k], __ldg(x + col[k])));
    y[j] = s;
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

// ─── FP64 FMA rate probe ──────────────────────────────────────────────────
// Eight independent dependent-FMA chains per thread (enough to cover the FP64
// pipe's latency), four resident blocks of 256 threads per SM: the FP64 FMA
// throughput the FP64 apply and the clipper are compared against. The
// result is written so the chains are not removed.
__global__ void __launch_bounds__(256) k_fp64_fma(double *out, i64 iters, double b, double c) {
    const double x = 1.0 + 1e-3 * threadIdx.x;
    double a0 = x, a1 = x + 1, a2 = x + 2, a3 = x + 3, a4 = x + 4, a5 = x + 5, a6 = x + 6, a7 = x + 7;
    for (i64 i = 0; i < iters; ++i) {
        a0 = fma(a0, b, c);
        a1 = fma(a1, b, c);
        a2 = fma(a2, b, c);
        a3 = fma(a3, b, c);
        a4 = fma(a4, b, c);
        a5 = fma(a5, b, c);
        a6 = fma(a6, b, c);
        a7 = fma(a7, b, c);
    }
    const double r = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
    if (r == 12345.678) out[0] = r;  // never true for these inputs; keeps the chains live
}

}  // namespace

double fp64_fma_tflops(i64 iters) {
    int dev = 0, sms = 0;
    AXGB_CUDA(cudaGetDevice(&dev));
    AXGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    DBuf<double> out(1);
    cudaEvent_t e0, e1;
    AXGB_CUDA(cudaEventCreate(&e0));
    AXGB_CUDA(cudaEventCreate(&e1));
    const unsigned blocks = static_cast<unsigned>(4 * sms);
    k_fp64_fma<<<blocks, 256>>>(out.p, iters / 8 + 1, 0.999999, 1e-7);  // warm-up
    AXGB_CUDA(cudaEventRecord(e0));
    k_fp64_fma<<<blocks, 256>>>(out.p, iters, 0.999999, 1e-7);
    AXGB_CUDA(cudaEventRecord(e1));
    AXGB_CUDA(cudaEventSynchronize(e1));
    float ms = 0.f;
    AXGB_CUDA(cudaEventElapsedTime(&ms, e0, e1));
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    const double flops = 2.0 * 8.0 * static_cast<double>(iters) * blocks * 256.0;
    return flops / (static_cast<double>(ms) * 1e-3) / 1e12;
}

namespace {

// ─── conservation report without allocation ───────────────────────────────
// For callers that cannot allocate device memory while they run (a model
// whose device memory is owned by its own pool, or code between
// allocation-free phases): the per-block partial sums live in a fixed
// file-scope device array instead of cudaMalloc'd scratch. The call copies
// its two results to the host and synchronises its stream, so it is made
// before or between stream captures, never inside one.
// Each block reduces a fixed span of 2048 cells; the partials are then
// reduced by one block in a fixed order, so results are deterministic.

constexpr int kNaThreads = 256;
constexpr i64 kNaCellsPerBlock = 2048;                      // 8 cells per thread
constexpr int kNaMaxBlocks = 8192;                          // per integral
constexpr i64 kNaMaxCells = kNaCellsPerBlock * kNaMaxBlocks;  // 16,777,216 cells per side
// [0, K): source partials, [K, 2K): destination partials, [2K, 2K+2): results.
// Every slot a call reads is written earlier in the same call.
static __device__ __align__(256) double g_noalloc_scratch[2 * kNaMaxBlocks + 2];

template <class T>
__global__ void k_integral_span(const T *f, const double *area, const double *frac, i64 n, int mode, double *partial) {
    __shared__ double sh[kNaThreads];
    const i64 b0 = static_cast<i64>(blockIdx.x) * kNaCellsPerBlock;
    double acc = 0.0;
    for (int q = 0; q < kNaCellsPerBlock / kNaThreads; ++q) {
        const i64 i = b0 + q * kNaThreads + threadIdx.x;
        if (i < n) {
            double v = static_cast<double>(f[i]);
            if (mode == 0)
                acc += v * area[i] * frac[i];
            else if (frac[i] != 0.0)
                acc += v * area[i];
        }
    }
    sh[threadIdx.x] = acc;
    __syncthreads();
    for (int o = kNaThreads / 2; o > 0; o >>= 1) {
        if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
        __syncthreads();
    }
    if (threadIdx.x == 0) partial[blockIdx.x] = sh[0];
}

// One block: result[w] = sum of partial[w*K .. w*K + nb[w]) for w = 0, 1.
__global__ void k_sum_partials(const double *partial, int nb0, int nb1, double *result) {
    __shared__ double sh[kNaThreads];
    for (int w = 0; w < 2; ++w) {
        const int nb = w == 0 ? nb0 : nb1;
        const double *p = partial + static_cast<i64>(w) * kNaMaxBlocks;
        double acc = 0.0;
        for (int i = threadIdx.x; i < nb; i += kNaThreads) acc += p[i];
        sh[threadIdx.x] = acc;
        __syncthreads();
        for (int o = kNaThreads / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) sh[threadIdx.x] += sh[threadIdx.x + o];
            __syncthreads();
        }
        if (threadIdx.x == 0) result[w] = sh[0];
        __syncthreads();
    }
}

// Device address of g_noalloc_scratch for the current device, looked up
// once per device (the host-side name is not a device address). The cached
// address belongs to the device's current context: after cudaDeviceReset
// it is stale, as is every other handle of this library on that device.
double *noalloc_scratch() {
    static std::mutex mu;
    static double *ptr[256] = {};
    int dev = 0;
    AXGB_CUDA(cudaGetDevice(&dev));
    AXGB_REQUIRE(dev >= 0 && dev < 256, "conservation_noalloc: device ordinal out of range");
    std::lock_guard<std::mutex> lk(mu);
    if (!ptr[dev]) {
        void *p = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess)
            throw Error(AXGB_ERR_CUDA, std::string("cudaGetSymbolAddress(g_noalloc_scratch): ") + cudaGetErrorString(e));
        ptr[dev] = static_cast<double *>(p);
    }
    return ptr[dev];
}

// ─── persistent batch kernel ───────────────────────────────────────────────
// Items of all matrices are handed out by one atomic counter (no waiting):
// item -> (matrix, tile, slice). Entries of up to 32 per row are cached in
// registers; longer rows are read from global memory.
// ROWS: the row items (modes 1, 2), else the slice items (mode 0). The two
// run as separate kernels: the slice items cache 16 entries a lane and need
// about 128 registers (two blocks an SM); the row items are chains of
// dependent gathers that want warps, so their kernel carries four fields a
// long-row item and is held to 64 registers, four blocks an SM (measured on
// the 17-pair batch: 1.14 ms, against 1.18 ms at three blocks, 1.23 ms with
// two fields an item at five, 1.45 ms with eight fields at two).
template <bool ROWS>
__global__ void __launch_bounds__(256, ROWS ? 4 : 2) k_batch(const Batch::Desc *__restrict__ desc, int n_desc, i64 total,
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
        const i64 local = static_cast<i64>(it) - d.item_begin;
        if constexpr (ROWS) {
        if (d.mode == 2) {  // rows of more than 32 entries
            LongRows L{};
            L.row = d.lrow;
            L.ptr = d.lptr;
            L.col = d.lcol;
            L.hi = d.lhi;
            L.lo = d.llo;
            L.w64 = nullptr;
            L.n = d.n_ids;
            split_long_row<kBatchLongF>(L, local, d.x, d.ldx, d.y, d.ldy, d.nrhs);
            continue;
        }
        if (d.mode == 1) {  // short rows of long-class slices: lane = field
            const i64 per = d.n_ids * 32;
            const i64 fc = local / per;
            const i64 q = local - fc * per;
            const int sid = d.ids[q >> 5];
            const int p = static_cast<int>(q & 31);
            const i64 row = static_cast<i64>(sid) * 32 + p;
            const i64 f = fc * 32 + lane;
            if (row < d.n_rows && f < d.nrhs) {
                const int n = d.rlen[row];
                if (n <= 32) {
                    const int e0 = d.base[sid] + p;
                    const float *xf = d.x + f * d.ldx;
                    float s = 0.f, c = 0.f;
                    for (int k = 0; k < n; ++k) {
                        const int e = e0 + 32 * k;
                        csum1(s, c, d.hi[e], d.lo[e], __ldg(xf + d.col[e]));
                    }
                    d.y[f * d.ldy + row] = __fadd_rn(s, c);
                }
            }
            continue;
        }
        } else {
        const i64 t = local / d.n_ids;
        const i64 sid = d.ids[local - t * d.n_ids];
        const i64 row = sid * 32 + lane;
        const int base = d.base[sid];
        const int rl = d.rlen[sid * 32 + lane];
        const i64 f0 = t * d.tile, f1 = min(f0 + d.tile, d.nrhs);
        const bool store = row < d.n_rows;
        constexpr int L = 16;
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
            for (int k = L; k < rl; ++k) {  // rows of 17..32 entries: the tail from global memory
                int e = base + k * 32 + lane;
                csum1(s, cc, d.hi[e], d.lo[e], __ldg(xf + d.col[e]));
            }
            if (store) d.y[f * d.ldy + row] = __fadd_rn(s, cc);
        }
        }
    }
}

}  // namespace

void matrix_prepare(Matrix &m, int format, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(m.mu);
    if (format == 3) {  // segmented layout (it fixes the split order through the blocked build first)
        build_segmented(m, s);
        return;
    }
    if (format >= 1) build_blocked(m, s);  // fixes the split entry order (split_perm) first
    if (format == 2) {
        build_sell(m, 1, s);  // slices of blocks that do not fit the blocked kernels use the direct kernel
        m.stats[6] = blocked_launches(m);
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

namespace {
// xr[f][j] = x[f][inv[j]]: fields into the split layouts' source numbering.
__global__ void k_gather_src(const float *__restrict__ x, i64 ldx, const int *__restrict__ inv, i64 n, i64 nrhs,
                             float *__restrict__ xr, i64 ldr) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    const i64 f = blockIdx.y;
    if (j >= n || f >= nrhs) return;
    xr[f * ldr + j] = __ldg(x + f * ldx + inv[j]);
}
}  // namespace

// Same for a batch member: arguments read from device memory, so a captured
// graph picks up new field pointers.
__global__ void k_gather_desc(const GatherDesc *__restrict__ g) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    const GatherDesc d = *g;
    if (j >= d.n) return;
    for (i64 f = blockIdx.y; f < d.nrhs; f += gridDim.y) d.xr[f * d.ldr + j] = __ldg(d.x + f * d.ldx + d.inv[j]);
}

i64 renum_ld(const Matrix &m) { return (m.n_src + 3) / 4 * 4; }

void gather_source(const Matrix &m, const float *x, i64 ldx, i64 nrhs, float *xr, cudaStream_t s) {
    for (i64 f0 = 0; f0 < nrhs; f0 += 65535) {
        const i64 nf = std::min<i64>(65535, nrhs - f0);
        dim3 grid(nblk(m.n_src, 256), static_cast<unsigned>(nf));
        k_gather_src<<<grid, 256, 0, s>>>(x + f0 * ldx, ldx, m.src_inv.p, m.n_src, nf, xr + f0 * renum_ld(m),
                                           renum_ld(m));
    }
    AXGB_CUDA(cudaGetLastError());
}

void apply_split_layouts(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                         cudaStream_t s, float *ylo, i64 ldylo);

// A renumbered matrix first gathers the fields into stream-ordered scratch
// (cudaMallocAsync, freed on the same stream after the apply).
void apply_split(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                 cudaStream_t s, float *ylo, i64 ldylo) {
    if (nrhs <= 0) return;
    if (p.variant == 5) {  // segmented: cells staged by their own ids, no renumbering gather
        if (!m.seg.built) matrix_prepare(m, 3, s);
        apply_segmented(m, x, ldx, y, ldy, nrhs, s, ylo, ldylo, p.stages);
        return;
    }
    if (!m.blocked.built) matrix_prepare(m, 2, s);
    if (!m.src_renum) {
        apply_split_layouts(m, x, ldx, y, ldy, nrhs, p, s, ylo, ldylo);
        return;
    }
    const i64 ldr = renum_ld(m);
    float *xr = nullptr;
    AXGB_CUDA(cudaMallocAsync(reinterpret_cast<void **>(&xr), sizeof(float) * static_cast<size_t>(ldr * nrhs), s));
    gather_source(m, x, ldx, nrhs, xr, s);
    apply_split_layouts(m, xr, ldr, y, ldy, nrhs, p, s, ylo, ldylo);
    AXGB_CUDA(cudaFreeAsync(xr, s));
}

void apply_split_layouts(Matrix &m, const float *x, i64 ldx, float *y, i64 ldy, i64 nrhs, const SplitParams &p,
                         cudaStream_t s, float *ylo, i64 ldylo) {
    if (nrhs <= 0) return;
    if (p.variant >= 1 && p.variant <= 3 && blocked_eligible(m, x, ldx, p.variant == 2)) {
        if (!m.blocked.built) matrix_prepare(m, 2, s);
        apply_blocked(m, x, ldx, y, ldy, nrhs, p.variant, p.unroll, p.stages, p.fields_per_pass, s, ylo, ldylo);
        const Blocked &B = m.blocked;
        if (B.n_fallback > 0) {
            SellArgs a = sell_args(m, m.sell32, 4, ylo, ldylo);
            a.ids = B.fallback_slices.p;
            a.n_ids = B.n_fallback;
            launch_split_rows(a, x, ldx, y, ldy, nrhs, s);
        }
        launch_split_long(m.sell32, x, ldx, y, ldy, nrhs, s, ylo, ldylo);
        AXGB_CUDA(cudaGetLastError());
        return;
    }
    if (!m.sell32.built) matrix_prepare(m, 1, s);
    const Sell &S = m.sell32;
    if (p.variant == 4) {  // one launch for the whole matrix (few fields)
        launch_split_fused(m, S, x, ldx, y, ldy, nrhs, s, ylo, ldylo);
        AXGB_CUDA(cudaGetLastError());
        return;
    }
    i64 tile = (p.fields_per_pass <= 0 || p.fields_per_pass > nrhs) ? nrhs : p.fields_per_pass;
    const int unroll = p.variant == 0 ? p.unroll : 4;
    launch_split<8>(sell_args(m, S, 0, ylo, ldylo), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<16>(sell_args(m, S, 1, ylo, ldylo), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split<32>(sell_args(m, S, 2, ylo, ldylo), x, ldx, y, ldy, nrhs, tile, unroll, s);
    launch_split_rows(sell_args(m, S, 3, ylo, ldylo), x, ldx, y, ldy, nrhs, s);
    launch_split_rows(sell_args(m, S, 4, ylo, ldylo), x, ldx, y, ldy, nrhs, s);
    launch_split_long(S, x, ldx, y, ldy, nrhs, s, ylo, ldylo);
    AXGB_CUDA(cudaGetLastError());
}

void apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, cudaStream_t s) {
    if (!m.sell64.built) matrix_prepare(m, 0, s);
    const Sell &S = m.sell64;
    i64 tile = nrhs;
    if (tile <= 0) return;
    if (nrhs <= kFusedMaxF64) {  // one launch; same bits as the class kernels
        launch_f64_fused(m, S, x, ldx, y, ldy, nrhs, s);
        AXGB_CUDA(cudaGetLastError());
        return;
    }
    launch_f64<8>(sell_args(m, S, 0), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<16>(sell_args(m, S, 1), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64<32>(sell_args(m, S, 2), x, ldx, y, ldy, nrhs, tile, s);
    launch_f64_rows(sell_args(m, S, 3), x, ldx, y, ldy, nrhs, s);
    launch_f64_rows(sell_args(m, S, 4), x, ldx, y, ldy, nrhs, s);
    launch_f64_long(S, x, ldx, y, ldy, nrhs, s);
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

void conservation_noalloc(Matrix &m, const double *src, const double *dst, int norm_type, double *out,
                          cudaStream_t s) {
    if (m.n_src > kNaMaxCells || m.n_dst > kNaMaxCells)
        throw Error(AXGB_ERR_INVALID, "conservation_noalloc: n_src (" + std::to_string(m.n_src) + ") or n_dst (" +
                                          std::to_string(m.n_dst) + ") exceeds the fixed scratch limit of " +
                                          std::to_string(kNaMaxCells) + " cells; use axgb_conservation_f64");
    double *scr = noalloc_scratch();
    const int nbs = static_cast<int>((m.n_src + kNaCellsPerBlock - 1) / kNaCellsPerBlock);
    const int nbd = static_cast<int>((m.n_dst + kNaCellsPerBlock - 1) / kNaCellsPerBlock);
    if (nbs > 0) k_integral_span<double><<<nbs, kNaThreads, 0, s>>>(src, m.area_a.p, m.frac_a.p, m.n_src, 0, scr);
    if (nbd > 0)
        k_integral_span<double><<<nbd, kNaThreads, 0, s>>>(dst, m.area_b.p, m.frac_b.p, m.n_dst,
                                                           norm_type == 0 ? 1 : 0, scr + kNaMaxBlocks);
    k_sum_partials<<<1, kNaThreads, 0, s>>>(scr, nbs, nbd, scr + 2 * kNaMaxBlocks);
    AXGB_CUDA(cudaGetLastError());
    double two[2] = {0.0, 0.0};
    AXGB_CUDA(cudaMemcpyAsync(two, scr + 2 * kNaMaxBlocks, sizeof(two), cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaStreamSynchronize(s));
    const double si = two[0], di = two[1];
    const double ae = std::abs(si - di);
    const double den = std::max({std::abs(si), std::abs(di), 2.220446049250313e-16});
    out[0] = si;
    out[1] = di;
    out[2] = ae;
    out[3] = ae / den;
}

void nan_batch_apply_f64(Matrix &m, const double *x, i64 ldx, double *y, i64 ldy, i64 nrhs, double na_thres,
                         cudaStream_t s) {
    if (nrhs <= 0 || m.n_dst == 0) return;
    if (!m.sell64.built) matrix_prepare(m, 0, s);
    const Sell &S = m.sell64;
    auto launch = [&](auto kernel, int cls, unsigned gy) {
        const SellArgs a = sell_args(m, S, cls);
        if (a.n_ids > 0) kernel<<<dim3(nblk(a.n_ids * 32, 256), gy), 256, 0, s>>>(a, x, ldx, y, ldy, nrhs, na_thres);
    };
    const unsigned fy = static_cast<unsigned>(std::min<i64>(nrhs, 65535));
    launch(k_nan_sell<8>, 0, 1);
    launch(k_nan_sell<16>, 1, 1);
    launch(k_nan_sell<32>, 2, 1);
    launch(k_nan_sell<0>, 3, fy);
    launch(k_nan_sell<0>, 4, fy);
    AXGB_CUDA(cudaGetLastError());
}

void apply_masked_f64(Matrix &m, const double *x, const int *mask, double *y, cudaStream_t s) {
    if (m.n_dst == 0) return;
    k_masked_apply<<<nblk(m.n_dst, 256), 256, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, m.n_dst, x, mask, y);
    AXGB_CUDA(cudaGetLastError());
}

std::shared_ptr<Batch> batch_create(const std::vector<std::shared_ptr<Matrix>> &mats, const std::vector<i64> &nrhs) {
    auto b = std::make_shared<Batch>();
    b->mats = mats;
    b->nrhs = nrhs;
    for (auto &m : mats) matrix_prepare(*m, 2, 0);
    int dev = 0, sms = 0;
    AXGB_CUDA(cudaGetDevice(&dev));
    AXGB_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    int per_sm = 0;
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<false>, 256, 0));
    b->blocks_slices = std::max(1, sms * std::max(1, per_sm));
    AXGB_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_batch<true>, 256, 0));
    b->blocks_rows = std::max(1, sms * std::max(1, per_sm));
    b->counter.alloc(2);
    return b;
}

namespace {

// Work of the direct persistent kernel: for a matrix on the staged kernels,
// the slices the blocked layout leaves out (their rows of at most 32
// entries) and the rows of more than 32 entries; for the others, all of it.
void plan_direct(Batch &b) {
    b.desc.clear();
    i64 items = 0;
    b.n_slice_desc = 0;
    b.total_slice_items = 0;
    for (int group = 0; group < 2; ++group) {  // slice items (mode 0), then row items (modes 1, 2)
    items = 0;
    for (size_t q = 0; q < b.mats.size(); ++q) {
        Matrix &m = *b.mats[q];
        const Sell &S = m.sell32;
        const i64 k = b.nrhs[q];
        for (int mode = 0; mode < 3; ++mode) {
            if ((mode == 0) != (group == 0)) continue;
            Batch::Desc d{};
            d.base = S.base.p;
            d.len = nullptr;
            d.rlen = S.len.p;
            d.col = S.col.p;
            d.hi = S.hi.p;
            d.lo = S.lo.p;
            d.lrow = S.lrow.p;
            d.lptr = S.lptr.p;
            d.lcol = S.lcol.p;
            d.lhi = S.lhi.p;
            d.llo = S.llo.p;
            d.mode = mode;
            d.mat = static_cast<int>(q);
            d.n_rows = m.n_dst;
            d.n_slices = S.n_slices;
            d.nrhs = k;
            d.tile = std::max<i64>(1, std::min<i64>(k, 8));
            d.n_tiles = (k + d.tile - 1) / d.tile;
            if (mode == 2) {
                d.n_ids = S.n_lrows;
            } else if (b.use[q]) {
                if (mode == 0) continue;
                d.ids = m.blocked.fallback_slices.p;  // classes of the blocked layout's left-out slices
                d.n_ids = m.blocked.n_fallback;
            } else {
                // classes 0..2: slices of rows of at most 32 entries; 3..4: the others
                const i64 c0 = S.class_begin[mode == 0 ? 0 : 3], c1 = S.class_begin[mode == 0 ? 3 : 5];
                d.ids = S.class_ids.p + c0;
                d.n_ids = c1 - c0;
            }
            const i64 n_items = mode == 0   ? d.n_tiles * d.n_ids
                                : mode == 1 ? d.n_ids * 32 * ((k + 31) / 32)
                                            : d.n_ids * ((k + kBatchLongF - 1) / kBatchLongF);
            if (n_items == 0) continue;
            d.item_begin = items;
            items += n_items;
            b.desc.push_back(d);
        }
    }
    if (group == 0) {
        b.n_slice_desc = static_cast<int>(b.desc.size());
        b.total_slice_items = items;
    } else {
        b.total_row_items = items;
    }
    }
    b.total_items = b.total_slice_items + b.total_row_items;
    b.d_desc.alloc(std::max<size_t>(1, b.desc.size()));
}

void drop_graphs(Batch &b) {
    for (auto &g : b.graphs) {
        cudaGraphExecDestroy(g.second.second);
        cudaGraphDestroy(g.second.first);
    }
    b.graphs.clear();
}

}  // namespace

// Ends a stream capture that an exception left open (dropping the partial
// graph) and destroys the private capture stream when there is one.
struct CaptureGuard {
    cudaStream_t st;
    bool own;
    bool open = true;
    ~CaptureGuard() {
        if (open) {
            cudaGraph_t g = nullptr;
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
        }
        if (own) cudaStreamDestroy(st);
    }
};

// Stream-ordered. The first call (and a call whose fields change which
// matrices can use the staged kernels) plans the work and captures a CUDA
// graph per stream; later calls update the field pointers in the device
// descriptors the graph reads and replay it. Calls on different streams are
// ordered after one another on the GPU (they share the batch's device
// buffers).
void batch_apply(Batch &b, const float *const *x, const i64 *ldx, float *const *y, const i64 *ldy, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(b.mu);
    if (!b.done) AXGB_CUDA(cudaEventCreateWithFlags(&b.done, cudaEventDisableTiming));
    if (b.launched && b.last_stream != s) AXGB_CUDA(cudaStreamWaitEvent(s, b.done, 0));
    const size_t nm = b.mats.size();
    std::vector<const void *> ptrs;
    std::vector<char> use(nm, 0);
    // members with renumbered sources read their fields from b.xr (gathered first)
    if (b.xr.size() != nm) b.xr.resize(nm);
    std::vector<const float *> ex(nm);
    std::vector<i64> eld(nm);
    for (size_t q = 0; q < nm; ++q) {
        const Matrix &m = *b.mats[q];
        AXGB_REQUIRE(ldx[q] >= m.n_src && ldy[q] >= m.n_dst, "batch_apply: leading dimension");
        ptrs.push_back(x[q]);
        ptrs.push_back(y[q]);
        ptrs.push_back(reinterpret_cast<const void *>(ldx[q]));
        ptrs.push_back(reinterpret_cast<const void *>(ldy[q]));
        if (m.src_renum) {
            const size_t need = static_cast<size_t>(std::max<i64>(1, renum_ld(m) * b.nrhs[q]));
            if (b.xr[q].n < need) {
                b.xr[q].alloc(need);
                b.planned = false;  // new scratch address: re-plan and re-capture
            }
            ex[q] = b.xr[q].p;
            eld[q] = renum_ld(m);
        } else {
            ex[q] = x[q];
            eld[q] = ldx[q];
        }
        use[q] = (b.nrhs[q] > 0 && m.blocked.built && blocked_eligible(m, ex[q], eld[q], false)) ? 1 : 0;
    }
    if (!b.planned || use != b.use) {
        b.use = use;
        plan_direct(b);
        std::vector<Matrix *> raw;
        for (auto &m : b.mats) raw.push_back(m.get());
        b.blk = blk_batch_create(raw, b.nrhs, b.use);
        drop_graphs(b);
        b.last_ptrs.clear();
        b.planned = true;
    }
    if (ptrs != b.last_ptrs) {
        for (auto &d : b.desc) {
            d.x = ex[d.mat];
            d.ldx = eld[d.mat];
            d.y = y[d.mat];
            d.ldy = ldy[d.mat];
        }
        b.gdesc.clear();
        for (size_t q = 0; q < nm; ++q)
            if (b.mats[q]->src_renum && b.nrhs[q] > 0)
                b.gdesc.push_back({x[q], ldx[q], b.mats[q]->src_inv.p, b.mats[q]->n_src, b.nrhs[q], b.xr[q].p, eld[q]});
        if (b.d_gdesc.n < b.gdesc.size()) b.d_gdesc.alloc(b.gdesc.size());
        // stream-ordered update of the descriptors the graph reads
        if (!b.desc.empty())
            AXGB_CUDA(cudaMemcpyAsync(b.d_desc.p, b.desc.data(), sizeof(Batch::Desc) * b.desc.size(),
                                      cudaMemcpyHostToDevice, s));
        if (!b.gdesc.empty())
            AXGB_CUDA(cudaMemcpyAsync(b.d_gdesc.p, b.gdesc.data(), sizeof(GatherDesc) * b.gdesc.size(),
                                      cudaMemcpyHostToDevice, s));
        blk_batch_set_fields(*b.blk, ex.data(), eld.data(), y, ldy, s);
        AXGB_CUDA(cudaStreamSynchronize(s));
        b.last_ptrs = ptrs;
    }
    auto it = b.graphs.find(s);
    if (it == b.graphs.end()) {
        cudaStream_t cap = s;
        bool own = false;
        if (cap == 0) {  // legacy stream cannot be captured: capture on a private stream
            AXGB_CUDA(cudaStreamCreateWithFlags(&cap, cudaStreamNonBlocking));
            own = true;
        }
        CaptureGuard guard{cap, own};
        cudaGraph_t g;
        cudaGraphExec_t ge;
        AXGB_CUDA(cudaStreamBeginCapture(cap, cudaStreamCaptureModeThreadLocal));
        for (size_t i = 0; i < b.gdesc.size(); ++i) {  // renumbered members: gather their fields first
            const GatherDesc &g = b.gdesc[i];
            dim3 grid(nblk(g.n, 256), static_cast<unsigned>(std::min<i64>(g.nrhs, 65535)));
            k_gather_desc<<<grid, 256, 0, cap>>>(b.d_gdesc.p + i);
        }
        // fork: the direct persistent kernel on its own side stream, the staged
        // class kernels over the others, joined back before the capture ends
        if (!b.fork) {
            AXGB_CUDA(cudaEventCreateWithFlags(&b.fork, cudaEventDisableTiming));
            for (int q = 0; q < Batch::kSide; ++q) {
                AXGB_CUDA(cudaStreamCreateWithFlags(&b.side[q], cudaStreamNonBlocking));
                AXGB_CUDA(cudaEventCreateWithFlags(&b.join[q], cudaEventDisableTiming));
            }
        }
        AXGB_CUDA(cudaEventRecord(b.fork, cap));
        for (int q = 0; q < Batch::kSide; ++q) AXGB_CUDA(cudaStreamWaitEvent(b.side[q], b.fork, 0));
        if (b.total_row_items > 0) {  // the row items (long chains of gathers) on their own side stream
            AXGB_CUDA(cudaMemsetAsync(b.counter.p + 1, 0, sizeof(unsigned long long), b.side[0]));
            k_batch<true><<<b.blocks_rows, 256, 0, b.side[0]>>>(
                b.d_desc.p + b.n_slice_desc, static_cast<int>(b.desc.size()) - b.n_slice_desc, b.total_row_items,
                b.counter.p + 1);
        }
        if (b.total_slice_items > 0) {
            AXGB_CUDA(cudaMemsetAsync(b.counter.p, 0, sizeof(unsigned long long), b.side[1]));
            k_batch<false><<<b.blocks_slices, 256, 0, b.side[1]>>>(b.d_desc.p, b.n_slice_desc, b.total_slice_items,
                                                                   b.counter.p);
        }
        blk_batch_launch(*b.blk, b.side + 2, Batch::kSide - 2);
        for (int q = 0; q < Batch::kSide; ++q) {
            AXGB_CUDA(cudaEventRecord(b.join[q], b.side[q]));
            AXGB_CUDA(cudaStreamWaitEvent(cap, b.join[q], 0));
        }
        guard.open = false;
        AXGB_CUDA(cudaStreamEndCapture(cap, &g));
        cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
        if (e != cudaSuccess) {
            cudaGraphDestroy(g);
            AXGB_CUDA(e);
        }
        it = b.graphs.emplace(s, std::make_pair(g, ge)).first;
    }
    AXGB_CUDA(cudaGraphLaunch(it->second.second, s));
    AXGB_CUDA(cudaEventRecord(b.done, s));
    b.last_stream = s;
    b.launched = true;
}

}  // namespace axgb
