// Weight generation on the device.
//
// Conservative (Conservative1stOrder, GreatCircle) replaces
// generate_conservative_impl<3> (libs/axis/src/solver/weight_generator.cpp:
// 3304-3770):
//   1. cell prep per mesh (prep.cu);
//   2. an LBVH over the source cells' bounding caps: 30-bit Morton codes of
//      the cap centroids, radix-sorted leaves, Karras hierarchy, bottom-up
//      refit of FP32 boxes padded outward, and per-node ropes (escape
//      links) for stackless traversal;
//   3. one thread per destination cell walks the ropes; every leaf hit goes
//      through the reference's exact gates (source mask / degenerate /
//      area > 0, the reference's float AABB test, the FP64 cap test) and is
//      counted (pass 1) or written (pass 2) row-grouped, so the candidate
//      list is deterministic;
//   4. one thread per candidate runs the FP64 great-circle clip and the
//      spherical area (geom.cuh, --fmad=false); pairs whose polygons
//      exceed 16 vertices are redone with the reference's 32-vertex cap;
//   5. kept pairs (overlap > 0, the reference threshold at :3682) are
//      compacted, radix-sorted by (row, col) into CSR, and the weights,
//      frac_b (row order) and frac_a (column order, rows ascending) sums are
//      formed per row / per column by one thread each.
// Bilinear with a rectilinear source replaces
// generate_bilinear_rect_nonuniform
// (src/solver/weight_generator_bilinear_rect_nonuniform.cpp:22-149).
#include <chrono>

#include "geom.cuh"
#include "internal.hpp"
#include "lbvh.cuh"

namespace axgb {
namespace {

constexpr unsigned char kExcluded = 1 | 2 | 4;  // degenerate | masked | area <= 0

// ─── LBVH (lbvh.cuh) ───────────────────────────────────────────────────────

// Chord radius of a cap of angular radius r, rounded up into float with
// slack for the float rounding of the centre (|dc| <= 2^-24 per axis).
__device__ __forceinline__ float ball_radius(double r) {
    double rho = 2.0 * sin(0.5 * fmin(r, 3.141592653589793));
    return __double2float_ru(rho * (1.0 + 1e-6) + 1e-6);
}

__global__ void k_leaf_keys(MeshView S, unsigned *keys, int *vals) {
    i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= S.n_cells) return;
    DCap c = S.cap[i];
    keys[i] = morton30(c.x, c.y, c.z);
    vals[i] = static_cast<int>(i);
}

__global__ void k_leaves(Bvh t, MeshView S, const int *vals) {
    int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= t.n) return;
    int cell = vals[q];
    DCap c = S.cap[cell];
    float r = ball_radius(c.r);
    float4 lo, hi;
    lo.x = __fsub_rd(__double2float_rd(c.x), r);
    lo.y = __fsub_rd(__double2float_rd(c.y), r);
    lo.z = __fsub_rd(__double2float_rd(c.z), r);
    hi.x = __fadd_ru(__double2float_ru(c.x), r);
    hi.y = __fadd_ru(__double2float_ru(c.y), r);
    hi.z = __fadd_ru(__double2float_ru(c.z), r);
    lo.w = __int_as_float(cell);
    hi.w = __int_as_float(-1);
    t.lo[t.n - 1 + q] = lo;
    t.hi[t.n - 1 + q] = hi;
}

// ─── candidate search (two passes) ─────────────────────────────────────────

__device__ __forceinline__ bool fbox_meet(const float *a, const float *b) {
#pragma unroll
    for (int d = 0; d < 3; ++d)
        if (a[d] > b[3 + d] || a[3 + d] < b[d]) return false;
    return true;
}

// The cap test acos(clamp(dot(c_s, c_d))) > r_s + r_d is taken in FP64 as
// the reference takes it (spherical_cap_filter.hpp:190-197), but most pairs
// are decided in FP32 first. On unit vectors the angle exceeds R exactly
// when the chord |c_s - c_d| exceeds 2 sin(R/2) (for R below pi, where
// both sides are monotone). From the float copies of the centroids and
// radii (rounding 6e-8 relative each) the float chord lies within 1.1e-6
// of the chord of the double centroids, and 2 sinf(R/2) within 0.6e-6 of
// its double value; the FP64 acos and sum differ from the exact angle and
// sum by less than 2e-8. So when the float sides differ by more than
// kCapMargin, the FP64 test returns the same answer. Nearer pairs, and sums
// above 3, take the FP64 test.
constexpr float kCapMargin = 4.0e-6f;

// Exact reference gates for a pair that the LBVH admitted.
__device__ __forceinline__ bool gate(const MeshView &S, int i, const float *dbox, const DCap &dc, const float4 &dcf) {
    if (S.flags[i] & kExcluded) return false;
    if (!fbox_meet(S.box + 6 * static_cast<i64>(i), dbox)) return false;
    const float4 sf = S.capf[i];
    const float rs = sf.w + dcf.w;
    if (rs < 3.0f) {
        const float ex = sf.x - dcf.x, ey = sf.y - dcf.y, ez = sf.z - dcf.z;
        const float ch = sqrtf(ex * ex + ey * ey + ez * ez);
        const float t = 2.0f * sinf(0.5f * rs);
        if (ch > t + kCapMargin) return false;
        if (ch < t - kCapMargin) return true;
    }
    DCap sc = S.cap[i];
    double cd = sc.x * dc.x + sc.y * dc.y + sc.z * dc.z;  // dot(centroid_s, centroid_d)
    cd = fmin(1.0, fmax(-1.0, cd));
    return !(acos(cd) > (sc.r + dc.r));
}

template <bool FILL>
__global__ void k_search(MeshView S, MeshView D, const float4 *__restrict__ nlo, const float4 *__restrict__ nhi,
                         int root, int n_leaf_base, int *counts, const i64 *offs, int *out_src,
                         unsigned long long *raw_hits, int *err) {
    i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    unsigned long long hits = 0;
    if (j < D.n_cells) {
        int cnt = 0;
        if (!(D.flags[j] & kExcluded) && root >= 0) {
            DCap dc = D.cap[j];
            const float4 dcf = D.capf[j];
            float dbox[6];
#pragma unroll
            for (int d = 0; d < 6; ++d) dbox[d] = D.box[6 * j + d];
            float qx = static_cast<float>(dc.x), qy = static_cast<float>(dc.y), qz = static_cast<float>(dc.z);
            float rq = ball_radius(dc.r);
            float rq2 = __fmul_ru(rq, rq) * 1.000001f + 1e-12f;
            i64 wbase = FILL ? offs[j] : 0;
            int node = root;
            // Ropes visit every node at most once; a longer walk means a
            // malformed tree: flag it and stop instead of spinning.
            const int max_steps = 2 * (2 * n_leaf_base + 1) + 8;
            int steps = 0;
            while (node >= 0) {
                if (++steps > max_steps) {
                    atomicOr(err, 1);
                    break;
                }
                float4 lo = nlo[node], hi = nhi[node];
                float dx = fmaxf(fmaxf(lo.x - qx, 0.f), qx - hi.x);
                float dy = fmaxf(fmaxf(lo.y - qy, 0.f), qy - hi.y);
                float dz = fmaxf(fmaxf(lo.z - qz, 0.f), qz - hi.z);
                float d2 = dx * dx + dy * dy + dz * dz;
                if (d2 <= rq2) {
                    if (node >= n_leaf_base) {
                        int cell = __float_as_int(lo.w);
                        ++hits;
                        if (gate(S, cell, dbox, dc, dcf)) {
                            if (FILL) out_src[wbase + cnt] = cell;
                            ++cnt;
                        }
                        node = __float_as_int(hi.w);
                    } else {
                        node = __float_as_int(lo.w);
                    }
                } else {
                    node = __float_as_int(hi.w);
                }
            }
        }
        if (!FILL) counts[j] = cnt;
    }
    if (!FILL) {
        // warp-aggregated counter of raw leaf hits
        for (int o = 16; o > 0; o >>= 1) hits += __shfl_down_sync(0xffffffffu, hits, o);
        if ((threadIdx.x & 31) == 0 && hits) atomicAdd(raw_hits, hits);
    }
}

__global__ void k_fill_rows(const i64 *offs, i64 n_dst, int *out_dst) {
    i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    for (i64 k = offs[j]; k < offs[j + 1]; ++k) out_dst[k] = static_cast<int>(j);
}

// ─── clipping ──────────────────────────────────────────────────────────────

template <int CAP>
__device__ __forceinline__ void load_poly(const MeshView &m, i64 c, DPoly<CAP> &p) {
    p.clear();
    if (m.regular) {
        // node trig cache (trig_cache.hpp:284-289, weight_generator.cpp:492-520)
        const int ni = m.ni, nj = m.nj;
        const double *slon = m.trig, *clon = m.trig + (ni + 1), *slat = m.trig + 2 * (ni + 1),
                     *clat = m.trig + 2 * (ni + 1) + (nj + 1);
        i64 ci = c % ni, cj = c / ni;
        auto at = [&](i64 i, i64 j) {
            double cl = clat[j];
            p.push({cl * clon[i], cl * slon[i], slat[j]});
        };
        at(ci, cj);
        at(ci + 1, cj);
        at(ci + 1, cj + 1);
        at(ci, cj + 1);
    } else {
        const int b = m.off[c], e = m.off[c + 1];
        for (int k = b; k < e && k < b + 32; ++k) {
            const double *q = m.xyz + 3 * static_cast<i64>(m.idx[k]);
            p.push({q[0], q[1], q[2]});
        }
    }
}

template <int CAP>
__global__ void __launch_bounds__(128) k_clip(MeshView S, MeshView D, const int *__restrict__ cs,
                                              const int *__restrict__ cd, i64 n, const int *list, double *ov,
                                              int *over_list, int *n_over) {
    i64 t = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (t >= n) return;
    i64 k = list ? list[t] : t;
    DPoly<CAP> sp, dp, ba, bb;
    load_poly(S, cs[k], sp);
    load_poly(D, cd[k], dp);
    bool over = false;
    double a = d_overlap_area(sp, dp, ba, bb, &over);
    if (over && CAP < 32) {
        int q = atomicAdd(n_over, 1);
        over_list[q] = static_cast<int>(k);
        ov[k] = 0.0;
    } else {
        ov[k] = a;
    }
}

// ─── assembly ──────────────────────────────────────────────────────────────

__global__ void k_keep_flags(const double *ov, i64 n, int *keep) {
    i64 k = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) keep[k] = ov[k] > 0.0 ? 1 : 0;
}

__global__ void k_compact(const double *ov, const double *fac, const int *cs, const int *cd, const i64 *pos, i64 n,
                          std::uint64_t *key, int *vals, double *kov, double *kfac) {
    i64 k = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    if (ov[k] > 0.0) {
        i64 p = pos[k];
        key[p] = (static_cast<unsigned long long>(cd[k]) << 32) | static_cast<unsigned>(cs[k]);
        vals[p] = static_cast<int>(p);
        kov[p] = ov[k];
        if (fac) kfac[p] = fac[k];
    }
}

__global__ void k_count_keys(const std::uint64_t *key, i64 n, int *cnt) {
    i64 k = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) atomicAdd(&cnt[key[k] >> 32], 1);
}

__global__ void k_csr_cols(const std::uint64_t *key, const int *perm, const double *kov, const double *kfac, i64 n,
                           int *col, double *ov_sorted, double *fac_sorted, std::uint64_t *key2, int *vals2) {
    i64 k = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k >= n) return;
    unsigned long long kk = key[k];
    unsigned i = static_cast<unsigned>(kk & 0xffffffffu);
    unsigned j = static_cast<unsigned>(kk >> 32);
    col[k] = static_cast<int>(i);
    ov_sorted[k] = kov[perm[k]];
    if (kfac) fac_sorted[k] = kfac[perm[k]];
    key2[k] = (static_cast<unsigned long long>(i) << 32) | j;
    vals2[k] = static_cast<int>(k);
}

// Weights and frac_b per row (weight_generator.cpp:3684-3716); fb_pre, when
// given, holds the row sums already taken in the generator's own order.
__global__ void k_rows(const int *row_ptr, const double *ov, const double *area_dst, const double *fb_pre, i64 n_dst,
                       int fracarea, double *w, double *frac_b) {
    i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    double ad = area_dst[j];
    double fb = 0.0;
    for (int k = row_ptr[j]; k < row_ptr[j + 1]; ++k) {
        double o = ov[k];
        double wij = o / ad;
        w[k] = fmax(wij, 0.0);
        fb += o / ad;
    }
    if (fb_pre) fb = fb_pre[j];
    if (fracarea && fb > 0.0)
        for (int k = row_ptr[j]; k < row_ptr[j + 1]; ++k) w[k] /= fb;
    frac_b[j] = fmin(fb, 1.0);
}

// frac_a per source cell, contributions in ascending row order: ov / area,
// or the per-pair contributions fac when the generator gives them.
__global__ void k_cols(const int *col_ptr, const int *perm2, const double *ov, const double *fac,
                       const double *area_src, i64 n_src, double *frac_a) {
    i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i >= n_src) return;
    double as = area_src[i];
    double fa = 0.0;
    for (int k = col_ptr[i]; k < col_ptr[i + 1]; ++k) fa += fac ? fac[perm2[k]] : ov[perm2[k]] / as;
    frac_a[i] = fmin(fa, 1.0);
}

__global__ void k_unmapped(MeshView D, const int *row_ptr, int *bad) {
    i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= D.n_cells) return;
    unsigned char f = D.flags[j];
    if (f & (1 | 2)) return;  // degenerate or masked
    if ((f & 4) || row_ptr[j + 1] == row_ptr[j]) atomicAdd(bad, 1);
}

// ─── bilinear (rectilinear source) ─────────────────────────────────────────

__device__ int upper_bound_d(const double *a, int n, double v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        int mid = (lo + hi) >> 1;
        if (!(v < a[mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__global__ void k_bilinear(MeshView D, const double *clon, int ni, const double *clat, int nj, int *row_ptr, int *col,
                           double *w) {
    i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c > D.n_cells) return;
    row_ptr[c] = static_cast<int>(4 * c);
    if (c == D.n_cells) return;
    int b = D.off[c], e = D.off[c + 1];
    double ls = 0.0, ts = 0.0;
    for (int k = b; k < e; ++k) {
        i64 n = D.idx[k];
        ls += D.lonlat[n];
        ts += D.lonlat[n + D.n_nodes];
    }
    double ld = ls / static_cast<double>(e - b);
    double td = ts / static_cast<double>(e - b);
    int i = upper_bound_d(clon, ni, ld) - 1;
    int j = upper_bound_d(clat, nj, td) - 1;
    if (i < 0) i = 0;
    if (i >= ni - 1) i = ni - 2;
    if (i < 0) i = 0;
    if (j < 0) j = 0;
    if (j >= nj - 1) j = nj - 2;
    if (j < 0) j = 0;
    double x0 = clon[i], x1 = clon[i + 1], y0 = clat[j], y1 = clat[j + 1];
    double tx = (ld - x0) / (x1 - x0);
    double ty = (td - y0) / (y1 - y0);
    tx = fmax(0.0, fmin(1.0, tx));
    ty = fmax(0.0, fmin(1.0, ty));
    i64 o = 4 * c;
    col[o] = j * ni + i;
    col[o + 1] = j * ni + i + 1;
    col[o + 2] = (j + 1) * ni + i;
    col[o + 3] = (j + 1) * ni + i + 1;
    w[o] = (1.0 - tx) * (1.0 - ty);
    w[o + 1] = tx * (1.0 - ty);
    w[o + 2] = (1.0 - tx) * ty;
    w[o + 3] = tx * ty;
}

// Regular x regular bilinear: generate_bilinear_rect
// (src/solver/weight_generator_bilinear_rect.cpp:31-320), one thread per
// destination cell. The point is the mean of the cell's vertex (lon, lat)
// degrees, wrapped into [lon_min, lon_min + 360) on a periodic source; its
// fractional cell-centre index is bounds-tested with a 1e-9 slack, floored,
// clamped (wrapped in longitude when periodic), and the four weights are
// written column-ascending (ties in emission order, as a stable to_csr).
// cnt = 4 for a mapped row, 0 otherwise.
struct BilRegArgs {
    double lon_min, lat_min, dlon, dlat;
    int ni, nj;
    bool periodic;
};

__global__ void k_bilinear_reg(MeshView D, BilRegArgs g, int *cnt, int *col4, double *w4, int *gen4,
                               int *n_unmapped) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= D.n_cells) return;
    const int b = D.off[c], e = D.off[c + 1];
    double ls = 0.0, ts = 0.0;
    for (int k = b; k < e; ++k) {
        const i64 n = D.idx[k];
        ls += D.lonlat[n];
        ts += D.lonlat[n + D.n_nodes];
    }
    double ld = ls / static_cast<double>(e - b);
    const double td = ts / static_cast<double>(e - b);
    if (g.periodic) {
        double off = ld - g.lon_min;
        off = off - floor(off / 360.0) * 360.0;
        ld = g.lon_min + off;
    }
    const double fi = (ld - g.lon_min) / g.dlon - 0.5, fj = (td - g.lat_min) / g.dlat - 0.5;
    const double tol = 1.0e-9;
    bool inside = fj >= -0.5 - tol && fj <= static_cast<double>(g.nj) - 0.5 + tol;
    if (!g.periodic) inside = inside && fi >= -0.5 - tol && fi <= static_cast<double>(g.ni) - 0.5 + tol;
    if (!inside) {
        cnt[c] = 0;
        atomicAdd(n_unmapped, 1);
        return;
    }
    int i = static_cast<int>(floor(fi)), j = static_cast<int>(floor(fj));
    j = max(0, min(j, g.nj - 2));
    i = g.periodic ? ((i % g.ni) + g.ni) % g.ni : max(0, min(i, g.ni - 2));
    const double tx = fmin(1.0, fmax(0.0, fi - static_cast<double>(i)));
    const double ty = fmin(1.0, fmax(0.0, fj - static_cast<double>(j)));
    int i1 = i + 1;
    if (i1 >= g.ni) i1 = g.periodic ? 0 : g.ni - 1;
    const int j1 = min(j + 1, g.nj - 1);
    int cc[4] = {j * g.ni + i, j * g.ni + i1, j1 * g.ni + i, j1 * g.ni + i1};
    double ww[4] = {(1.0 - tx) * (1.0 - ty), tx * (1.0 - ty), (1.0 - tx) * ty, tx * ty};
    int rk[4] = {0, 1, 2, 3};  // corner = place in the generation order
    for (int a = 1; a < 4; ++a)  // stable insertion sort by column
        for (int q = a; q > 0 && cc[q - 1] > cc[q]; --q) {
            const int tc = cc[q];
            cc[q] = cc[q - 1];
            cc[q - 1] = tc;
            const double tw = ww[q];
            ww[q] = ww[q - 1];
            ww[q - 1] = tw;
            const int tr = rk[q];
            rk[q] = rk[q - 1];
            rk[q - 1] = tr;
        }
    cnt[c] = 4;
    for (int k = 0; k < 4; ++k) {
        col4[4 * c + k] = cc[k];
        w4[4 * c + k] = ww[k];
        gen4[4 * c + k] = rk[k];
    }
}

__global__ void k_bilinear_reg_pack(const int *row_ptr, const int *cnt, const int *col4, const double *w4,
                                    const int *gen4, i64 n_dst, int *col, double *w, int *gen, double *frac_b) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n_dst) return;
    const int p = row_ptr[c];
    for (int k = 0; k < cnt[c]; ++k) {
        col[p + k] = col4[4 * c + k];
        w[p + k] = w4[4 * c + k];
        gen[p + k] = gen4[4 * c + k];
    }
    frac_b[c] = cnt[c] ? 1.0 : 0.0;
}

__global__ void k_fill(double *a, i64 n, double v) {
    i64 k = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (k < n) a[k] = v;
}

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// ─── regular x regular conservative fast path ──────────────────────────────
// generate_conservative_rect (src/solver/weight_generator_conservative_rect.cpp
// :87-415): per destination cell the overlapping source cells by index
// arithmetic and their exact spherical-rectangle overlap (:50-66), one thread
// per destination cell, counted (pass 1) then written (pass 2) in the
// reference's (js, is) loop order.
struct RectGrid {
    i64 ni, nj;
    double lon_min, dlon, lat_min, dlat;
};
struct RectArgs {
    RectGrid sg, dg;
    bool src_global;
    const double *sa, *da;  // cell areas
    const int *smask, *dmask;
    i64 n_src, n_dst;
};

__device__ __forceinline__ double band_area(double lo, double dlat, double dlon) {
    constexpr double d2r = 3.14159265358979323846 / 180.0;
    const double hi = lo + dlat;
    return (dlon * d2r) * (sin(hi * d2r) - sin(lo * d2r));
}

__global__ void k_band_area(RectGrid g, const double *user, i64 n, double *area) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    area[c] = user ? user[c] : band_area(g.lat_min + static_cast<double>(c / g.ni) * g.dlat, g.dlat, g.dlon);
}

template <bool FILL>
__global__ void k_rect(RectArgs a, int *count, const i64 *offs, int *cs, int *cd, double *ov, double *fb) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= a.n_dst) return;
    int n = 0;
    double fbj = 0.0;  // frac_b in the reference's emission order
    i64 at = FILL ? offs[j] : 0;
    const i64 jd = j / a.dg.ni, id = j - jd * a.dg.ni;
    if (!(a.dmask && a.dmask[j] == 0) && a.da[j] > 0.0) {
        const double d_lo_x = a.dg.lon_min + static_cast<double>(id) * a.dg.dlon, d_hi_x = d_lo_x + a.dg.dlon;
        const double d_lo_y = a.dg.lat_min + static_cast<double>(jd) * a.dg.dlat, d_hi_y = d_lo_y + a.dg.dlat;
        double dlx = d_lo_x, dhx = d_hi_x;
        if (a.src_global) {
            const double shift = 360.0 * floor((d_lo_x - a.sg.lon_min) / 360.0);
            dlx = d_lo_x - shift;
            dhx = d_hi_x - shift;
        }
        const int sni = static_cast<int>(a.sg.ni), snj = static_cast<int>(a.sg.nj);
        int is_lo = static_cast<int>(floor((dlx - a.sg.lon_min) / a.sg.dlon));
        int is_hi = static_cast<int>(floor((dhx - a.sg.lon_min) / a.sg.dlon));
        int js_lo = static_cast<int>(floor((d_lo_y - a.sg.lat_min) / a.sg.dlat));
        int js_hi = static_cast<int>(floor((d_hi_y - a.sg.lat_min) / a.sg.dlat));
        if (!a.src_global) {
            is_lo = max(0, is_lo);
            is_hi = min(sni - 1, is_hi);
        }
        js_lo = max(0, js_lo);
        js_hi = min(snj - 1, js_hi);
        constexpr double d2r = 3.14159265358979323846 / 180.0;
        if (is_lo <= is_hi && js_lo <= js_hi) {
            for (int js = js_lo; js <= js_hi; ++js)
                for (int is = is_lo; is <= is_hi; ++is) {
                    const int ia = a.src_global ? ((is % sni) + sni) % sni : is;
                    const i64 c = static_cast<i64>(js) * sni + ia;
                    if (c >= a.n_src || (a.smask && a.smask[c] == 0) || a.sa[c] <= 0.0) continue;
                    const double s_lo_x = a.sg.lon_min + static_cast<double>(is) * a.sg.dlon, s_hi_x = s_lo_x + a.sg.dlon;
                    const double s_lo_y = a.sg.lat_min + static_cast<double>(js) * a.sg.dlat, s_hi_y = s_lo_y + a.sg.dlat;
                    const double dx = fmax(0.0, fmin(s_hi_x, dhx) - fmax(s_lo_x, dlx));
                    const double lo_y = fmax(s_lo_y, d_lo_y), hi_y = fmin(s_hi_y, d_hi_y);
                    if (hi_y <= lo_y || dx <= 0.0) continue;
                    const double o = (dx * d2r) * (sin(hi_y * d2r) - sin(lo_y * d2r));
                    if (o <= 0.0) continue;
                    if (FILL) {
                        cs[at] = static_cast<int>(c);
                        cd[at] = static_cast<int>(j);
                        ov[at] = o;
                        fbj += o / a.da[j];
                        ++at;
                    } else {
                        ++n;
                    }
                }
        }
    }
    if (!FILL) count[j] = n;
    if (FILL) fb[j] = fbj;
}

// Non-uniform rectilinear grids: generate_conservative_rect_nonuniform
// (src/solver/weight_generator_conservative_rect_nonuniform.cpp:52-311). Cell
// c is (c % ni, c / ni) on the sorted unique edge coordinates ulon/ulat.
struct RectNuGrid {
    int ni, nj;
    const double *ulon, *ulat;  // ni+1, nj+1 edges
};
struct RectNuArgs {
    RectNuGrid sg, dg;
    bool src_global;
    double s_lon_min, s_lon_max;
    const double *s_user, *d_user;  // mesh cell areas, or null
    const int *smask, *dmask;
    i64 n_src, n_dst;
};

__device__ __forceinline__ double band_area_edges(double lo_x, double hi_x, double lo_y, double hi_y) {
    constexpr double d2r = 3.14159265358979323846 / 180.0;
    double dlon = hi_x - lo_x;
    dlon *= d2r;
    return dlon * (sin(hi_y * d2r) - sin(lo_y * d2r));
}

__device__ __forceinline__ int lower_bound_d(const double *a, int n, double v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] < v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ int upper_bound_e(const double *a, int n, double v) {
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (!(v < a[mid])) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}

// Reported areas from the unshifted edges (:251-300).
__global__ void k_edge_area(RectNuGrid g, const double *user, i64 n, double *area) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n) return;
    const i64 ci = c % g.ni, cj = c / g.ni;
    area[c] = user ? user[c] : band_area_edges(g.ulon[ci], g.ulon[ci + 1], g.ulat[cj], g.ulat[cj + 1]);
}

// One thread per destination cell, in the reference's loop order: the
// destination box (shifted by whole turns onto a global source), its area
// from those shifted edges, binary searches for the source index ranges
// (:140-156), then every (js, is) with overlap > 1e-12 and a positive source
// area, that area taken from the source edges as placed (+360 past the last
// column). FILL writes the pairs, the overlap, the frac_a contribution, the
// row's frac_b (emission order) and the area the weights divide by.
template <bool FILL>
__global__ void k_rect_nu(RectNuArgs a, int *count, const i64 *offs, int *cs, int *cd, double *ov, double *fac,
                          double *fb, double *da_w) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= a.n_dst) return;
    int n = 0;
    i64 at = FILL ? offs[j] : 0;
    double fbj = 0.0, area_dst = 0.0;
    const int sni = a.sg.ni, snj = a.sg.nj;
    const i64 jd = j / a.dg.ni, id = j - jd * a.dg.ni;
    if (!(a.dmask && a.dmask[j] == 0)) {
        const double d_lo_y = a.dg.ulat[jd], d_hi_y = a.dg.ulat[jd + 1];
        double dlx = a.dg.ulon[id], dhx = a.dg.ulon[id + 1];
        if (a.src_global) {
            const double shift = 360.0 * floor((dlx - a.s_lon_min) / 360.0);
            dlx = dlx - shift;
            dhx = dhx - shift;
        }
        area_dst = a.d_user ? a.d_user[j] : band_area_edges(dlx, dhx, d_lo_y, d_hi_y);
        if (area_dst > 0.0) {
            const int is0 = max(0, lower_bound_d(a.sg.ulon, sni + 1, dlx) - 1);
            int is1 = upper_bound_e(a.sg.ulon, sni + 1, dhx);
            if (!a.src_global || dhx <= a.s_lon_max) is1 = min(sni - 1, is1);
            const int js0 = max(0, lower_bound_d(a.sg.ulat, snj + 1, d_lo_y) - 1);
            const int js1 = min(snj - 1, upper_bound_e(a.sg.ulat, snj + 1, d_hi_y));
            constexpr double d2r = 3.14159265358979323846 / 180.0;
            for (int js = js0; js <= js1; ++js)
                for (int is = is0; is <= is1; ++is) {
                    const int ia = a.src_global ? ((is % sni) + sni) % sni : is;
                    const i64 c = ia + static_cast<i64>(js) * sni;
                    if (a.smask && a.smask[c] == 0) continue;
                    double s_lo_x = a.sg.ulon[ia], s_hi_x = a.sg.ulon[ia + 1];
                    if (a.src_global && is >= sni) {
                        s_lo_x += 360.0;
                        s_hi_x += 360.0;
                    }
                    const double s_lo_y = a.sg.ulat[js], s_hi_y = a.sg.ulat[js + 1];
                    const double dx = fmax(0.0, fmin(s_hi_x, dhx) - fmax(s_lo_x, dlx));
                    const double lo_y = fmax(s_lo_y, d_lo_y), hi_y = fmin(s_hi_y, d_hi_y);
                    if (hi_y <= lo_y || dx <= 0.0) continue;
                    const double o = (dx * d2r) * (sin(hi_y * d2r) - sin(lo_y * d2r));
                    if (!(o > 1e-12)) continue;
                    const double area_src = a.s_user ? a.s_user[c] : band_area_edges(s_lo_x, s_hi_x, s_lo_y, s_hi_y);
                    if (area_src <= 0.0) continue;
                    if (FILL) {
                        cs[at] = static_cast<int>(c);
                        cd[at] = static_cast<int>(j);
                        ov[at] = o;
                        fac[at] = o / area_src;
                        fbj += o / area_dst;
                        ++at;
                    } else {
                        ++n;
                    }
                }
        }
    }
    if (!FILL) count[j] = n;
    if (FILL) {
        fb[j] = fbj;
        da_w[j] = area_dst;
    }
}

using Clock = std::chrono::steady_clock;
inline double ms_since(Clock::time_point t0) {
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

}  // namespace

// What a fast path hands the assembly besides (cs, cd, ov).
struct AssembleOpts {
    const double *fac = nullptr;         // per-pair frac_a contribution (instead of ov / area_src)
    const double *fb_pre = nullptr;      // per-row frac_b, summed in the generator's order
    const double *area_a_out = nullptr;  // reported areas, when not the ones the weights divide by
    const double *area_b_out = nullptr;
    bool check_unmapped = true;          // the general path's UnmappedAction::Error check
    bool keep_gen = false;               // keep each entry's candidate position (generation order)
};

// Kept pairs (overlap > 0, weight_generator.cpp:3682) of the candidate list
// (cs, cd, ov) into the CSR of out: weights, frac_b per row and frac_a per
// column (the steps of :3684-3724), areas copied from area_src / area_dst.
static void assemble(DBuf<int> &cs, DBuf<int> &cd, DBuf<double> &ov, i64 n_cand, const double *area_src,
                     const double *area_dst, const MeshView &D, const axgb_regrid_config &cfg, Matrix &out,
                     cudaStream_t s, const AssembleOpts &o = AssembleOpts{}) {
    const i64 n_src = out.n_src, n_dst = out.n_dst;
    DBuf<int> keep(n_cand);
    DBuf<i64> pos(n_cand + 1);
    i64 nnz = 0;
    if (n_cand > 0) {
        k_keep_flags<<<nblk(n_cand, 256), 256, 0, s>>>(ov.p, n_cand, keep.p);
        scan_exclusive_i32_to_i64(keep.p, pos.p, n_cand, s);
        AXGB_CUDA(cudaMemcpy(&nnz, pos.p + n_cand, sizeof(i64), cudaMemcpyDeviceToHost));
    }
    DBuf<std::uint64_t> key(nnz), key2(nnz);
    DBuf<int> vals(nnz), vals2(nnz);
    DBuf<double> kov(nnz), kfac(o.fac ? nnz : 0), facs(o.fac ? nnz : 0);
    out.row_ptr.alloc(n_dst + 1);
    out.col.alloc(nnz);
    out.val.alloc(nnz);
    out.frac_a.alloc(n_src);
    out.frac_b.alloc(n_dst);
    out.area_a.alloc(n_src);
    out.area_b.alloc(n_dst);
    DBuf<double> ovs(nnz);
    DBuf<int> rcnt(n_dst), ccnt(n_src), col_ptr(n_src + 1);
    rcnt.zero(s);
    ccnt.zero(s);
    if (nnz > 0) {
        k_compact<<<nblk(n_cand, 256), 256, 0, s>>>(ov.p, o.fac, cs.p, cd.p, pos.p, n_cand, key.p, vals.p, kov.p,
                                                    kfac.p);
        int rbits = 32;
        while (rbits < 64 && (static_cast<unsigned long long>(n_dst) >> (rbits - 32)) > 0) ++rbits;
        radix_sort_pairs_u64(key.p, vals.p, nnz, rbits, s);
        k_count_keys<<<nblk(nnz, 256), 256, 0, s>>>(key.p, nnz, rcnt.p);
        k_csr_cols<<<nblk(nnz, 256), 256, 0, s>>>(key.p, vals.p, kov.p, o.fac ? kfac.p : nullptr, nnz, out.col.p,
                                                  ovs.p, facs.p, key2.p, vals2.p);
        AXGB_CUDA(cudaGetLastError());
        int cbits = 32;
        while (cbits < 64 && (static_cast<unsigned long long>(n_src) >> (cbits - 32)) > 0) ++cbits;
        radix_sort_pairs_u64(key2.p, vals2.p, nnz, cbits, s);
        k_count_keys<<<nblk(nnz, 256), 256, 0, s>>>(key2.p, nnz, ccnt.p);
        AXGB_CUDA(cudaGetLastError());
        // vals: each CSR entry's position in the compacted candidate list,
        // which the fast paths fill row by row in the reference's loop order
        if (o.keep_gen) out.gen_rank = std::move(vals);
    }
    scan_exclusive_i32(rcnt.p, out.row_ptr.p, n_dst, s);
    scan_exclusive_i32(ccnt.p, col_ptr.p, n_src, s);
    AXGB_CUDA(cudaMemcpyAsync(out.area_a.p, o.area_a_out ? o.area_a_out : area_src, sizeof(double) * n_src,
                              cudaMemcpyDeviceToDevice, s));
    AXGB_CUDA(cudaMemcpyAsync(out.area_b.p, o.area_b_out ? o.area_b_out : area_dst, sizeof(double) * n_dst,
                              cudaMemcpyDeviceToDevice, s));
    if (n_dst > 0)
        k_rows<<<nblk(n_dst, 256), 256, 0, s>>>(out.row_ptr.p, ovs.p, area_dst, o.fb_pre, n_dst,
                                               cfg.norm_type == AXGB_FRACAREA ? 1 : 0, out.val.p, out.frac_b.p);
    if (n_src > 0)
        k_cols<<<nblk(n_src, 256), 256, 0, s>>>(col_ptr.p, vals2.p, ovs.p, o.fac ? facs.p : nullptr, area_src, n_src,
                                               out.frac_a.p);
    AXGB_CUDA(cudaGetLastError());
    if (o.check_unmapped && cfg.unmapped == AXGB_UNMAPPED_ERROR && n_dst > 0) {
        DBuf<int> bad(1);
        bad.zero(s);
        k_unmapped<<<nblk(n_dst, 256), 256, 0, s>>>(D, out.row_ptr.p, bad.p);
        int h_bad = 0;
        AXGB_CUDA(cudaMemcpy(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (h_bad > 0)
            throw Error(AXGB_ERR_UNMAPPED,
                        "generate_conservative: " + std::to_string(h_bad) + " unmapped destination cell(s)");
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.nnz = nnz;
    out.stats[3] = nnz;
}

void generate_conservative(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    cudaStream_t s = 0;
    auto t_all = Clock::now();
    auto t0 = Clock::now();
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    out.times_ms[0] = ms_since(t0);
    MeshView S = src.view(), D = dst.view();
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    AXGB_REQUIRE(n_src < (i64(1) << 31) - 1 && n_dst < (i64(1) << 31) - 1, "meshes above 2^31 cells");
    out.n_src = n_src;
    out.n_dst = n_dst;

    // 2. LBVH
    t0 = Clock::now();
    const int n = static_cast<int>(n_src);
    DBuf<float4> nlo(n > 0 ? 2 * n - 1 : 1), nhi(n > 0 ? 2 * n - 1 : 1);
    DBuf<int> parent(n > 0 ? 2 * n - 1 : 1), right(n > 1 ? n - 1 : 1), flag(n > 1 ? n - 1 : 1);
    int root = -1;
    if (n > 0) {
        DBuf<unsigned> keys(n);
        DBuf<int> vals(n);
        k_leaf_keys<<<nblk(n, 256), 256, 0, s>>>(S, keys.p, vals.p);
        AXGB_CUDA(cudaGetLastError());
        radix_sort_pairs_u32(keys.p, vals.p, n, 30, s);
        Bvh t{n, n > 1 ? 0 : 0, nlo.p, nhi.p, parent.p, right.p, flag.p, keys.p};
        root = 0;  // internal node 0, or the single leaf (index n-1 = 0)
        AXGB_CUDA(cudaMemsetAsync(parent.p, 0xff, sizeof(int) * (2 * n - 1), s));
        flag.zero(s);
        k_leaves<<<nblk(n, 256), 256, 0, s>>>(t, S, vals.p);
        if (n > 1) {
            k_internal<<<nblk(n - 1, 256), 256, 0, s>>>(t);
            k_refit<<<nblk(n, 256), 256, 0, s>>>(t);
        }
        k_ropes<<<nblk(2 * n - 1, 256), 256, 0, s>>>(t);
        AXGB_CUDA(cudaGetLastError());
        AXGB_CUDA(cudaStreamSynchronize(s));
    }
    out.stats[4] = n > 0 ? 2 * n - 1 : 0;
    out.times_ms[1] = ms_since(t0);

    // 3. candidates
    t0 = Clock::now();
    DBuf<int> counts(n_dst);
    DBuf<i64> offs(n_dst + 1);
    DBuf<unsigned long long> raw(1);
    raw.zero(s);
    const int n_leaf_base = n > 0 ? n - 1 : 0;
    DBuf<int> err(1);
    err.zero(s);
    k_search<false><<<nblk(n_dst, 128), 128, 0, s>>>(S, D, nlo.p, nhi.p, root, n_leaf_base, counts.p, nullptr,
                                                    nullptr, raw.p, err.p);
    AXGB_CUDA(cudaGetLastError());
    scan_exclusive_i32_to_i64(counts.p, offs.p, n_dst, s);
    i64 n_cand = 0;
    unsigned long long n_raw = 0;
    AXGB_CUDA(cudaMemcpy(&n_cand, offs.p + n_dst, sizeof(i64), cudaMemcpyDeviceToHost));
    AXGB_CUDA(cudaMemcpy(&n_raw, raw.p, sizeof(n_raw), cudaMemcpyDeviceToHost));
    AXGB_REQUIRE(n_cand < (i64(1) << 31), "more than 2^31 candidate pairs");
    DBuf<int> cs(n_cand), cd(n_cand);
    if (n_cand > 0) {
        k_search<true><<<nblk(n_dst, 128), 128, 0, s>>>(S, D, nlo.p, nhi.p, root, n_leaf_base, nullptr, offs.p, cs.p,
                                                       nullptr, err.p);
        k_fill_rows<<<nblk(n_dst, 256), 256, 0, s>>>(offs.p, n_dst, cd.p);
        AXGB_CUDA(cudaGetLastError());
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
    int h_err = 0;
    AXGB_CUDA(cudaMemcpy(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_err) throw Error(AXGB_ERROR, "LBVH traversal exceeded its step bound (malformed tree)");
    out.stats[0] = static_cast<i64>(n_raw);
    out.stats[1] = n_cand;
    out.times_ms[2] = ms_since(t0);

    // 4. clip
    t0 = Clock::now();
    DBuf<double> ov(n_cand);
    DBuf<int> over_list(n_cand), n_over(1);
    n_over.zero(s);
    int h_over = 0;
    if (n_cand > 0) {
        k_clip<16><<<nblk(n_cand, 128), 128, 0, s>>>(S, D, cs.p, cd.p, n_cand, nullptr, ov.p, over_list.p, n_over.p);
        AXGB_CUDA(cudaGetLastError());
        AXGB_CUDA(cudaMemcpy(&h_over, n_over.p, sizeof(int), cudaMemcpyDeviceToHost));
        if (h_over > 0) {
            k_clip<32><<<nblk(h_over, 64), 64, 0, s>>>(S, D, cs.p, cd.p, h_over, over_list.p, ov.p, nullptr, nullptr);
            AXGB_CUDA(cudaGetLastError());
        }
    }
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.stats[2] = h_over;
    out.times_ms[3] = ms_since(t0);

    // 5. assembly
    t0 = Clock::now();
    assemble(cs, cd, ov, n_cand, S.area, D.area, D, cfg, out, s);
    out.times_ms[4] = ms_since(t0);
    out.times_ms[5] = ms_since(t_all);
    slice_centroids(D, out, s);  // locality hint for the blocked apply layout (not timed)
}

bool generate_conservative_regular(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    const GridInfo &sg = src.grid, &dg = dst.grid;
    // decline non-global grids whose longitude ranges do not fit (:127-147)
    const bool src_global = static_cast<double>(sg.ni) * sg.dlon > 350.0;
    const bool dst_global = static_cast<double>(dg.ni) * dg.dlon > 350.0;
    if (!src_global && !dst_global &&
        (dg.lon_min < sg.lon_min - sg.dlon * 0.5 || dg.lon_max > sg.lon_max + sg.dlon * 0.5))
        return false;
    cudaStream_t s = 0;
    auto t_all = Clock::now();
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    MeshView D = dst.view();
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    AXGB_REQUIRE(n_src < (i64(1) << 31) - 1 && n_dst < (i64(1) << 31) - 1, "meshes above 2^31 cells");
    out.n_src = n_src;
    out.n_dst = n_dst;
    RectArgs a;
    a.sg = {sg.ni, sg.nj, sg.lon_min, sg.dlon, sg.lat_min, sg.dlat};
    a.dg = {dg.ni, dg.nj, dg.lon_min, dg.dlon, dg.lat_min, dg.dlat};
    a.src_global = src_global;
    a.n_src = n_src;
    a.n_dst = n_dst;
    a.smask = src.has_mask ? src.d_mask.p : nullptr;
    a.dmask = dst.has_mask ? dst.d_mask.p : nullptr;
    DBuf<double> sa(n_src), da(n_dst);
    if (n_src) k_band_area<<<nblk(n_src, 256), 256, 0, s>>>(a.sg, src.has_area ? src.d_user_area.p : nullptr, n_src, sa.p);
    if (n_dst) k_band_area<<<nblk(n_dst, 256), 256, 0, s>>>(a.dg, dst.has_area ? dst.d_user_area.p : nullptr, n_dst, da.p);
    a.sa = sa.p;
    a.da = da.p;
    DBuf<int> counts(n_dst);
    DBuf<i64> offs(n_dst + 1);
    if (n_dst) k_rect<false><<<nblk(n_dst, 128), 128, 0, s>>>(a, counts.p, nullptr, nullptr, nullptr, nullptr, nullptr);
    AXGB_CUDA(cudaGetLastError());
    scan_exclusive_i32_to_i64(counts.p, offs.p, n_dst, s);
    i64 n_cand = 0;
    AXGB_CUDA(cudaMemcpy(&n_cand, offs.p + n_dst, sizeof(i64), cudaMemcpyDeviceToHost));
    AXGB_REQUIRE(n_cand < (i64(1) << 31), "more than 2^31 overlapping pairs");
    if (cfg.unmapped == AXGB_UNMAPPED_ERROR && n_cand == 0) return false;  // the general path diagnoses it
    DBuf<int> cs(n_cand), cd(n_cand);
    DBuf<double> ov(n_cand), fb(n_dst);
    fb.zero(s);
    if (n_cand) k_rect<true><<<nblk(n_dst, 128), 128, 0, s>>>(a, nullptr, offs.p, cs.p, cd.p, ov.p, fb.p);
    AXGB_CUDA(cudaGetLastError());
    out.stats[0] = out.stats[1] = n_cand;
    auto t0 = Clock::now();
    AssembleOpts o;
    o.keep_gen = true;  // rows generated in the reference's (js, is) loop order
    o.fb_pre = fb.p;
    o.check_unmapped = false;  // the fast path returns its matrix as it is (:380-415)
    assemble(cs, cd, ov, n_cand, sa.p, da.p, D, cfg, out, s, o);
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.times_ms[4] = ms_since(t0);
    out.times_ms[5] = ms_since(t_all);
    slice_centroids(D, out, s);
    return true;
}

bool generate_conservative_rectilinear(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    const GridInfo &sg = src.grid, &dg = dst.grid;
    cudaStream_t s = 0;
    auto t_all = Clock::now();
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    MeshView D = dst.view();
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    AXGB_REQUIRE(n_src < (i64(1) << 31) - 1 && n_dst < (i64(1) << 31) - 1, "meshes above 2^31 cells");
    out.n_src = n_src;
    out.n_dst = n_dst;
    DBuf<double> sl, st, dl, dt;
    sl.upload(sg.ulon.data(), sg.ulon.size(), s);
    st.upload(sg.ulat.data(), sg.ulat.size(), s);
    dl.upload(dg.ulon.data(), dg.ulon.size(), s);
    dt.upload(dg.ulat.data(), dg.ulat.size(), s);
    RectNuArgs a;
    a.sg = {static_cast<int>(sg.ni), static_cast<int>(sg.nj), sl.p, st.p};
    a.dg = {static_cast<int>(dg.ni), static_cast<int>(dg.nj), dl.p, dt.p};
    a.s_lon_min = sg.ulon.front();
    a.s_lon_max = sg.ulon.back();
    a.src_global = (a.s_lon_max - a.s_lon_min) > 350.0;  // degrees (:81-83)
    a.s_user = src.has_area ? src.d_user_area.p : nullptr;
    a.d_user = dst.has_area ? dst.d_user_area.p : nullptr;
    a.smask = src.has_mask ? src.d_mask.p : nullptr;
    a.dmask = dst.has_mask ? dst.d_mask.p : nullptr;
    a.n_src = n_src;
    a.n_dst = n_dst;
    DBuf<int> counts(n_dst);
    DBuf<i64> offs(n_dst + 1);
    if (n_dst)
        k_rect_nu<false><<<nblk(n_dst, 128), 128, 0, s>>>(a, counts.p, nullptr, nullptr, nullptr, nullptr, nullptr,
                                                          nullptr, nullptr);
    AXGB_CUDA(cudaGetLastError());
    scan_exclusive_i32_to_i64(counts.p, offs.p, n_dst, s);
    i64 n_cand = 0;
    AXGB_CUDA(cudaMemcpy(&n_cand, offs.p + n_dst, sizeof(i64), cudaMemcpyDeviceToHost));
    AXGB_REQUIRE(n_cand < (i64(1) << 31), "more than 2^31 overlapping pairs");
    // under UnmappedAction::Error an empty matrix goes on to the general path (weight_generator.cpp:3286-3295)
    if (n_dst == 0 || (cfg.unmapped == AXGB_UNMAPPED_ERROR && n_cand == 0)) return false;
    DBuf<int> cs(n_cand), cd(n_cand);
    DBuf<double> ov(n_cand), fac(n_cand), fb(n_dst), da_w(n_dst), sa(n_src), da(n_dst);
    k_rect_nu<true><<<nblk(n_dst, 128), 128, 0, s>>>(a, nullptr, offs.p, cs.p, cd.p, ov.p, fac.p, fb.p, da_w.p);
    if (n_src) k_edge_area<<<nblk(n_src, 256), 256, 0, s>>>(a.sg, a.s_user, n_src, sa.p);
    k_edge_area<<<nblk(n_dst, 256), 256, 0, s>>>(a.dg, a.d_user, n_dst, da.p);
    AXGB_CUDA(cudaGetLastError());
    out.stats[0] = out.stats[1] = n_cand;
    auto t0 = Clock::now();
    AssembleOpts o;
    o.keep_gen = true;  // rows generated in the reference's (js, is) loop order
    o.fac = fac.p;
    o.fb_pre = fb.p;
    o.area_b_out = da.p;
    o.check_unmapped = false;
    assemble(cs, cd, ov, n_cand, sa.p, da_w.p, D, cfg, out, s, o);
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.times_ms[4] = ms_since(t0);
    out.times_ms[5] = ms_since(t_all);
    slice_centroids(D, out, s);
    return true;
}

bool generate_bilinear_regular(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    const GridInfo &g = src.grid;
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    if (n_dst == 0 || g.ni == 0 || g.nj == 0) return false;  // the reference's fall-through signal
    cudaStream_t s = 0;
    auto t_all = Clock::now();
    mesh_prepare(dst, s);
    AXGB_REQUIRE(4 * n_dst < (i64(1) << 31) && n_src < (i64(1) << 31), "bilinear: meshes too large");
    BilRegArgs a{g.lon_min, g.lat_min, g.dlon, g.dlat, static_cast<int>(g.ni), static_cast<int>(g.nj),
                 std::abs((g.lon_max - g.lon_min) - 360.0) < 1.0e-10 * g.dlon};
    DBuf<int> cnt(n_dst), col4(4 * n_dst), gen4(4 * n_dst), bad(1);
    DBuf<double> w4(4 * n_dst);
    bad.zero(s);
    k_bilinear_reg<<<nblk(n_dst, 128), 128, 0, s>>>(dst.view(), a, cnt.p, col4.p, w4.p, gen4.p, bad.p);
    AXGB_CUDA(cudaGetLastError());
    int h_bad = 0;
    AXGB_CUDA(cudaMemcpy(&h_bad, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    if (h_bad > 0 && cfg.unmapped == AXGB_UNMAPPED_ERROR)
        throw Error(AXGB_ERR_UNMAPPED, "bilinear: " + std::to_string(h_bad) +
                                           " unmapped destination cell(s) in the regular-grid fast path");
    out.n_src = n_src;
    out.n_dst = n_dst;
    out.row_ptr.alloc(n_dst + 1);
    scan_exclusive_i32(cnt.p, out.row_ptr.p, n_dst, s);
    int nnz = 0;
    AXGB_CUDA(cudaMemcpy(&nnz, out.row_ptr.p + n_dst, sizeof(int), cudaMemcpyDeviceToHost));
    out.nnz = nnz;
    out.col.alloc(std::max(1, nnz));
    out.val.alloc(std::max(1, nnz));
    out.gen_rank.alloc(std::max(1, nnz));
    out.frac_a.alloc(n_src);
    out.frac_b.alloc(n_dst);
    out.area_a.alloc(n_src);
    out.area_b.alloc(n_dst);
    k_bilinear_reg_pack<<<nblk(n_dst, 256), 256, 0, s>>>(out.row_ptr.p, cnt.p, col4.p, w4.p, gen4.p, n_dst,
                                                         out.col.p, out.val.p, out.gen_rank.p, out.frac_b.p);
    if (n_src) k_fill<<<nblk(n_src, 256), 256, 0, s>>>(out.frac_a.p, n_src, 1.0);
    out.area_a.zero(s);
    out.area_b.zero(s);
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.stats[3] = nnz;
    out.times_ms[5] = ms_since(t_all);
    slice_centroids(dst.view(), out, s);
    return true;
}

void generate_bilinear(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    (void)cfg;
    cudaStream_t s = 0;
    auto t_all = Clock::now();
    const GridInfo &g = src.grid;
    const i64 ni = g.ni, nj = g.nj, n_dst = dst.n_cells, n_src = src.n_cells;
    AXGB_REQUIRE(ni >= 2 && nj >= 2, "bilinear: rectilinear source needs at least 2x2 cells");
    std::vector<double> cl(ni), ct(nj);
    for (i64 i = 0; i < ni; ++i) cl[i] = 0.5 * (g.ulon[i] + g.ulon[i + 1]);
    for (i64 j = 0; j < nj; ++j) ct[j] = 0.5 * (g.ulat[j] + g.ulat[j + 1]);
    DBuf<double> dcl, dct;
    dcl.upload(cl.data(), cl.size(), s);
    dct.upload(ct.data(), ct.size(), s);
    AXGB_REQUIRE(4 * n_dst < (i64(1) << 31), "bilinear: too many destination cells");
    out.n_src = n_src;
    out.n_dst = n_dst;
    out.nnz = 4 * n_dst;
    out.row_ptr.alloc(n_dst + 1);
    out.col.alloc(4 * n_dst);
    out.val.alloc(4 * n_dst);
    out.frac_a.alloc(n_src);
    out.frac_b.alloc(n_dst);
    out.area_a.alloc(n_src);
    out.area_b.alloc(n_dst);
    k_bilinear<<<nblk(n_dst + 1, 128), 128, 0, s>>>(dst.view(), dcl.p, static_cast<int>(ni), dct.p,
                                                   static_cast<int>(nj), out.row_ptr.p, out.col.p, out.val.p);
    k_fill<<<nblk(n_src, 256), 256, 0, s>>>(out.frac_a.p, n_src, 1.0);
    k_fill<<<nblk(n_dst, 256), 256, 0, s>>>(out.frac_b.p, n_dst, 1.0);
    out.area_a.zero(s);
    out.area_b.zero(s);
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.stats[3] = out.nnz;
    out.times_ms[5] = ms_since(t_all);
    mesh_prepare(dst, s);
    slice_centroids(dst.view(), out, s);
}

}  // namespace axgb
