// Coastal post-pass of weight generation: coastal_renormalize_and_extrapolate
// (libs/axis/src/solver/weight_generator.cpp:1736-1881), which generate()
// (:2014) applies to every method's weights when the source mesh carries a
// cell mask. Entries from wet sources (mask > 0) are kept, and a row whose wet
// weights sum to s in (0, 1) is divided by s. With ExtrapolationAction::
// NearestWet, a row left without wet entries gets one entry of weight 1 from
// the wet source whose centroid is nearest its own, by Euclidean distance in
// float (lon, lat) degrees (the 2-D point query of the reference; centroids
// as compute_cell_centroids_xy, :75-138). Ties go to the lower source index.
// The nearest wet source is found through a uniform grid of the wet
// centroids with a ring search whose stop rule keeps the result exact.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.hpp"

namespace axgb {
namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// Cell centroid in degrees as compute_cell_centroids_xy: mean of the vertex
// unit vectors (not normalised), lat = asin(z), lon = atan2(y, x) in [0, 2pi).
__global__ void k_centroid_xy(const double *lonlat, i64 n_nodes, const int *off, const int *idx, i64 n_cells,
                              int spherical, float *cx, float *cy) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= n_cells) return;
    const int b = off[c], e = off[c + 1], nv = e - b;
    const double pi = 3.14159265358979323846;
    double ox, oy;
    if (spherical) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int k = b; k < e; ++k) {
            const double lon = lonlat[idx[k]] * pi / 180.0, lat = lonlat[idx[k] + n_nodes] * pi / 180.0;
            sx += cos(lat) * cos(lon);
            sy += cos(lat) * sin(lon);
            sz += sin(lat);
        }
        const double inv = nv > 0 ? 1.0 / static_cast<double>(nv) : 0.0;
        double lat_avg = asin(sz * inv), lon_avg = atan2(sy * inv, sx * inv);
        if (lon_avg < 0.0) lon_avg += 2.0 * pi;
        ox = lon_avg * 180.0 / pi;
        oy = lat_avg * 180.0 / pi;
    } else {
        double sx = 0.0, sy = 0.0;
        for (int k = b; k < e; ++k) {
            sx += lonlat[idx[k]];
            sy += lonlat[idx[k] + n_nodes];
        }
        const double inv = nv > 0 ? 1.0 / static_cast<double>(nv) : 0.0;
        ox = sx * inv;
        oy = sy * inv;
    }
    cx[c] = static_cast<float>(ox);
    cy[c] = static_cast<float>(oy);
}

// Per row: wet weight sum s (CSR order), wet count; new entry count.
__global__ void k_wet_rows(const int *rp, const int *col, const double *val, const int *mask, i64 n_dst, int extrap,
                           int any_wet, double *wsum, int *cnt) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    double s = 0.0;
    int n = 0;
    for (int k = rp[j]; k < rp[j + 1]; ++k)
        if (mask[col[k]] > 0) {
            s += val[k];
            ++n;
        }
    wsum[j] = s;
    cnt[j] = n > 0 ? n : (extrap && any_wet ? 1 : 0);
}

struct WetGrid {
    float x0, y0, bw, bh;
    int gx, gy;
    const int *start;  // [gx*gy + 1] offsets into pts
    const int *pts;    // wet source indices, bucket-major, ascending within a bucket
    const float *cx, *cy;
};

__device__ __forceinline__ int bucket_of(const WetGrid &g, float v, float v0, float w, int n) {
    int b = static_cast<int>(floorf((v - v0) / w));
    return b < 0 ? 0 : (b >= n ? n - 1 : b);
}

// Nearest wet source to (qx, qy): rings of buckets around the query's own;
// stop once the best distance is below the gap to the next ring.
__device__ int nearest_wet(const WetGrid &g, float qx, float qy) {
    const int bx = bucket_of(g, qx, g.x0, g.bw, g.gx), by = bucket_of(g, qy, g.y0, g.bh, g.gy);
    float best = INFINITY;
    int besti = -1;
    const int rmax = max(g.gx, g.gy);
    for (int r = 0; r <= rmax; ++r) {
        for (int yy = by - r; yy <= by + r; ++yy) {
            if (yy < 0 || yy >= g.gy) continue;
            const bool edge_row = (yy == by - r || yy == by + r);
            for (int xx = bx - r; xx <= bx + r; xx += (edge_row ? 1 : 2 * r)) {
                if (xx >= 0 && xx < g.gx) {
                    const int bk = yy * g.gx + xx;
                    for (int q = g.start[bk]; q < g.start[bk + 1]; ++q) {
                        const int i = g.pts[q];
                        const float dx = __fsub_rn(qx, g.cx[i]), dy = __fsub_rn(qy, g.cy[i]);
                        const float d = __fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy));
                        if (d < best || (d == best && i < besti)) {
                            best = d;
                            besti = i;
                        }
                    }
                }
                if (r == 0) break;
            }
        }
        // every point outside rings 0..r is at least r bucket widths away on one
        // axis; one ring of slack covers bucket assignment rounding
        const float gap = static_cast<float>(r - 1) * fminf(g.bw, g.bh);
        if (besti >= 0 && r >= 1 && best < gap * gap) break;
    }
    return besti;
}

__global__ void k_coastal_fill(const int *rp, const int *col, const double *val, const int *mask, i64 n_dst,
                               const double *wsum, const int *nrp, WetGrid g, const float *dcx, const float *dcy,
                               int *ncol, double *nval) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    int at = nrp[j];
    const int end = nrp[j + 1];
    if (at == end) return;
    const double s = wsum[j];
    bool any = false;
    for (int k = rp[j]; k < rp[j + 1]; ++k)
        if (mask[col[k]] > 0) {
            double w = val[k];
            if (s > 0.0 && s < 1.0) w /= s;
            ncol[at] = col[k];
            nval[at] = w;
            ++at;
            any = true;
        }
    if (!any) {  // dry row: nearest wet source, weight 1
        ncol[at] = nearest_wet(g, dcx[j], dcy[j]);
        nval[at] = 1.0;
    }
}

}  // namespace

void coastal_postpass(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &m) {
    if (!src.has_mask) return;
    cudaStream_t s = 0;
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    const i64 n_src = m.n_src, n_dst = m.n_dst;
    std::vector<int> hmask(n_src);
    src.d_mask.download(hmask.data(), n_src, s);
    AXGB_CUDA(cudaStreamSynchronize(s));
    std::vector<int> wet;
    for (i64 i = 0; i < n_src; ++i)
        if (hmask[i] != 0) wet.push_back(static_cast<int>(i));  // candidates of the nearest query (mask != 0)
    const int extrap = cfg.extrap_method == AXGB_EXTRAP_NEAREST_WET ? 1 : 0;
    const int any_wet = wet.empty() ? 0 : 1;
    DBuf<double> wsum(n_dst);
    DBuf<int> cnt(n_dst), nrp(n_dst + 1);
    if (n_dst) k_wet_rows<<<nblk(n_dst, 256), 256, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, src.d_mask.p, n_dst, extrap,
                                                            any_wet, wsum.p, cnt.p);
    AXGB_CUDA(cudaGetLastError());
    scan_exclusive_i32(cnt.p, nrp.p, n_dst, s);
    int nnz = 0;
    AXGB_CUDA(cudaMemcpy(&nnz, nrp.p + n_dst, sizeof(int), cudaMemcpyDeviceToHost));
    // wet-centroid grid (only needed when some row is dry; built anyway when extrapolating)
    const bool spherical = src.coord_sys != AXGB_CARTESIAN3D;
    DBuf<float> scx(n_src), scy(n_src), dcx(n_dst), dcy(n_dst);
    WetGrid g{};
    DBuf<int> gstart(1), gpts(std::max<size_t>(1, wet.size()));
    if (extrap && any_wet) {
        MeshView S = src.view(), D = dst.view();
        k_centroid_xy<<<nblk(n_src, 256), 256, 0, s>>>(S.lonlat, S.n_nodes, S.off, S.idx, n_src, spherical, scx.p, scy.p);
        k_centroid_xy<<<nblk(n_dst, 256), 256, 0, s>>>(D.lonlat, D.n_nodes, D.off, D.idx, n_dst, spherical, dcx.p, dcy.p);
        AXGB_CUDA(cudaGetLastError());
        std::vector<float> hx(n_src), hy(n_src);
        scx.download(hx.data(), n_src, s);
        scy.download(hy.data(), n_src, s);
        AXGB_CUDA(cudaStreamSynchronize(s));
        float x0 = INFINITY, x1 = -INFINITY, y0 = INFINITY, y1 = -INFINITY;
        for (int i : wet) {
            x0 = std::min(x0, hx[i]);
            x1 = std::max(x1, hx[i]);
            y0 = std::min(y0, hy[i]);
            y1 = std::max(y1, hy[i]);
        }
        const double nb = std::max(1.0, static_cast<double>(wet.size()) / 4.0);
        const double ex = std::max(1e-6, static_cast<double>(x1 - x0)), ey = std::max(1e-6, static_cast<double>(y1 - y0));
        int gx = std::max(1, static_cast<int>(std::sqrt(nb * ex / ey)));
        int gy = std::max(1, static_cast<int>(nb / gx));
        gx = std::min(gx, 4096);
        gy = std::min(gy, 4096);
        g.x0 = x0;
        g.y0 = y0;
        g.bw = static_cast<float>(ex / gx) * 1.0001f;
        g.bh = static_cast<float>(ey / gy) * 1.0001f;
        g.gx = gx;
        g.gy = gy;
        // bucket the wet sources (ascending index within a bucket)
        std::vector<int> bstart(static_cast<size_t>(gx) * gy + 1, 0), order(wet.size());
        auto bucket = [&](int i) {
            int bx = static_cast<int>(std::floor((hx[i] - g.x0) / g.bw)), by = static_cast<int>(std::floor((hy[i] - g.y0) / g.bh));
            bx = std::clamp(bx, 0, gx - 1);
            by = std::clamp(by, 0, gy - 1);
            return by * gx + bx;
        };
        for (int i : wet) bstart[bucket(i) + 1]++;
        for (size_t b = 0; b + 1 < bstart.size(); ++b) bstart[b + 1] += bstart[b];
        std::vector<int> fillp(bstart.begin(), bstart.end() - 1);
        for (int i : wet) order[fillp[bucket(i)]++] = i;
        gstart.upload_vec(bstart, s);
        gpts.upload_vec(order, s);
        g.start = gstart.p;
        g.pts = gpts.p;
        g.cx = scx.p;
        g.cy = scy.p;
    }
    DBuf<int> ncol(std::max(1, nnz));
    DBuf<double> nval(std::max(1, nnz));
    if (n_dst) k_coastal_fill<<<nblk(n_dst, 128), 128, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, src.d_mask.p, n_dst,
                                                                wsum.p, nrp.p, g, dcx.p, dcy.p, ncol.p, nval.p);
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
    m.row_ptr = std::move(nrp);
    m.col = std::move(ncol);
    m.val = std::move(nval);
    m.nnz = nnz;
    m.stats[3] = nnz;
}

}  // namespace axgb
