// Coastal post-pass of weight generation: coastal_renormalize_and_extrapolate
// (libs/axis/src/solver/weight_generator.cpp:1736-1881), which generate()
// (:2014) applies to every method's weights when the source mesh carries a
// cell mask. Entries from wet sources (mask > 0) are kept, and a row whose wet
// weights sum to s in (0, 1) is divided by s. With ExtrapolationAction::
// NearestWet, a row left without wet entries gets one entry of weight 1 from
// the wet source whose centroid is nearest its own, by Euclidean distance in
// float (lon, lat) degrees (the 2-D point query of the reference; centroids
// as compute_cell_centroids_xy, :75-138). Ties go to the lower source index.
// The nearest wet source comes from an exact LBVH nearest query over the wet
// centroids (lbvh.cuh), in float degrees, as the reference's 2-D BVH query
// does; the Morton codes map (lon, lat) into the unit cube by lon/180 - 1,
// lat/180.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.hpp"
#include "lbvh.cuh"

namespace axgb {
namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// Cell centroid in degrees as compute_cell_centroids_xy: mean of the vertex
// unit vectors (not normalised), lat = asin(z), lon = atan2(y, x) in [0, 2pi).
__global__ void k_centroid_xy(const double *lonlat, i64 n_nodes, const int *off, const int *idx, i64 n_cells,
                              int spherical, float4 *pt) {
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
    pt[c] = make_float4(static_cast<float>(ox), static_cast<float>(oy), 0.0f, 0.0f);
}

// Per row: wet weight sum s, wet count; new entry count. The sum runs in
// the order the generator emitted the row's entries (weight_generator.cpp:
// 1769-1777): gen (one key per CSR entry, distinct within a row) orders
// them; without gen, or where gen already ascends, that is CSR order. Rows
// out of order are walked by repeated selection of the next key.
__global__ void k_wet_rows(const int *rp, const int *col, const double *val, const int *gen, const int *mask,
                           i64 n_dst, int extrap, int any_wet, double *wsum, int *cnt) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    const int b = rp[j], e = rp[j + 1];
    bool in_order = true;
    if (gen)
        for (int k = b + 1; k < e; ++k)
            if (gen[k] < gen[k - 1]) in_order = false;
    double s = 0.0;
    int n = 0;
    if (in_order) {
        for (int k = b; k < e; ++k)
            if (mask[col[k]] > 0) {
                s += val[k];
                ++n;
            }
    } else {
        long long prev = -1;  // keys are non-negative
        for (int t = b; t < e; ++t) {
            int at = -1;
            for (int k = b; k < e; ++k)
                if (gen[k] > prev && (at < 0 || gen[k] < gen[at])) at = k;
            prev = gen[at];
            if (mask[col[at]] > 0) {
                s += val[at];
                ++n;
            }
        }
    }
    wsum[j] = s;
    cnt[j] = n > 0 ? n : (extrap && any_wet ? 1 : 0);
}

__global__ void k_coastal_fill(const int *rp, const int *col, const double *val, const int *mask, i64 n_dst,
                               const double *wsum, const int *nrp, PtTreeView wet, const float4 *dpt, int *ncol,
                               double *nval, int *err) {
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
        ncol[at] = pt_nearest(wet, dpt[j], err);
        nval[at] = 1.0;
    }
}

}  // namespace

void coastal_postpass(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &m) {
    if (!src.has_mask) {
        m.gen_rank.release();
        return;
    }
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
    if (n_dst)
        k_wet_rows<<<nblk(n_dst, 256), 256, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, m.nnz > 0 ? m.gen_rank.p : nullptr,
                                                    src.d_mask.p, n_dst, extrap, any_wet, wsum.p, cnt.p);
    AXGB_CUDA(cudaGetLastError());
    scan_exclusive_i32(cnt.p, nrp.p, n_dst, s);
    int nnz = 0;
    AXGB_CUDA(cudaMemcpy(&nnz, nrp.p + n_dst, sizeof(int), cudaMemcpyDeviceToHost));
    // wet-centroid tree (only walked for rows left dry)
    const bool spherical = src.coord_sys != AXGB_CARTESIAN3D;
    DBuf<float4> spt(n_src), dpt(n_dst);
    DBuf<int> wet_ids(std::max<size_t>(1, wet.size())), err(1);
    err.zero(s);
    PtTree T;
    if (extrap && any_wet) {
        MeshView S = src.view(), D = dst.view();
        k_centroid_xy<<<nblk(n_src, 256), 256, 0, s>>>(S.lonlat, S.n_nodes, S.off, S.idx, n_src, spherical, spt.p);
        k_centroid_xy<<<nblk(n_dst, 256), 256, 0, s>>>(D.lonlat, D.n_nodes, D.off, D.idx, n_dst, spherical, dpt.p);
        AXGB_CUDA(cudaGetLastError());
        wet_ids.upload_vec(wet, s);
        build_pt_tree(T, spt.p, wet_ids.p, static_cast<int>(wet.size()), PtMap{1.0 / 180.0, -1.0, 0.0, 0.0}, s);
    }
    DBuf<int> ncol(std::max(1, nnz));
    DBuf<double> nval(std::max(1, nnz));
    if (n_dst) k_coastal_fill<<<nblk(n_dst, 128), 128, 0, s>>>(m.row_ptr.p, m.col.p, m.val.p, src.d_mask.p, n_dst,
                                                                wsum.p, nrp.p, T.view(spt.p), dpt.p, ncol.p, nval.p,
                                                                err.p);
    AXGB_CUDA(cudaGetLastError());
    int h_err = 0;
    AXGB_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaStreamSynchronize(s));
    if (h_err) throw Error(AXGB_ERROR, "coastal_postpass: LBVH walk exceeded its step bound (malformed tree)");
    m.row_ptr = std::move(nrp);
    m.col = std::move(ncol);
    m.val = std::move(nval);
    m.gen_rank.release();
    m.nnz = nnz;
    m.stats[3] = nnz;
}

}  // namespace axgb
