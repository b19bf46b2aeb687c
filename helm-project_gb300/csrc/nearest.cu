// Nearest-neighbour weights: WeightGenerator::generate_nearest
// (src/solver/weight_generator.cpp:2097-2118). Each destination cell takes
// weight 1 from one source cell.
//   * Two regular grids: generate_nearest_rect (:2025-2080). The
//     destination cell's lower-left corner (lon_min + i*dlon, lat_min +
//     j*dlat) is rounded to the nearest source index, wrapped in longitude
//     and clamped in latitude; frac and area arrays stay zero.
//   * Otherwise generate_nearest_impl<3> (:2132-2260): cell centroids as
//     compute_cell_centroids_xy (:75-138), turned into float unit vectors
//     (cos/sin of the degree values times pi/180, in double, then rounded),
//     and for each destination point the source point at the least float
//     squared Euclidean distance. The reference asks ArborX v2.1 for
//     nearest(point, 1), which this checkout does not vendor; here exact
//     ties go to the lower source index. frac arrays are 1 and the areas
//     are get_cell_areas (:297-312): the mesh's own areas where it has them,
//     else the planar shoelace area of the cell's (lon, lat) degree corners
//     (compute_single_cell_area, :266-293). Masks play no part (the coastal
//     post-pass handles a masked source afterwards).
// The search is exact and logarithmic, as the reference's BVH query: an
// LBVH over the source points (lbvh.cuh) and, per destination point, a
// stackless walk that skips every node whose box is farther than the best
// point so far, seeded with the points next to the query in Morton order.
// A box's float distance never exceeds that of a point inside it (the same
// clamped differences, summed in the same order, no contraction), so no
// nearer point is ever skipped.
#include <algorithm>
#include <cmath>
#include <vector>

#include "internal.hpp"
#include "lbvh.cuh"

namespace axgb {
namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

// Float unit vector of a cell's centroid (compute_cell_centroids_xy, then
// the point construction of generate_nearest_impl<3>).
__global__ void k_nn_points(MeshView m, float4 *pts) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const double pi = 3.14159265358979323846;
    const int b = m.off[c], e = m.off[c + 1], nv = e - b;
    double sx = 0.0, sy = 0.0, sz = 0.0;
    for (int k = b; k < e; ++k) {
        const double lon = m.lonlat[m.idx[k]] * pi / 180.0, lat = m.lonlat[m.idx[k] + m.n_nodes] * pi / 180.0;
        sx += cos(lat) * cos(lon);
        sy += cos(lat) * sin(lon);
        sz += sin(lat);
    }
    const double inv = nv > 0 ? 1.0 / static_cast<double>(nv) : 0.0;
    double lat_avg = asin(sz * inv), lon_avg = atan2(sy * inv, sx * inv);
    if (lon_avg < 0.0) lon_avg += 2.0 * pi;
    lon_avg = lon_avg * 180.0 / pi;
    lat_avg = lat_avg * 180.0 / pi;
    const double lon = lon_avg * pi / 180.0, lat = lat_avg * pi / 180.0;
    pts[c] = make_float4(static_cast<float>(cos(lat) * cos(lon)), static_cast<float>(cos(lat) * sin(lon)),
                         static_cast<float>(sin(lat)), 0.0f);
}

__global__ void k_nn_query(PtTreeView T, const float4 *__restrict__ dp, i64 n_dst, int *col, int *err) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < n_dst) col[j] = pt_nearest(T, dp[j], err);
}

struct RectNN {
    i64 s_ni, s_nj, d_ni;
    double s_lon, s_lat, s_dlon, s_dlat, d_lon, d_lat, d_dlon, d_dlat;
};

// generate_nearest_rect (:2050-2077).
__global__ void k_nn_rect(RectNN a, i64 n_dst, int *col) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    const i64 di = j % a.d_ni, dj = j / a.d_ni;
    const double lon = a.d_lon + static_cast<double>(di) * a.d_dlon;
    const double lat = a.d_lat + static_cast<double>(dj) * a.d_dlat;
    i64 si = static_cast<i64>(round((lon - a.s_lon) / a.s_dlon));
    si = si % a.s_ni;
    if (si < 0) si += a.s_ni;
    i64 sj = static_cast<i64>(round((lat - a.s_lat) / a.s_dlat));
    if (sj < 0) sj = 0;
    if (sj >= a.s_nj) sj = a.s_nj - 1;
    col[j] = static_cast<int>(sj * a.s_ni + si);
}

__global__ void k_nn_csr(const int *col_all, i64 n_dst, int *cnt) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j < n_dst) cnt[j] = col_all[j] >= 0 ? 1 : 0;
}

__global__ void k_nn_pack(const int *col_all, const int *row_ptr, i64 n_dst, int *col, double *val) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst || col_all[j] < 0) return;
    col[row_ptr[j]] = col_all[j];
    val[row_ptr[j]] = 1.0;
}

__global__ void k_nn_fill(double *a, i64 n, double v) {
    const i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

// get_cell_areas (:297-312) with compute_single_cell_area (:266-293): the
// shoelace sum of lon0*lat1 - lon1*lat0 over the cell's edges in degrees,
// halved in magnitude; 0 below three corners. Built without contraction.
__global__ void k_planar_area(MeshView m, double *out) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    if (m.user_area) {
        out[c] = m.user_area[c];
        return;
    }
    const int b = m.off[c], n = m.off[c + 1] - b;
    if (n < 3) {
        out[c] = 0.0;
        return;
    }
    double a = 0.0;
    for (int i = 0; i < n; ++i) {
        const int p = m.idx[b + i], q = m.idx[b + (i + 1) % n];
        const double x0 = m.lonlat[p], y0 = m.lonlat[p + m.n_nodes];
        const double x1 = m.lonlat[q], y1 = m.lonlat[q + m.n_nodes];
        a += x0 * y1 - x1 * y0;
    }
    out[c] = fabs(a) * 0.5;
}

}  // namespace

void planar_cell_areas(const MeshView &m, double *out, cudaStream_t s) {
    if (m.n_cells) k_planar_area<<<nblk(m.n_cells, 256), 256, 0, s>>>(m, out);
    AXGB_CUDA(cudaGetLastError());
}

void generate_nearest(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    cudaStream_t s = 0;
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    AXGB_REQUIRE(n_src < (i64(1) << 31) - 1 && n_dst < (i64(1) << 31) - 1, "meshes above 2^31 cells");
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    out.n_src = n_src;
    out.n_dst = n_dst;
    DBuf<int> col_all(n_dst);
    const bool rect = src.grid.regular && dst.grid.regular;
    if (rect) {
        const GridInfo &sg = src.grid, &dg = dst.grid;
        RectNN a{sg.ni, sg.nj, dg.ni, sg.lon_min, sg.lat_min, sg.dlon, sg.dlat, dg.lon_min, dg.lat_min, dg.dlon, dg.dlat};
        if (n_dst) k_nn_rect<<<nblk(n_dst, 256), 256, 0, s>>>(a, n_dst, col_all.p);
        AXGB_CUDA(cudaGetLastError());
    } else if (n_src == 0) {
        if (n_dst) AXGB_CUDA(cudaMemsetAsync(col_all.p, 0xff, sizeof(int) * n_dst, s));
        if (n_dst && cfg.unmapped == AXGB_UNMAPPED_ERROR)
            throw Error(AXGB_ERR_UNMAPPED, "generate_nearest: unmapped destination cell 0 (no source cells)");
    } else {
        DBuf<float4> sp(n_src), dp(n_dst);
        k_nn_points<<<nblk(n_src, 128), 128, 0, s>>>(src.view(), sp.p);
        if (n_dst) k_nn_points<<<nblk(n_dst, 128), 128, 0, s>>>(dst.view(), dp.p);
        AXGB_CUDA(cudaGetLastError());
        // LBVH over the source points (the construction of the candidate search)
        PtTree T;
        build_pt_tree(T, sp.p, nullptr, static_cast<int>(n_src), PtMap{1.0, 0.0, 0.0, 0.0}, s);
        DBuf<int> err(1);
        err.zero(s);
        if (n_dst) k_nn_query<<<nblk(n_dst, 128), 128, 0, s>>>(T.view(sp.p), dp.p, n_dst, col_all.p, err.p);
        AXGB_CUDA(cudaGetLastError());
        int h_err = 0;
        AXGB_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        AXGB_CUDA(cudaStreamSynchronize(s));
        if (h_err) throw Error(AXGB_ERROR, "generate_nearest: LBVH walk exceeded its step bound (malformed tree)");
        AXGB_CUDA(cudaGetLastError());
    }
    DBuf<int> cnt(n_dst);
    out.row_ptr.alloc(n_dst + 1);
    if (n_dst) k_nn_csr<<<nblk(n_dst, 256), 256, 0, s>>>(col_all.p, n_dst, cnt.p);
    scan_exclusive_i32(cnt.p, out.row_ptr.p, n_dst, s);
    int nnz = 0;
    AXGB_CUDA(cudaMemcpy(&nnz, out.row_ptr.p + n_dst, sizeof(int), cudaMemcpyDeviceToHost));
    out.nnz = nnz;
    out.col.alloc(std::max(1, nnz));
    out.val.alloc(std::max(1, nnz));
    if (n_dst) k_nn_pack<<<nblk(n_dst, 256), 256, 0, s>>>(col_all.p, out.row_ptr.p, n_dst, out.col.p, out.val.p);
    out.frac_a.alloc(n_src);
    out.frac_b.alloc(n_dst);
    out.area_a.alloc(n_src);
    out.area_b.alloc(n_dst);
    if (rect) {  // default-initialised views in generate_nearest_rect
        out.frac_a.zero(s);
        out.frac_b.zero(s);
        out.area_a.zero(s);
        out.area_b.zero(s);
    } else {
        if (n_src) k_nn_fill<<<nblk(n_src, 256), 256, 0, s>>>(out.frac_a.p, n_src, 1.0);
        if (n_dst) k_nn_fill<<<nblk(n_dst, 256), 256, 0, s>>>(out.frac_b.p, n_dst, 1.0);
        planar_cell_areas(src.view(), out.area_a.p, s);
        planar_cell_areas(dst.view(), out.area_b.p, s);
    }
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.stats[3] = nnz;
    slice_centroids(dst.view(), out, s);
}

}  // namespace axgb
