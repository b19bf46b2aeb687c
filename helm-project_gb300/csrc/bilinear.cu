// Bilinear weights from a source that is not rectilinear: the general path
// of WeightGenerator::generate_bilinear (src/solver/weight_generator.cpp:
// 2346-2667), one thread per destination cell.
//   * Candidates: the k = min(8, n_src) source cells whose centroids
//     (compute_cell_centroids_xy, :75-138, float lon/lat degrees) are
//     nearest the destination centroid in the plane. The reference asks
//     ArborX v2.1 (not vendored) for nearest(point, k); here they come from
//     the point LBVH (lbvh.cuh) in ascending (float distance, index) order.
//   * Phase A (:2423-2489): every 4-combination of the candidates in that
//     order, their double centroids projected gnomonically around the
//     destination centroid, is handed to the Newton map onto the reference
//     quad; the first that converges gives the four shape-function weights
//     of the clamped (xi, eta).
//   * Phase B (:2492-2557): else the first 3-combination whose barycentric
//     coordinates are all >= -1e-10 (clamped at 0, renormalised).
//   * Phase C (:2560-2615): else inverse chord distances to the first four
//     candidates (one weight 1 at a zero distance).
// The transcendental inputs come from the host's libm, as in the
// reference: the centroids, the gnomonic projection of every (destination,
// candidate) pair and the centroids' unit vectors. The Newton map is chaotic
// where it does not converge in its 20 iterations, so a last-bit difference
// in a sine would change those rows. The device then runs the phases on
// those values in the reference's operation order (--fmad=false), so every
// weight is bitwise the reference's arithmetic. Entries of a row are stored
// column-ascending (to_csr). frac = 1, area_a = 0, area_b the destination
// cells' get_cell_areas (mesh areas, else planar shoelace areas in degrees).
#include <algorithm>
#include <cmath>
#include <thread>
#include <vector>

#include "internal.hpp"
#include "lbvh.cuh"

namespace axgb {
namespace {

inline unsigned nblk(i64 n, int t) { return static_cast<unsigned>((n + t - 1) / t); }

constexpr double kPiB = 3.14159265358979323846;

__global__ void k_ll_points(const double2 *ll, i64 n, float4 *pts) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c < n) pts[c] = make_float4(static_cast<float>(ll[c].x), static_cast<float>(ll[c].y), 0.0f, 0.0f);
}

struct V2 {
    double x, y;
};

// map_to_reference_quad (:596-666): Newton iteration for (xi, eta).
__device__ bool ref_quad(double px, double py, const V2 &v0, const V2 &v1, const V2 &v2, const V2 &v3, double &xi_out,
                         double &eta_out) {
    double xi = 0.0, eta = 0.0;
    const double tol = 1e-12;
    for (int iter = 0; iter < 20; ++iter) {
        const double N0 = 0.25 * (1.0 - xi) * (1.0 - eta);
        const double N1 = 0.25 * (1.0 + xi) * (1.0 - eta);
        const double N2 = 0.25 * (1.0 + xi) * (1.0 + eta);
        const double N3 = 0.25 * (1.0 - xi) * (1.0 + eta);
        const double x_cur = N0 * v0.x + N1 * v1.x + N2 * v2.x + N3 * v3.x;
        const double y_cur = N0 * v0.y + N1 * v1.y + N2 * v2.y + N3 * v3.y;
        const double rx = px - x_cur;
        const double ry = py - y_cur;
        if (fabs(rx) < tol && fabs(ry) < tol) {
            xi_out = xi;
            eta_out = eta;
            return true;
        }
        const double dN0_dxi = -0.25 * (1.0 - eta);
        const double dN1_dxi = 0.25 * (1.0 - eta);
        const double dN2_dxi = 0.25 * (1.0 + eta);
        const double dN3_dxi = -0.25 * (1.0 + eta);
        const double dN0_deta = -0.25 * (1.0 - xi);
        const double dN1_deta = -0.25 * (1.0 + xi);
        const double dN2_deta = 0.25 * (1.0 + xi);
        const double dN3_deta = 0.25 * (1.0 - xi);
        const double dx_dxi = dN0_dxi * v0.x + dN1_dxi * v1.x + dN2_dxi * v2.x + dN3_dxi * v3.x;
        const double dy_dxi = dN0_dxi * v0.y + dN1_dxi * v1.y + dN2_dxi * v2.y + dN3_dxi * v3.y;
        const double dx_deta = dN0_deta * v0.x + dN1_deta * v1.x + dN2_deta * v2.x + dN3_deta * v3.x;
        const double dy_deta = dN0_deta * v0.y + dN1_deta * v1.y + dN2_deta * v2.y + dN3_deta * v3.y;
        const double det = dx_dxi * dy_deta - dx_deta * dy_dxi;
        if (fabs(det) < 1e-30) return false;
        const double inv_det = 1.0 / det;
        const double dxi = inv_det * (dy_deta * rx - dx_deta * ry);
        const double deta = inv_det * (-dy_dxi * rx + dx_dxi * ry);
        xi += dxi;
        eta += deta;
        xi = fmax(-2.0, fmin(2.0, xi));
        eta = fmax(-2.0, fmin(2.0, eta));
    }
    xi_out = xi;
    eta_out = eta;
    return (fabs(xi) <= 1.0 + 1e-6 && fabs(eta) <= 1.0 + 1e-6);
}

// barycentric_triangle (:670-684).
__device__ __forceinline__ bool bary(double px, double py, const V2 &v0, const V2 &v1, const V2 &v2, double &l0, double &l1,
                                     double &l2) {
    const double denom = (v1.y - v2.y) * (v0.x - v2.x) + (v2.x - v1.x) * (v0.y - v2.y);
    if (fabs(denom) < 1e-30) {
        l0 = l1 = l2 = 1.0 / 3.0;
        return false;
    }
    const double inv = 1.0 / denom;
    l0 = ((v1.y - v2.y) * (px - v2.x) + (v2.x - v1.x) * (py - v2.y)) * inv;
    l1 = ((v2.y - v0.y) * (px - v2.x) + (v0.x - v2.x) * (py - v2.y)) * inv;
    l2 = 1.0 - l0 - l1;
    const double eps = -1e-10;
    return (l0 >= eps && l1 >= eps && l2 >= eps);
}

constexpr int kCand = 8;

// The min(8, n) nearest source centroids of each destination centroid.
__global__ void k_bil_candidates(PtTreeView T, const float4 *__restrict__ dpt, i64 n_dst, int *cand, int *navail,
                                 int *err) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    int c[kCand];
    float d[kCand];
    const int n = pt_knearest<kCand>(T, dpt[j], c, d, err);
    navail[j] = n;
    for (int k = 0; k < kCand; ++k) cand[kCand * j + k] = k < n ? c[k] : -1;
}

// Phases A, B, C on the projected candidates q[8*j + a] (host libm) and the
// unit vectors of the centroids (host libm).
__global__ void k_bilinear_general(const int *__restrict__ cand, const int *__restrict__ navail,
                                   const double2 *__restrict__ proj, const double *__restrict__ sxyz,
                                   const double *__restrict__ dxyz, i64 n_dst, int *cnt, int *col4, double *w4,
                                   int *gen4) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    const int n_avail = navail[j];
    int nc = 0;
    int oc[4];
    double ow[4];
    int ork[4] = {0, 1, 2, 3};
    if (n_avail > 0) {
        const int *cj = cand + kCand * j;
        V2 q[kCand];
        for (int a = 0; a < n_avail; ++a) q[a] = {proj[kCand * j + a].x, proj[kCand * j + a].y};
        const double tpx = 0.0, tpy = 0.0;  // the projection's origin is the destination centroid
        bool done = false;
        // Phase A: containing quad
        if (n_avail >= 4)
            for (int a = 0; a < n_avail - 3 && !done; ++a)
                for (int b = a + 1; b < n_avail - 2 && !done; ++b)
                    for (int c = b + 1; c < n_avail - 1 && !done; ++c)
                        for (int d = c + 1; d < n_avail && !done; ++d) {
                            double xi = 0.0, eta = 0.0;
                            if (ref_quad(tpx, tpy, q[a], q[b], q[c], q[d], xi, eta)) {
                                xi = fmax(-1.0, fmin(1.0, xi));
                                eta = fmax(-1.0, fmin(1.0, eta));
                                oc[0] = cj[a];
                                oc[1] = cj[b];
                                oc[2] = cj[c];
                                oc[3] = cj[d];
                                ow[0] = 0.25 * (1.0 - xi) * (1.0 - eta);
                                ow[1] = 0.25 * (1.0 + xi) * (1.0 - eta);
                                ow[2] = 0.25 * (1.0 + xi) * (1.0 + eta);
                                ow[3] = 0.25 * (1.0 - xi) * (1.0 + eta);
                                nc = 4;
                                done = true;
                            }
                        }
        // Phase B: containing triangle
        if (n_avail >= 3 && !done)
            for (int a = 0; a < n_avail - 2 && !done; ++a)
                for (int b = a + 1; b < n_avail - 1 && !done; ++b)
                    for (int c = b + 1; c < n_avail && !done; ++c) {
                        double l0 = 0.0, l1 = 0.0, l2 = 0.0;
                        if (bary(tpx, tpy, q[a], q[b], q[c], l0, l1, l2)) {
                            l0 = fmax(0.0, l0);
                            l1 = fmax(0.0, l1);
                            l2 = fmax(0.0, l2);
                            const double sum = l0 + l1 + l2;
                            if (sum > 0.0) {
                                l0 /= sum;
                                l1 /= sum;
                                l2 /= sum;
                            } else {
                                l0 = l1 = l2 = 1.0 / 3.0;
                            }
                            oc[0] = cj[a];
                            oc[1] = cj[b];
                            oc[2] = cj[c];
                            ow[0] = l0;
                            ow[1] = l1;
                            ow[2] = l2;
                            nc = 3;
                            done = true;
                        }
                    }
        // Phase C: inverse chord distances to the first four candidates
        if (!done) {
            const int n_idw = min(4, n_avail);
            double dist[4];
            double sum_inv = 0.0;
            int zero = -1;
            for (int k = 0; k < n_idw; ++k) {
                const double *ps = sxyz + 3 * static_cast<i64>(cj[k]), *pd = dxyz + 3 * j;
                const double dx = pd[0] - ps[0];
                const double dy = pd[1] - ps[1];
                const double dz = pd[2] - ps[2];
                const double dd = sqrt(dx * dx + dy * dy + dz * dz);
                if (dd <= 0.0) {
                    zero = k;
                    break;
                }
                dist[k] = dd;
                sum_inv += 1.0 / dd;
            }
            if (zero >= 0) {
                oc[0] = cj[zero];
                ow[0] = 1.0;
                nc = 1;
            } else {
                for (int k = 0; k < n_idw; ++k) {
                    oc[k] = cj[k];
                    ow[k] = (1.0 / dist[k]) / sum_inv;
                }
                nc = n_idw;
            }
        }
        // column-ascending within the row (the columns are distinct); ork
        // keeps each entry's place in the stencil (generation) order
        for (int a = 1; a < nc; ++a)
            for (int b = a; b > 0 && oc[b - 1] > oc[b]; --b) {
                const int tc = oc[b];
                oc[b] = oc[b - 1];
                oc[b - 1] = tc;
                const double tw = ow[b];
                ow[b] = ow[b - 1];
                ow[b - 1] = tw;
                const int tr = ork[b];
                ork[b] = ork[b - 1];
                ork[b - 1] = tr;
            }
    }
    cnt[j] = nc;
    for (int k = 0; k < nc; ++k) {
        col4[4 * j + k] = oc[k];
        w4[4 * j + k] = ow[k];
        gen4[4 * j + k] = ork[k];
    }
}

__global__ void k_bil_pack(const int *row_ptr, const int *cnt, const int *col4, const double *w4, const int *gen4,
                           i64 n_dst, int *col, double *w, int *gen) {
    const i64 j = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (j >= n_dst) return;
    const int p = row_ptr[j];
    for (int k = 0; k < cnt[j]; ++k) {
        col[p + k] = col4[4 * j + k];
        w[p + k] = w4[4 * j + k];
        gen[p + k] = gen4[4 * j + k];
    }
}

__global__ void k_bil_fill(double *a, i64 n, double v) {
    const i64 i = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (i < n) a[i] = v;
}

template <class F>
void host_parallel(i64 n, F f) {
    const unsigned nt = std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    if (n < 4096 || nt == 1) {
        f(0, n);
        return;
    }
    std::vector<std::thread> th;
    const i64 chunk = (n + nt - 1) / nt;
    for (unsigned t = 0; t < nt; ++t) {
        const i64 b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) th.emplace_back([=] { f(b, e); });
    }
    for (auto &t : th) t.join();
}

// compute_cell_centroids_xy (:75-138), host libm, degrees.
void host_centroids(const Mesh &m, std::vector<double> &cx, std::vector<double> &cy) {
    cx.resize(m.n_cells);
    cy.resize(m.n_cells);
    const double *lon = m.lonlat.data(), *lat = m.lonlat.data() + m.n_nodes;
    host_parallel(m.n_cells, [&](i64 b0, i64 e0) {
        for (i64 c = b0; c < e0; ++c) {
            double sx = 0.0, sy = 0.0, sz = 0.0;
            const i64 b = m.off[c], e = m.off[c + 1];
            for (i64 k = b; k < e; ++k) {
                const double lo = lon[m.idx[k]] * kPiB / 180.0, la = lat[m.idx[k]] * kPiB / 180.0;
                sx += std::cos(la) * std::cos(lo);
                sy += std::cos(la) * std::sin(lo);
                sz += std::sin(la);
            }
            const double inv = (e - b > 0) ? 1.0 / static_cast<double>(e - b) : 0.0;
            double la = std::asin(sz * inv), lo = std::atan2(sy * inv, sx * inv);
            if (lo < 0.0) lo += 2.0 * kPiB;
            cx[c] = lo * 180.0 / kPiB;
            cy[c] = la * 180.0 / kPiB;
        }
    });
}

// Unit vectors of the centroids as the inverse-distance phase forms them.
std::vector<double> host_xyz(const std::vector<double> &cx, const std::vector<double> &cy) {
    std::vector<double> v(3 * cx.size());
    host_parallel(static_cast<i64>(cx.size()), [&](i64 b, i64 e) {
        for (i64 c = b; c < e; ++c) {
            const double lo = cx[c] * kPiB / 180.0, la = cy[c] * kPiB / 180.0;
            v[3 * c] = std::cos(la) * std::cos(lo);
            v[3 * c + 1] = std::cos(la) * std::sin(lo);
            v[3 * c + 2] = std::sin(la);
        }
    });
    return v;
}

}  // namespace

void generate_bilinear_general(Mesh &src, Mesh &dst, const axgb_regrid_config &cfg, Matrix &out) {
    cudaStream_t s = 0;
    const i64 n_src = src.n_cells, n_dst = dst.n_cells;
    AXGB_REQUIRE(static_cast<i64>(kCand) * n_dst < (i64(1) << 31) && n_src < (i64(1) << 31),
                 "bilinear: meshes too large");
    mesh_prepare(src, s);
    mesh_prepare(dst, s);
    if (n_src == 0 && n_dst > 0 && cfg.unmapped == AXGB_UNMAPPED_ERROR)
        throw Error(AXGB_ERR_UNMAPPED, "generate_bilinear: unmapped destination cell 0 (no source cells)");
    std::vector<double> scx, scy, dcx, dcy;
    host_centroids(src, scx, scy);
    host_centroids(dst, dcx, dcy);
    // candidates on the device: the point tree over the float centroids
    std::vector<double2> sll(n_src), dll(n_dst);
    for (i64 i = 0; i < n_src; ++i) sll[i] = make_double2(scx[i], scy[i]);
    for (i64 j = 0; j < n_dst; ++j) dll[j] = make_double2(dcx[j], dcy[j]);
    DBuf<double2> d_sll, d_dll;
    d_sll.upload(sll.data(), sll.size(), s);
    d_dll.upload(dll.data(), dll.size(), s);
    DBuf<float4> spt(n_src), dpt(n_dst);
    if (n_src) k_ll_points<<<nblk(n_src, 256), 256, 0, s>>>(d_sll.p, n_src, spt.p);
    if (n_dst) k_ll_points<<<nblk(n_dst, 256), 256, 0, s>>>(d_dll.p, n_dst, dpt.p);
    AXGB_CUDA(cudaGetLastError());
    PtTree T;
    build_pt_tree(T, spt.p, nullptr, static_cast<int>(n_src), PtMap{1.0 / 180.0, -1.0, 0.0, 0.0}, s);
    DBuf<int> cand(kCand * n_dst), navail(n_dst), err(1);
    err.zero(s);
    if (n_dst) k_bil_candidates<<<nblk(n_dst, 128), 128, 0, s>>>(T.view(spt.p), dpt.p, n_dst, cand.p, navail.p, err.p);
    AXGB_CUDA(cudaGetLastError());
    std::vector<int> hc(kCand * n_dst), hn(n_dst);
    int h_err = 0;
    cand.download(hc.data(), hc.size(), s);
    navail.download(hn.data(), hn.size(), s);
    AXGB_CUDA(cudaMemcpyAsync(&h_err, err.p, sizeof(int), cudaMemcpyDeviceToHost, s));
    AXGB_CUDA(cudaStreamSynchronize(s));
    if (h_err) throw Error(AXGB_ERROR, "generate_bilinear: LBVH walk exceeded its step bound (malformed tree)");
    // project_gnomonic (:584-590) of every (destination, candidate) pair, host libm
    std::vector<double2> proj(kCand * n_dst);
    host_parallel(n_dst, [&](i64 b, i64 e) {
        for (i64 j = b; j < e; ++j) {
            const double lon0 = dcx[j] * kPiB / 180.0, lat0 = dcy[j] * kPiB / 180.0;
            for (int a = 0; a < hn[j]; ++a) {
                const i64 c = hc[kCand * j + a];
                const double lon = scx[c] * kPiB / 180.0, lat = scy[c] * kPiB / 180.0;
                double cos_c = std::sin(lat0) * std::sin(lat) + std::cos(lat0) * std::cos(lat) * std::cos(lon - lon0);
                if (cos_c <= 0.0) cos_c = 1e-15;
                proj[kCand * j + a] =
                    make_double2((std::cos(lat) * std::sin(lon - lon0)) / cos_c,
                                 (std::sin(lat) * std::cos(lat0) - std::cos(lat) * std::sin(lat0) * std::cos(lon - lon0)) /
                                     cos_c);
            }
        }
    });
    const std::vector<double> sx = host_xyz(scx, scy), dx = host_xyz(dcx, dcy);
    DBuf<double2> d_proj;
    DBuf<double> d_sx, d_dx;
    d_proj.upload(proj.data(), proj.size(), s);
    d_sx.upload(sx.data(), sx.size(), s);
    d_dx.upload(dx.data(), dx.size(), s);
    DBuf<int> cnt(n_dst), col4(4 * n_dst), gen4(4 * n_dst);
    DBuf<double> w4(4 * n_dst);
    if (n_dst)
        k_bilinear_general<<<nblk(n_dst, 64), 64, 0, s>>>(cand.p, navail.p, d_proj.p, d_sx.p, d_dx.p, n_dst, cnt.p,
                                                          col4.p, w4.p, gen4.p);
    AXGB_CUDA(cudaGetLastError());
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
    if (n_dst)
        k_bil_pack<<<nblk(n_dst, 256), 256, 0, s>>>(out.row_ptr.p, cnt.p, col4.p, w4.p, gen4.p, n_dst, out.col.p,
                                                    out.val.p, out.gen_rank.p);
    out.frac_a.alloc(n_src);
    out.frac_b.alloc(n_dst);
    out.area_a.alloc(n_src);
    out.area_b.alloc(n_dst);
    if (n_src) k_bil_fill<<<nblk(n_src, 256), 256, 0, s>>>(out.frac_a.p, n_src, 1.0);
    if (n_dst) k_bil_fill<<<nblk(n_dst, 256), 256, 0, s>>>(out.frac_b.p, n_dst, 1.0);
    out.area_a.zero(s);  // the ESMF convention for bilinear (:2646-2650)
    planar_cell_areas(dst.view(), out.area_b.p, s);  // get_cell_areas(dst_mesh) (:2652-2655)
    AXGB_CUDA(cudaGetLastError());
    AXGB_CUDA(cudaStreamSynchronize(s));
    out.stats[3] = nnz;
    slice_centroids(dst.view(), out, s);
}

}  // namespace axgb
