// Per-cell geometry on the device: spherical area, bounding cap, the
// reference's dilated float AABB and the degenerate class, for every cell of
// a mesh, in one kernel (one thread per cell). Compiled with --fmad=false.
#include "geom.cuh"
#include "internal.hpp"

namespace axgb {

MeshView Mesh::view() const {
    MeshView v;
    v.n_nodes = n_nodes;
    v.n_cells = n_cells;
    v.off = d_off.p;
    v.idx = d_idx.p;
    v.xyz = d_xyz.p;
    v.lonlat = d_lonlat.p;
    v.regular = grid.regular ? 1 : 0;
    v.ni = static_cast<int>(grid.ni);
    v.nj = static_cast<int>(grid.nj);
    v.trig = d_trig.p;
    v.user_area = has_area ? d_user_area.p : nullptr;
    v.mask = has_mask ? d_mask.p : nullptr;
    v.area = d_area.p;
    v.cap = d_cap.p;
    v.capf = d_capf.p;
    v.box = d_box.p;
    v.flags = d_flags.p;
    return v;
}

namespace {

constexpr double kPi = 3.14159265358979323846;

__global__ void k_cell_prep(MeshView m) {
    const i64 c = static_cast<i64>(blockIdx.x) * blockDim.x + threadIdx.x;
    if (c >= m.n_cells) return;
    const int b = m.off[c], e = m.off[c + 1];
    const int nv = e - b;
    // Polygon of the first 32 vertices (SphericalPolygon<32> semantics):
    // cell area (weight_generator.cpp:523-552) and degenerate scan
    // (degenerate_cell_handler.hpp:190-223).
    DPoly<32> p;
    p.clear();
    for (int k = b; k < e && k < b + 32; ++k) {
        const double *q = m.xyz + 3 * static_cast<i64>(m.idx[k]);
        p.push({q[0], q[1], q[2]});
    }
    double poly_area = d_poly_area(p);
    double area = m.user_area ? m.user_area[c] : poly_area;
    int cls = d_classify(p, poly_area);
    // Bounding cap over all vertices (spherical_cap_filter.hpp:85-173).
    DCap cap{0.0, 0.0, 0.0, 0.0};
    if (nv >= 1) {
        double sx = 0.0, sy = 0.0, sz = 0.0;
        for (int k = b; k < e; ++k) {
            const double *q = m.xyz + 3 * static_cast<i64>(m.idx[k]);
            sx += q[0];
            sy += q[1];
            sz += q[2];
        }
        double inv = 1.0 / static_cast<double>(nv);
        DV3 cen = d_normalize({sx * inv, sy * inv, sz * inv});
        double mx = 0.0;
        for (int k = b; k < e; ++k) {
            const double *q = m.xyz + 3 * static_cast<i64>(m.idx[k]);
            double d = d_dot(cen, {q[0], q[1], q[2]});
            d = fmin(1.0, fmax(-1.0, d));
            double a = acos(d);
            if (a > mx) mx = a;
        }
        cap = DCap{cen.x, cen.y, cen.z, mx};
    }
    // Dilated float AABB (weight_generator.cpp:198-262); its trig uses
    // lon*pi/180.0, not the deg2rad constant.
    double mn[3] = {1.7976931348623157e308, 1.7976931348623157e308, 1.7976931348623157e308};
    double mxv[3] = {-1.7976931348623157e308, -1.7976931348623157e308, -1.7976931348623157e308};
    for (int k = b; k < e; ++k) {
        i64 n = m.idx[k];
        double lon = m.lonlat[n] * kPi / 180.0;
        double lat = m.lonlat[n + m.n_nodes] * kPi / 180.0;
        double cl = cos(lat);
        double q[3] = {cl * cos(lon), cl * sin(lon), sin(lat)};
        for (int d = 0; d < 3; ++d) {
            mn[d] = fmin(mn[d], q[d]);
            mxv[d] = fmax(mxv[d], q[d]);
        }
    }
    double ext = fmax(fmax(mxv[0] - mn[0], mxv[1] - mn[1]), mxv[2] - mn[2]);
    double eps = fmin(fmax(0.25 * ext, 1.0e-6), 0.02);
    float *bx = m.box + 6 * c;
    for (int d = 0; d < 3; ++d) {
        bx[d] = __double2float_rn(mn[d] - eps);
        bx[3 + d] = __double2float_rn(mxv[d] + eps);
    }
    unsigned char f = 0;
    if (cls != 0) f |= 1;
    if (m.mask && m.mask[c] == 0) f |= 2;
    if (area <= 0.0) f |= 4;
    f |= static_cast<unsigned char>(cls << 4);
    m.area[c] = area;
    m.cap[c] = cap;
    m.capf[c] = make_float4(__double2float_rn(cap.x), __double2float_rn(cap.y), __double2float_rn(cap.z),
                            __double2float_rn(cap.r));
    m.flags[c] = f;
}

}  // namespace

void mesh_prepare(Mesh &m, cudaStream_t s) {
    std::lock_guard<std::mutex> lk(m.mu);
    if (m.prepped) return;
    m.d_area.alloc(m.n_cells);
    m.d_cap.alloc(m.n_cells);
    m.d_capf.alloc(m.n_cells);
    m.d_box.alloc(6 * m.n_cells);
    m.d_flags.alloc(m.n_cells);
    if (m.n_cells > 0) {
        int threads = 128;
        unsigned blocks = static_cast<unsigned>((m.n_cells + threads - 1) / threads);
        k_cell_prep<<<blocks, threads, 0, s>>>(m.view());
        AXGB_CUDA(cudaGetLastError());
        AXGB_CUDA(cudaStreamSynchronize(s));
    }
    m.prepped = true;
}

}  // namespace axgb
