// Driver that runs the reference's OWN regular and rectilinear fast paths
// (AXIS src/solver/weight_generator_conservative_rect.cpp,
// weight_generator_conservative_rect_nonuniform.cpp,
// weight_generator_bilinear_rect.cpp, weight_generator_bilinear_rect_nonuniform.cpp,
// compiled unchanged from the checkout through the host shim in ref_shim/)
// with the reference's grid detection and InterpolationMatrix::to_csr, so
// that the oracle's restatements of those paths are pinned bit for bit.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into
// oracle/_ref/libaxisref_fast.so when the reference checkout exists, and
// loaded only by tests/ and tests/golden/make_golden.py.

#include <Kokkos_Core.hpp>
#include <axis/detail/regular_grid_detector.hpp>
#include <axis/solver/interpolation_matrix.hpp>
#include <axis/solver/regrid_config.hpp>
#include <axis/topology/unstructured_mesh.hpp>
#include <cstdint>
#include <stdexcept>

using HS = Kokkos::HostSpace;
using Mesh = axis::topology::UnstructuredMesh<HS>;
using IM = axis::solver::InterpolationMatrix<HS>;
using i64 = std::int64_t;

namespace axis::solver {
template <class MemorySpace>
InterpolationMatrix<MemorySpace> generate_conservative_rect(const topology::UnstructuredMesh<MemorySpace> &,
                                                            const topology::UnstructuredMesh<MemorySpace> &,
                                                            const RegridConfig &, const detail::RegularGridInfo &,
                                                            const detail::RegularGridInfo &);
template <class MemorySpace>
InterpolationMatrix<MemorySpace> generate_conservative_rect_nonuniform(const topology::UnstructuredMesh<MemorySpace> &,
                                                                       const topology::UnstructuredMesh<MemorySpace> &,
                                                                       const RegridConfig &,
                                                                       const detail::RectilinearGridInfo &,
                                                                       const detail::RectilinearGridInfo &);
template <class MemorySpace>
InterpolationMatrix<MemorySpace> generate_bilinear_rect(const topology::UnstructuredMesh<MemorySpace> &,
                                                        const topology::UnstructuredMesh<MemorySpace> &,
                                                        const RegridConfig &, const detail::RegularGridInfo &,
                                                        const detail::RegularGridInfo &);
template <class MemorySpace>
InterpolationMatrix<MemorySpace> generate_bilinear_rect_nonuniform(const topology::UnstructuredMesh<MemorySpace> &,
                                                                   const topology::UnstructuredMesh<MemorySpace> &,
                                                                   const RegridConfig &,
                                                                   const detail::RectilinearGridInfo &);
}  // namespace axis::solver

namespace {

Mesh make_mesh(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx) {
    Kokkos::View<double **, Kokkos::LayoutLeft, HS> nc("nc", n_nodes, 2);
    for (i64 i = 0; i < 2 * n_nodes; ++i) nc.data()[i] = lonlat[i];
    Kokkos::View<axis::index_t *, HS> o("o", n_cells + 1), x("x", off[n_cells]);
    for (i64 i = 0; i <= n_cells; ++i) o(i) = off[i];
    for (i64 i = 0; i < off[n_cells]; ++i) x(i) = idx[i];
    return Mesh(nc, o, x, axis::topology::CoordinateSystem::SphericalDeg);
}

}  // namespace

extern "C" {

// kind: 0 generate_conservative_rect, 1 generate_conservative_rect_nonuniform,
// 2 generate_bilinear_rect, 3 generate_bilinear_rect_nonuniform. norm_type:
// 0 DstArea, 1 FracArea; unmapped: 0 Error, 1 Ignore. Writes the to_csr rows
// (one per entry), columns and values and the frac/area arrays when nnz fits
// cap; returns 0, -1 when the path returned the decline signal (n_dst == 0),
// -2 when a grid is not regular/rectilinear as the path needs, -3 when the
// path threw.
int ref_fast(int kind, i64 sn, const double *sll, i64 sc, const i64 *soff, const i64 *sidx, i64 dn, const double *dll,
             i64 dc, const i64 *doff, const i64 *didx, int norm_type, int unmapped, i64 cap, i64 *nnz, i64 *row,
             i64 *col, double *w, double *fa, double *fb, double *aa, double *ab) {
    Mesh S = make_mesh(sn, sll, sc, soff, sidx), D = make_mesh(dn, dll, dc, doff, didx);
    axis::solver::RegridConfig cfg;
    cfg.norm_type = norm_type ? axis::solver::NormType::FracArea : axis::solver::NormType::DstArea;
    cfg.unmapped = unmapped ? axis::solver::UnmappedAction::Ignore : axis::solver::UnmappedAction::Error;
    IM m;
    try {
        if (kind == 0 || kind == 2) {
            auto sg = axis::detail::detect_regular_grid(S), dg = axis::detail::detect_regular_grid(D);
            if (!sg.is_regular || !dg.is_regular) return -2;
            m = kind == 0 ? axis::solver::generate_conservative_rect<HS>(S, D, cfg, sg, dg)
                          : axis::solver::generate_bilinear_rect<HS>(S, D, cfg, sg, dg);
        } else {
            auto sr = axis::detail::detect_rectilinear_grid(S);
            if (!sr.is_rectilinear) return -2;
            if (kind == 1) {
                auto dr = axis::detail::detect_rectilinear_grid(D);
                if (!dr.is_rectilinear) return -2;
                m = axis::solver::generate_conservative_rect_nonuniform<HS>(S, D, cfg, sr, dr);
            } else {
                m = axis::solver::generate_bilinear_rect_nonuniform<HS>(S, D, cfg, sr);
            }
        }
    } catch (const std::exception &) {
        return -3;
    }
    if (m.n_dst() == 0 && dc > 0) return -1;
    m.to_csr();
    auto rp = m.row_ptr();
    auto ci = m.col_idx();
    auto cv = m.csr_values();
    *nnz = static_cast<i64>(ci.extent(0));
    if (*nnz > cap) return 0;
    for (i64 j = 0; j < dc; ++j)
        for (i64 k = rp(j); k < rp(j + 1); ++k) {
            row[k] = j;
            col[k] = ci(k);
            w[k] = cv(k);
        }
    auto vfa = m.frac_a_view(), vfb = m.frac_b_view(), vaa = m.area_a_view(), vab = m.area_b_view();
    for (i64 i = 0; i < sc; ++i) {
        fa[i] = vfa(i);
        aa[i] = vaa(i);
    }
    for (i64 j = 0; j < dc; ++j) {
        fb[j] = vfb(j);
        ab[j] = vab(j);
    }
    return 0;
}

}  // extern "C"
