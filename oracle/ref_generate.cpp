// Driver that runs the reference's OWN weight generator,
// axis::solver::WeightGenerator::generate (AXIS src/solver/weight_generator.cpp
// with the regular/rectilinear fast-path sources, gradient_reconstructor.cpp,
// halo_pattern.cpp and interpolation_matrix.cpp, compiled unchanged from the
// checkout through the host shims in ref_shim/, ArborX's queries replaced by
// the exhaustive search of ref_shim/ArborX.hpp), with masks, user areas and
// the whole configuration, and returns InterpolationMatrix::to_csr. It pins
// the oracle's restatements of the nearest-neighbour, general bilinear,
// masked conservative and coastal (NearestWet) paths and of the dispatch.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into
// oracle/_ref/libaxisref_gen.so when the reference checkout exists, and
// loaded only by tests/ and tests/golden/make_golden.py. The exhaustive
// search is quadratic: small grids only.

#include <Kokkos_Core.hpp>
#include <axis/solver/interpolation_matrix.hpp>
#include <axis/solver/regrid_config.hpp>
#include <axis/solver/weight_generator.hpp>
#include <axis/topology/unstructured_mesh.hpp>
#include <cstdint>
#include <cstdio>
#include <stdexcept>

using HS = Kokkos::HostSpace;
using Mesh = axis::topology::UnstructuredMesh<HS>;
using IM = axis::solver::InterpolationMatrix<HS>;
using i64 = std::int64_t;

namespace {

char g_err[512];

Mesh make_mesh(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx, const int *mask,
               const double *areas) {
    Kokkos::View<double **, Kokkos::LayoutLeft, HS> nc("nc", n_nodes, 2);
    for (i64 i = 0; i < 2 * n_nodes; ++i) nc.data()[i] = lonlat[i];
    Kokkos::View<axis::index_t *, HS> o("o", n_cells + 1), x("x", off[n_cells]);
    for (i64 i = 0; i <= n_cells; ++i) o(i) = off[i];
    for (i64 i = 0; i < off[n_cells]; ++i) x(i) = idx[i];
    Kokkos::View<double *, HS> a;
    Kokkos::View<int *, HS> m;
    if (areas) {
        a = Kokkos::View<double *, HS>("a", n_cells);
        for (i64 i = 0; i < n_cells; ++i) a(i) = areas[i];
    }
    if (mask) {
        m = Kokkos::View<int *, HS>("m", n_cells);
        for (i64 i = 0; i < n_cells; ++i) m(i) = mask[i];
    }
    return Mesh(nc, o, x, axis::topology::CoordinateSystem::SphericalDeg, a, m);
}

}  // namespace

extern "C" {

const char *ref_generate_error() { return g_err; }

// method: InterpolationMethod (0 Bilinear, 1 NearestNeighbor, 2 Bicubic,
// 3 Patch, 4 Conservative1stOrder, 5 Conservative2ndOrder); norm_type
// 0 DstArea / 1 FracArea; line_type 0 Cartesian / 1 GreatCircle; unmapped
// 0 Error / 1 Ignore; extrap 0 None / 1 NearestWet. Masks (1 = wet) and
// areas may be null. Writes the to_csr rows (one per entry), columns,
// values and frac/area arrays when nnz fits cap; returns 0, or -3 when the
// generator threw (the message is in ref_generate_error()).
int ref_generate(int method, i64 sn, const double *sll, i64 sc, const i64 *soff, const i64 *sidx, const int *smask,
                 const double *sarea, i64 dn, const double *dll, i64 dc, const i64 *doff, const i64 *didx,
                 const int *dmask, const double *darea, int norm_type, int line_type, int unmapped, int extrap,
                 i64 cap, i64 *nnz, i64 *row, i64 *col, double *w, double *fa, double *fb, double *aa, double *ab) {
    g_err[0] = 0;
    Mesh S = make_mesh(sn, sll, sc, soff, sidx, smask, sarea), D = make_mesh(dn, dll, dc, doff, didx, dmask, darea);
    axis::solver::RegridConfig cfg;
    cfg.method = static_cast<axis::solver::InterpolationMethod>(method);
    cfg.norm_type = norm_type ? axis::solver::NormType::FracArea : axis::solver::NormType::DstArea;
    cfg.line_type = line_type ? axis::solver::LineType::GreatCircle : axis::solver::LineType::Cartesian;
    cfg.unmapped = unmapped ? axis::solver::UnmappedAction::Ignore : axis::solver::UnmappedAction::Error;
    cfg.extrap_method = extrap ? axis::solver::ExtrapolationAction::NearestWet : axis::solver::ExtrapolationAction::None;
    IM m;
    try {
        m = axis::solver::WeightGenerator::generate<HS>(S, D, cfg);
    } catch (const std::exception &e) {
        std::snprintf(g_err, sizeof(g_err), "%s", e.what());
        return -3;
    }
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
        fa[i] = vfa.extent(0) > static_cast<std::size_t>(i) ? vfa(i) : 0.0;
        aa[i] = vaa.extent(0) > static_cast<std::size_t>(i) ? vaa(i) : 0.0;
    }
    for (i64 j = 0; j < dc; ++j) {
        fb[j] = vfb.extent(0) > static_cast<std::size_t>(j) ? vfb(j) : 0.0;
        ab[j] = vab.extent(0) > static_cast<std::size_t>(j) ? vab(j) : 0.0;
    }
    return 0;
}

}  // extern "C"
