// Thin driver that runs the reference's OWN header-only geometry code
// (AXIS include/axis/detail/*.hpp and topology/unstructured_mesh.hpp,
// compiled unchanged through the host shim in ref_shim/) so that the
// restated oracle in oracle.cpp can be pinned against it bit for bit.
//
// TEST INFRASTRUCTURE ONLY: built by oracle/build.py into
// oracle/_ref/libaxisref.so from the reference sources where they lie, and
// loaded only by tests/. The glue that lives in the reference's
// weight_generator.cpp (which needs ArborX and cannot be compiled here) is
// restated below with citations: the float AABB, the cell-area polygon
// extraction, the centroid lon/lat for the Morton order, the exact box
// query that stands in for ArborX, the overlap loop and to_csr.

#include <Kokkos_Core.hpp>
#include <algorithm>
#include <axis/detail/degenerate_cell_handler.hpp>
#include <axis/detail/morton_sort.hpp>
#include <axis/detail/regular_grid_detector.hpp>
#include <axis/detail/spherical_cap_filter.hpp>
#include <axis/detail/spherical_clipper.hpp>
#include <axis/detail/spherical_geometry.hpp>
#include <axis/detail/trig_cache.hpp>
#include <axis/topology/unstructured_mesh.hpp>
#include <cstdint>
#include <numeric>
#include <vector>

using HS = Kokkos::HostSpace;
using Mesh = axis::topology::UnstructuredMesh<HS>;
using i64 = std::int64_t;
using axis::detail::SphericalPolygon;

namespace {

Mesh make_mesh(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx) {
    Kokkos::View<double **, Kokkos::LayoutLeft, HS> nc("nc", n_nodes, 2);
    for (i64 i = 0; i < 2 * n_nodes; ++i) nc.data()[i] = lonlat[i];
    Kokkos::View<axis::index_t *, HS> o("o", n_cells + 1), x("x", off[n_cells]);
    for (i64 i = 0; i <= n_cells; ++i) o(i) = off[i];
    for (i64 i = 0; i < off[n_cells]; ++i) x(i) = idx[i];
    return Mesh(nc, o, x, axis::topology::CoordinateSystem::SphericalDeg);
}

// extract_cell_polygon_spherical (src/solver/weight_generator.cpp:441-481)
SphericalPolygon<32> cell_poly(const Mesh &m, i64 c) {
    SphericalPolygon<32> sp;
    auto coords = m.node_coords();
    auto off = m.conn_offsets();
    auto idx = m.conn_indices();
    constexpr double deg2rad = axis::detail::spherical::pi / 180.0;
    for (i64 k = off[c]; k < off[c + 1]; ++k) {
        i64 n = idx[k];
        auto v = axis::detail::spherical::lonlat_to_xyz(coords(n, 0) * deg2rad, coords(n, 1) * deg2rad);
        sp.push(axis::detail::Vec3{v.x, v.y, v.z});
    }
    return sp;
}

// extract_cell_polygon_spherical_cached (src/solver/weight_generator.cpp:492-520)
SphericalPolygon<32> cached_poly(const axis::detail::NodeTrigCache<HS> &t, i64 c) {
    std::size_t ci = c % t.ni, cj = c / t.ni;
    SphericalPolygon<32> sp;
    auto at = [&](std::size_t i, std::size_t j) {
        auto v = axis::detail::lonlat_to_xyz_node_cached(t, i, j);
        sp.push(axis::detail::Vec3{v.x, v.y, v.z});
    };
    at(ci, cj);
    at(ci + 1, cj);
    at(ci + 1, cj + 1);
    at(ci, cj + 1);
    return sp;
}

struct FBox {
    float lo[3], hi[3];
};

// compute_cell_aabbs_3d (src/solver/weight_generator.cpp:198-262)
std::vector<FBox> boxes(const Mesh &m) {
    auto coords = m.node_coords();
    auto off = m.conn_offsets();
    auto idx = m.conn_indices();
    std::vector<FBox> b(m.n_cells());
    for (std::size_t c = 0; c < m.n_cells(); ++c) {
        double mn[3] = {std::numeric_limits<double>::max(), std::numeric_limits<double>::max(),
                        std::numeric_limits<double>::max()};
        double mx[3] = {-std::numeric_limits<double>::max(), -std::numeric_limits<double>::max(),
                        -std::numeric_limits<double>::max()};
        for (i64 k = off[c]; k < off[c + 1]; ++k) {
            i64 n = idx[k];
            const double pi = 3.14159265358979323846;
            double lon = coords(n, 0) * pi / 180.0, lat = coords(n, 1) * pi / 180.0;
            double p[3] = {std::cos(lat) * std::cos(lon), std::cos(lat) * std::sin(lon), std::sin(lat)};
            for (int d = 0; d < 3; ++d) {
                mn[d] = std::min(mn[d], p[d]);
                mx[d] = std::max(mx[d], p[d]);
            }
        }
        double ext = std::max({mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]});
        double eps = std::min(std::max(0.25 * ext, 1.0e-6), 0.02);
        for (int d = 0; d < 3; ++d) {
            b[c].lo[d] = static_cast<float>(mn[d] - eps);
            b[c].hi[d] = static_cast<float>(mx[d] + eps);
        }
    }
    return b;
}

bool meet(const FBox &a, const FBox &b) {
    for (int d = 0; d < 3; ++d)
        if (a.lo[d] > b.hi[d] || a.hi[d] < b.lo[d]) return false;
    return true;
}

// compute_cell_centroids_xy (src/solver/weight_generator.cpp:75-125)
void centroids_xy(const Mesh &m, Kokkos::View<double *, HS> &cx, Kokkos::View<double *, HS> &cy) {
    auto coords = m.node_coords();
    auto off = m.conn_offsets();
    auto idx = m.conn_indices();
    cx = Kokkos::View<double *, HS>("cx", m.n_cells());
    cy = Kokkos::View<double *, HS>("cy", m.n_cells());
    const double pi = 3.14159265358979323846;
    for (std::size_t c = 0; c < m.n_cells(); ++c) {
        double sx = 0, sy = 0, sz = 0;
        for (i64 k = off[c]; k < off[c + 1]; ++k) {
            double lon = coords(idx[k], 0) * pi / 180.0, lat = coords(idx[k], 1) * pi / 180.0;
            sx += std::cos(lat) * std::cos(lon);
            sy += std::cos(lat) * std::sin(lon);
            sz += std::sin(lat);
        }
        std::size_t nv = off[c + 1] - off[c];
        double inv = nv > 0 ? 1.0 / static_cast<double>(nv) : 0.0;
        double la = std::asin(sz * inv), lo = std::atan2(sy * inv, sx * inv);
        if (lo < 0.0) lo += 2.0 * pi;
        cx(c) = lo * 180.0 / pi;
        cy(c) = la * 180.0 / pi;
    }
}

}  // namespace

extern "C" {

int ref_cell_prep(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx, double *area,
                  double *cap_c, double *cap_r, float *box, int *degen) {
    Mesh m = make_mesh(n_nodes, lonlat, n_cells, off, idx);
    auto rep = axis::detail::DegenerateCellHandler::scan(m);
    for (i64 c = 0; c < n_cells; ++c) degen[c] = 0;
    for (std::size_t k = 0; k < rep.excluded_indices.size(); ++k)
        degen[rep.excluded_indices[k]] = static_cast<int>(rep.excluded_types[k]);
    auto caps = axis::detail::precompute_cap_data<HS>(m);
    auto bx = boxes(m);
    for (i64 c = 0; c < n_cells; ++c) {
        area[c] = cell_poly(m, c).area();
        cap_c[3 * c] = caps.centroids(c).x;
        cap_c[3 * c + 1] = caps.centroids(c).y;
        cap_c[3 * c + 2] = caps.centroids(c).z;
        cap_r[c] = caps.angular_radii(c);
        for (int d = 0; d < 3; ++d) {
            box[6 * c + d] = bx[c].lo[d];
            box[6 * c + 3 + d] = bx[c].hi[d];
        }
    }
    return 0;
}

int ref_detect(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx, int *flags, i64 *dims,
               double *vals) {
    Mesh m = make_mesh(n_nodes, lonlat, n_cells, off, idx);
    auto g = axis::detail::detect_regular_grid(m);
    auto r = axis::detail::detect_rectilinear_grid(m);
    flags[0] = g.is_regular;
    flags[1] = r.is_rectilinear;
    dims[0] = static_cast<i64>(r.ni);
    dims[1] = static_cast<i64>(r.nj);
    vals[0] = g.lon_min;
    vals[1] = g.delta_lon;
    vals[2] = g.lat_min;
    vals[3] = g.delta_lat;
    return 0;
}

int ref_morton_order(i64 n_nodes, const double *lonlat, i64 n_cells, const i64 *off, const i64 *idx, i64 *perm) {
    Mesh m = make_mesh(n_nodes, lonlat, n_cells, off, idx);
    Kokkos::View<double *, HS> cx, cy;
    centroids_xy(m, cx, cy);
    Kokkos::View<const double *, HS> ccx(cx), ccy(cy);
    auto p = axis::detail::morton_sort_indices<HS>(ccx, ccy, m.n_cells());
    for (i64 c = 0; c < n_cells; ++c) perm[c] = p(c);
    return 0;
}

std::uint64_t ref_morton_encode(std::uint32_t x, std::uint32_t y) { return axis::detail::morton_encode_2d(x, y); }
std::uint32_t ref_normalize_coord(double v, double lo, double hi) { return axis::detail::normalize_coord(v, lo, hi); }

double ref_clip(const double *subj, int ns, const double *clipp, int nc, double *out_xyz, int *out_n) {
    SphericalPolygon<32> a, b;
    for (int i = 0; i < ns; ++i) a.push(axis::detail::Vec3{subj[3 * i], subj[3 * i + 1], subj[3 * i + 2]});
    for (int i = 0; i < nc; ++i) b.push(axis::detail::Vec3{clipp[3 * i], clipp[3 * i + 1], clipp[3 * i + 2]});
    auto r = axis::detail::SphericalClipper::clip(a, b);
    if (out_xyz)
        for (int i = 0; i < r.n; ++i) {
            out_xyz[3 * i] = r.verts[i].x;
            out_xyz[3 * i + 1] = r.verts[i].y;
            out_xyz[3 * i + 2] = r.verts[i].z;
        }
    if (out_n) *out_n = r.n;
    return r.area();
}

// Conservative weights through the reference's geometry code. Outputs in
// CSR order (row, col ascending); counts nnz into *nnz and fills at most
// cap entries. The per-destination candidate list is ascending source
// index (the set ArborX returns, in a fixed order).
int ref_conservative(i64 sn, const double *sll, i64 sc, const i64 *so, const i64 *si, i64 dn, const double *dll, i64 dc,
                     const i64 *dof, const i64 *di, i64 cap, i64 *nnz, i64 *row, i64 *col, double *w, double *fa,
                     double *fb, double *aa, double *ab) {
    Mesh S = make_mesh(sn, sll, sc, so, si);
    Mesh D = make_mesh(dn, dll, dc, dof, di);
    auto sgi = axis::detail::detect_regular_grid(S), dgi = axis::detail::detect_regular_grid(D);
    auto sdr = axis::detail::DegenerateCellHandler::scan(S), ddr = axis::detail::DegenerateCellHandler::scan(D);
    std::vector<char> sdeg(sc, 0), ddeg(dc, 0);
    for (auto i : sdr.excluded_indices) sdeg[i] = 1;
    for (auto i : ddr.excluded_indices) ddeg[i] = 1;
    auto sb = boxes(S), db = boxes(D);
    // exact box pairs through a coarse uniform grid on the box minima
    const int G = 64;
    auto cell_of = [&](float v) { return std::max(0, std::min(G - 1, static_cast<int>((v + 1.5f) / 3.0f * G))); };
    std::vector<std::vector<int>> bucket(static_cast<size_t>(G) * G * G);
    for (i64 i = 0; i < sc; ++i)
        for (int x = cell_of(sb[i].lo[0]); x <= cell_of(sb[i].hi[0]); ++x)
            for (int y = cell_of(sb[i].lo[1]); y <= cell_of(sb[i].hi[1]); ++y)
                for (int z = cell_of(sb[i].lo[2]); z <= cell_of(sb[i].hi[2]); ++z)
                    bucket[(static_cast<size_t>(x) * G + y) * G + z].push_back(static_cast<int>(i));
    std::vector<double> sarea(sc), darea(dc);
    for (i64 c = 0; c < sc; ++c) sarea[c] = cell_poly(S, c).area();
    for (i64 c = 0; c < dc; ++c) darea[c] = cell_poly(D, c).area();
    Kokkos::View<double *, HS> cx, cy;
    centroids_xy(D, cx, cy);
    Kokkos::View<const double *, HS> ccx(cx), ccy(cy);
    auto order = axis::detail::morton_sort_indices<HS>(ccx, ccy, dc);
    auto scap = axis::detail::precompute_cap_data<HS>(S);
    auto dcap = axis::detail::precompute_cap_data<HS>(D);
    axis::detail::NodeTrigCache<HS> st, dt;
    if (sgi.is_regular) st = axis::detail::build_node_trig_cache<HS>(sgi);
    if (dgi.is_regular) dt = axis::detail::build_node_trig_cache<HS>(dgi);
    std::vector<double> fav(sc, 0.0), fbv(dc, 0.0), wv;
    std::vector<i64> rv, cv;
    std::vector<int> cand;
    for (i64 k = 0; k < dc; ++k) {
        i64 j = order(k);
        if (ddeg[j]) continue;
        double ad = darea[j];
        if (ad <= 0.0) continue;
        cand.clear();
        for (int x = cell_of(db[j].lo[0]); x <= cell_of(db[j].hi[0]); ++x)
            for (int y = cell_of(db[j].lo[1]); y <= cell_of(db[j].hi[1]); ++y)
                for (int z = cell_of(db[j].lo[2]); z <= cell_of(db[j].hi[2]); ++z)
                    for (int i : bucket[(static_cast<size_t>(x) * G + y) * G + z])
                        if (meet(sb[i], db[j])) cand.push_back(i);
        std::sort(cand.begin(), cand.end());
        cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
        auto dp = dt.valid ? cached_poly(dt, j) : cell_poly(D, j);
        for (int i : cand) {
            if (sdeg[i]) continue;
            double as = sarea[i];
            if (as <= 0.0) continue;
            if (axis::detail::spherical_cap_rejects(scap.centroids(i), scap.angular_radii(i), dcap.centroids(j),
                                                    dcap.angular_radii(j)))
                continue;
            auto sp = st.valid ? cached_poly(st, i) : cell_poly(S, i);
            double ov = axis::detail::SphericalClipper::overlap_area<32>(sp, dp);
            if (ov <= 0.0) continue;
            double wij = std::max(ov / ad, 0.0);
            wv.push_back(wij);
            rv.push_back(j);
            cv.push_back(i);
            fav[i] += ov / as;
            fbv[j] += ov / ad;
        }
    }
    for (auto &x : fav) x = std::min(x, 1.0);
    for (auto &x : fbv) x = std::min(x, 1.0);
    std::vector<i64> perm(wv.size());
    std::iota(perm.begin(), perm.end(), 0);
    std::sort(perm.begin(), perm.end(), [&](i64 a, i64 b) { return rv[a] != rv[b] ? rv[a] < rv[b] : cv[a] < cv[b]; });
    *nnz = static_cast<i64>(perm.size());
    for (i64 k = 0; k < std::min<i64>(cap, *nnz); ++k) {
        row[k] = rv[perm[k]];
        col[k] = cv[perm[k]];
        w[k] = wv[perm[k]];
    }
    if (*nnz <= cap) {
        std::copy(fav.begin(), fav.end(), fa);
        std::copy(fbv.begin(), fbv.end(), fb);
        std::copy(sarea.begin(), sarea.end(), aa);
        std::copy(darea.begin(), darea.end(), ab);
    }
    return 0;
}

}  // extern "C"
