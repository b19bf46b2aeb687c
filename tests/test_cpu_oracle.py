"""CPU tests of the oracle: pinned against the reference's own geometry
headers (oracle/_ref, built from the reference checkout where it exists) and
against the known answers of the reference's unit tests."""
import numpy as np
import pytest

from axgb import grids


def test_spmv_known_answers(oracle):
    # tests/test_spmv_apply.cpp:33-105 of the reference: 3 src, 2 dst
    from oracle import Weights
    w = Weights(3, 2, np.array([0, 0, 1, 1]), np.array([0, 1, 1, 2]), np.array([0.5, 0.3, 0.2, 1.0]),
                np.ones(3), np.ones(2), np.ones(3), np.ones(2))
    y = oracle.apply_csr(w, np.array([2.0, 4.0, 6.0]))[0]
    assert abs(y[0] - 2.2) < 1e-14 and abs(y[1] - 6.8) < 1e-14
    y = oracle.apply_csr(w, np.array([1.0, 1.0, 1.0]))[0]
    assert abs(y[0] - 0.8) < 1e-14 and abs(y[1] - 1.2) < 1e-14
    y2 = oracle.apply_coo_atomic(w, np.array([2.0, 4.0, 6.0]))[0]
    assert abs(y2[0] - 2.2) < 1e-14 and abs(y2[1] - 6.8) < 1e-14


def test_morton_known_answers(oracle):
    # tests/test_morton_sort.cpp:19-118 of the reference
    e = oracle.morton_encode
    assert e(0, 0) == 0 and e(1, 0) == 1 and e(0, 1) == 2 and e(1, 1) == 3 and e(2, 2) == 12
    assert e(65535, 65535) == 0xFFFFFFFF
    assert e(3, 5) != e(5, 3)
    n = oracle.normalize_coord
    assert n(0.0, 0.0, 100.0) == 0 and n(100.0, 0.0, 100.0) == 65535
    assert abs(n(50.0, 0.0, 100.0) - 32767.5) <= 1.0
    assert n(-10.0, 0.0, 100.0) == 0 and n(200.0, 0.0, 100.0) == 65535
    assert n(5.0, 10.0, 10.0) == 0 and n(5.0, 10.0, 5.0) == 0
    assert abs(n(0.0, -180.0, 180.0) - 32767.5) <= 1.0


def _cap_poly(center, radius, nv):
    c = np.asarray(center, float)
    c /= np.linalg.norm(c)
    arb = np.array([0, 0, 1.0]) if abs(c[2]) < 0.9 else np.array([1.0, 0, 0])
    u = np.cross(c, arb)
    u /= np.linalg.norm(u)
    v = np.cross(c, u)
    a = 2 * np.pi * np.arange(nv) / nv
    p = c[None] * np.cos(radius) + np.sin(radius) * (np.cos(a)[:, None] * u + np.sin(a)[:, None] * v)
    return p / np.linalg.norm(p, axis=1, keepdims=True)


def _ll(lon, lat):
    return np.array([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)])


def test_clipper_properties(oracle):
    # tests/prop_spherical_clipper.cpp:84-228 of the reference
    rng = np.random.default_rng(7)
    for _ in range(200):
        ca = _ll(rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3))
        cb = _ll(np.pi + rng.uniform(-0.3, 0.3), rng.uniform(-0.3, 0.3))
        a = _cap_poly(ca, rng.uniform(0.05, 0.5), rng.integers(4, 9))
        b = _cap_poly(cb, rng.uniform(0.05, 0.5), rng.integers(4, 9))
        area, _ = oracle.clip(a, b)
        assert area == 0.0
    for _ in range(200):
        c = _ll(rng.uniform(-3, 3), rng.uniform(-1.2, 1.2))
        big = _cap_poly(c, rng.uniform(0.3, 0.6), rng.integers(6, 12))
        small = _cap_poly(c, rng.uniform(0.05, 0.1), rng.integers(4, 9))
        a0 = oracle.poly_area(small)
        a1, _ = oracle.clip(small, big)
        assert abs(a1 - a0) / a0 < 1e-14
    for _ in range(300):
        a = _cap_poly(_ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 1.0), rng.integers(3, 12))
        b = _cap_poly(_ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 1.0), rng.integers(3, 12))
        area, poly = oracle.clip(a, b)
        assert poly.shape[0] == 0 or poly.shape[0] >= 3
        assert np.isfinite(poly).all() and area >= 0.0


def test_clip_matches_reference(oracle, reflib):
    rng = np.random.default_rng(11)
    for _ in range(500):
        a = _cap_poly(_ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 0.5), rng.integers(3, 12))
        b = _cap_poly(_ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 0.5), rng.integers(3, 12))
        x1, p1 = oracle.clip(a, b)
        x2, p2 = reflib.clip(a, b)
        assert x1 == x2 and np.array_equal(p1, p2)


GRID_CASES = [
    ("latlon5", lambda: grids.latlon_deg(5.0)),
    ("C8", lambda: grids.cubed_sphere(8)),
    ("latlon1", lambda: grids.latlon_deg(1.0)),
    ("C48", lambda: grids.cubed_sphere(48)),
]


@pytest.mark.parametrize("name,make", GRID_CASES)
def test_cell_prep_matches_reference(oracle, reflib, name, make):
    m = make()
    a = oracle.cell_prep(m)
    b = reflib.cell_prep(m)
    for k in a:
        assert np.array_equal(a[k], b[k]), k
    assert oracle.detect(m) == reflib.detect(m)
    assert np.array_equal(oracle.morton_order(m), reflib.morton_order(m))


PAIRS = [
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("5deg->C8", lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8))),
    ("C12->C8", lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8))),
]


@pytest.mark.parametrize("name,make", PAIRS)
def test_conservative_matches_reference(oracle, reflib, name, make):
    src, dst = make()
    wo = oracle.conservative(src, dst)
    wf = oracle.conservative(src, dst, faithful=True)
    wr = reflib.conservative(src, dst)
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(wo, k), getattr(wr, k)), k
        assert np.array_equal(getattr(wo, k), getattr(wf, k)), k
    # row sums of a global-to-global conservative map are 1 (DstArea)
    rs = np.bincount(wo.row, weights=wo.w, minlength=wo.n_dst)
    assert np.all(np.abs(rs - 1.0) < 1e-11)


def test_conservation_report(oracle):
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    w = oracle.conservative(src, dst)
    x = np.cos(np.radians(np.repeat(np.arange(-87.5, 90, 5.0), 72))) + 280.0
    y = oracle.apply_csr(w, x)[0]
    rep = oracle.conservation(w, x, y)
    assert rep["relative_error"] < 1e-12


def test_bilinear_rect_source(oracle):
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    w = oracle.bilinear(src, dst)
    assert w.nnz == 4 * dst.n_cells
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    assert np.allclose(rs, 1.0, atol=1e-14)
    assert np.all(w.w >= 0) and np.all(w.col < src.n_cells)


def test_voronoi_mesh(oracle):
    """The spherical Voronoi generator: closed, counter-clockwise cells that
    tile the sphere, mostly 5- to 7-gons, conservative row sums of 1."""
    g = grids.voronoi(10242, seed=5, jitter=0.2, lloyd=5)
    nv = np.diff(g.conn_offsets)
    assert g.n_cells == 10242 and np.mean((nv >= 5) & (nv <= 7)) > 0.98
    c = oracle.cell_prep(g)
    assert np.all(c["degen"] == 0)
    assert abs(c["area"].sum() / (4 * np.pi) - 1.0) < 1e-12
    w = oracle.conservative(g, grids.latlon_deg(5.0))
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    assert np.all(np.abs(rs - 1.0) < 1e-11)


def _nan_case(oracle):
    # the source mesh and NaN pattern of the reference's fused NaN SpMV test
    # (tests_python/test_fused_nan_spmv.py:23-60); the destination is a
    # cubed sphere (its regular -> regular bilinear fast path is not restated)
    src = grids.regular_latlon(10, 5, 0.0, -90.0, 36.0, 36.0)
    dst = grids.cubed_sphere(4)
    w = oracle.bilinear(src, dst)
    x = np.ones((3, w.n_src))
    x[0, ::3] = np.nan
    x[1, 1::4] = np.nan
    x[2, ::2] = np.nan
    return w, x


def test_nan_batch_apply_oracle(oracle):
    """The fused NaN-aware apply against the reference test's manual
    formula (masked sum / valid weight, NaN below the valid fraction)."""
    w, x = _nan_case(oracle)
    got = oracle.nan_batch_apply(w, x, 0.5)
    mask = np.isnan(x)
    num = oracle.apply_csr(w, np.where(mask, 0.0, x), compensated=False)
    den = oracle.apply_csr(w, (~mask).astype(np.float64), compensated=False)
    tot = oracle.apply_csr(w, np.ones((1, w.n_src)), compensated=False)[0]
    with np.errstate(divide="ignore", invalid="ignore"):
        exp = np.where(den / tot[None, :] < (1.0 - 0.5 - 1e-6), np.nan, num / den)
    np.testing.assert_allclose(got, exp, rtol=1e-12, equal_nan=True)
    assert np.isnan(got).any() and np.isfinite(got).any()


def test_apply_masked_oracle(oracle):
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    w = oracle.conservative(src, dst)
    x = np.cos(np.radians(np.repeat(np.arange(-87.5, 90, 5.0), 72))) + 280.0
    mask = (np.arange(w.n_dst) % 3 != 0).astype(np.int32)
    y0 = np.full(w.n_dst, -7.0)
    y = oracle.apply_masked(w, x, mask, y0)
    full = oracle.apply_csr(w, x, compensated=False)[0]
    assert np.all(y[mask == 0] == -7.0)
    assert np.allclose(y[mask == 1], full[mask == 1], rtol=1e-14)


def test_conservative_regular_known_answer(oracle):
    """The regular x regular fast path: a 2 deg cell over four 1 deg cells
    gets the exact spherical-band area fractions; row sums and source
    fractions are 1 for global grids."""
    w = oracle.conservative(grids.latlon_deg(1.0), grids.latlon_deg(2.0))
    d2r = np.pi / 180.0
    band = lambda lo, hi: np.sin(hi * d2r) - np.sin(lo * d2r)
    sel = w.row == 0
    assert np.array_equal(w.col[sel], [0, 1, 360, 361])
    exp = np.array([band(-90, -89), band(-90, -89), band(-89, -88), band(-89, -88)]) / band(-90, -88) / 2
    assert np.allclose(w.w[sel], exp, rtol=1e-14)
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    assert np.all(np.abs(rs - 1) < 1e-14) and np.all(np.abs(w.frac_a - 1) < 1e-14)


def _land_mask(src):
    # a rectangular "continent" of masked source cells
    c = grids.cell_centroids_xyz(src)
    lat = np.degrees(np.arcsin(c[:, 2]))
    lon = np.degrees(np.arctan2(c[:, 1], c[:, 0])) % 360
    return (~((lat > -30) & (lat < 40) & (lon > 20) & (lon < 110))).astype(np.int32)


def test_coastal_postpass_oracle(oracle):
    """Wet renormalisation and NearestWet extrapolation: coastal rows sum to
    1, land rows take the nearest wet source with weight 1."""
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    mask = _land_mask(src)
    w = oracle.conservative(src, dst, src_mask=mask)
    assert np.all(mask[w.col] > 0)
    wc = oracle.coastal(w, src, dst, mask)
    rs = np.bincount(wc.row, weights=wc.w, minlength=wc.n_dst)
    counts = np.bincount(wc.row, minlength=wc.n_dst)
    assert np.all(counts > 0)
    assert np.all(np.abs(rs - 1.0) < 1e-12)
    dry = np.setdiff1d(np.arange(w.n_dst), np.unique(w.row))
    assert len(dry) > 0 and np.all(counts[dry] == 1)
    none = oracle.coastal(w, src, dst, mask, nearest_wet=False)
    assert set(np.unique(none.row)) == set(np.unique(w.row))


def test_conservative_rectilinear_oracle(oracle):
    """Non-uniform rectilinear fast path (weight_generator_conservative_rect_
    nonuniform.cpp): on two global grids every row sums to 1 and every source
    cell is fully used (frac 1, area-weighted column sums = source areas)."""
    src = grids.equal_area_latlon(72, 36, stretch=0.4)
    dst = grids.equal_area_latlon(50, 28, lon_start=-180.0, stretch=0.3)
    w = oracle.conservative(src, dst)
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    assert np.all(np.abs(rs - 1.0) < 1e-12)
    assert np.all(np.abs(w.frac_a - 1.0) < 1e-12) and np.all(np.abs(w.frac_b - 1.0) < 1e-12)
    cs = np.bincount(w.col, weights=w.w * w.area_b[w.row], minlength=w.n_src)
    assert np.all(np.abs(cs - w.area_a) < 1e-12 * w.area_a.max())
    # equal-area bands: every source band has the same area per unit longitude
    band = w.area_a.reshape(36, 72).sum(axis=1)
    assert np.all(np.abs(band - band[0]) < 1e-12 * band[0])


def test_conservative_declined_regular_takes_rectilinear_path(oracle):
    """Two non-global regular grids whose longitudes do not fit are declined
    by the regular fast path and handled by the rectilinear one: band-overlap
    weights, rows inside the source sum to 1, rows outside stay empty."""
    src = grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0)  # lon 20..60, lat -10..20
    dst = grids.regular_latlon(20, 20, 10.0, -20.0, 2.0, 2.0)  # lon 10..50, lat -20..20
    w = oracle.conservative(src, dst)
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    counts = np.bincount(w.row, minlength=w.n_dst)
    assert np.all(rs <= 1.0 + 1e-12)
    inside = 5 * 20 + 5  # lon 20..22, lat -10..-8: four source cells
    assert counts[inside] == 4 and abs(rs[inside] - 1.0) < 1e-12
    assert counts[5 * 20 + 4] == 0  # lon 18..20 only touches the source edge
    assert counts[4 * 20 + 5] == 0  # lat -12..-10 likewise


def test_bilinear_regular_known_answer(oracle):
    """Regular bilinear fast path: 10 deg cells onto 20 deg cells put every
    destination centre on the corner of four source cells (weights 1/4); a
    field linear in latitude is reproduced exactly away from the poles."""
    src, dst = grids.latlon_deg(10.0), grids.latlon_deg(20.0)
    w = oracle.bilinear(src, dst)
    assert w.nnz == 4 * dst.n_cells
    assert np.all(w.w == 0.25)
    assert np.all(np.bincount(w.row, minlength=w.n_dst) == 4)
    lat_s = np.repeat(-85.0 + 10.0 * np.arange(18), 36)
    y = np.bincount(w.row, weights=w.w * lat_s[w.col], minlength=w.n_dst)
    lat_d = np.repeat(-80.0 + 20.0 * np.arange(9), 18)
    assert np.allclose(y, lat_d, rtol=0, atol=1e-12)


def test_nearest_regular_known_answer(oracle):
    """generate_nearest_rect: a 20 deg cell's lower-left corner (20i, -90+20j)
    rounds to the 10 deg source cell (2i, 2j); weights 1, frac and areas 0."""
    src, dst = grids.latlon_deg(10.0), grids.latlon_deg(20.0)
    w = oracle.nearest(src, dst)
    assert w.nnz == dst.n_cells and np.all(w.w == 1.0)
    j = np.arange(dst.n_cells)
    di, dj = j % 18, j // 18
    assert np.array_equal(w.row, j)
    assert np.array_equal(w.col, (2 * dj) * 36 + 2 * di)
    assert not np.any(w.frac_a) and not np.any(w.area_b)


def test_nearest_unstructured_is_nearest(oracle):
    """generate_nearest_impl<3>: one weight-1 entry per destination, at a
    source centroid as near as any (to float rounding of the points)."""
    src, dst = grids.cubed_sphere(8), grids.latlon_deg(10.0)
    w = oracle.nearest(src, dst)
    assert w.nnz == dst.n_cells and np.array_equal(w.row, np.arange(dst.n_cells)) and np.all(w.w == 1.0)

    def unit(m):
        # compute_cell_centroids_xy: lat = asin of the unnormalised mean z,
        # lon = atan2 of the mean y, x; then the unit vector of (lon, lat)
        ll = np.radians(m.node_lonlat[m.conn_indices])
        v = np.stack([np.cos(ll[:, 1]) * np.cos(ll[:, 0]), np.cos(ll[:, 1]) * np.sin(ll[:, 0]), np.sin(ll[:, 1])], 1)
        nv = np.diff(m.conn_offsets)
        mean = np.add.reduceat(v, m.conn_offsets[:-1], axis=0) / nv[:, None]
        lat, lon = np.arcsin(mean[:, 2]), np.arctan2(mean[:, 1], mean[:, 0])
        return np.stack([np.cos(lat) * np.cos(lon), np.cos(lat) * np.sin(lon), np.sin(lat)], 1)
    s, d = unit(src), unit(dst)
    dist = np.linalg.norm(d[:, None, :] - s[None, :, :], axis=2)
    chosen = dist[np.arange(dst.n_cells), w.col]
    assert np.all(chosen <= dist.min(axis=1) + 1e-6)
    assert np.all(w.frac_a == 1.0) and np.all(w.area_a > 0)


def test_bilinear_general_oracle(oracle):
    """Bilinear from a cubed sphere (the point-location path): 3 or 4
    non-negative weights per row (quad, triangle or inverse distance) summing
    to 1, each row's sources among its eight nearest centroids."""
    src, dst = grids.cubed_sphere(12), grids.latlon_deg(10.0)
    w = oracle.bilinear(src, dst)
    counts = np.bincount(w.row, minlength=w.n_dst)
    assert np.all((counts >= 1) & (counts <= 4))
    assert np.all(w.w >= 0.0)
    rs = np.bincount(w.row, weights=w.w, minlength=w.n_dst)
    assert np.abs(rs - 1.0).max() < 1e-12
    assert np.all(w.area_a == 0.0) and np.all(w.area_b > 0.0)


@pytest.mark.parametrize("make", [lambda: grids.cubed_sphere(12), lambda: grids.tripole(48, 36, seed=4, jitter=0.1),
                                  lambda: grids.voronoi(642, seed=5), lambda: grids.latlon_deg(5.0)])
def test_cap_radius_soundness(oracle, make):
    """prop_spherical_cap_filter.cpp: every vertex of a cell lies inside its
    bounding cap (angle from the centre <= radius, to 1e-12 with numpy trig), and the cap test
    never rejects a pair the clipper finds overlapping (every kept pair of a
    conservative weight set passes acos(c1.c2) <= r1 + r2)."""
    m = make()
    c = oracle.cell_prep(m)
    ll = np.radians(np.asarray(m.node_lonlat, np.float64))
    nodes = np.stack([np.cos(ll[:, 1]) * np.cos(ll[:, 0]), np.cos(ll[:, 1]) * np.sin(ll[:, 0]), np.sin(ll[:, 1])], 1)
    cell_of = np.repeat(np.arange(m.n_cells), np.diff(m.conn_offsets))
    dots = np.einsum("ij,ij->i", nodes[m.conn_indices], c["cap_c"][cell_of])
    ang = np.arccos(np.clip(dots, -1.0, 1.0))
    assert np.all(ang <= c["cap_r"][cell_of] + 1e-12)
    w = oracle.conservative(m, grids.latlon_deg(10.0))
    d = oracle.cell_prep(grids.latlon_deg(10.0))
    cosang = np.einsum("ij,ij->i", c["cap_c"][w.col], d["cap_c"][w.row])
    assert np.all(np.arccos(np.clip(cosang, -1.0, 1.0)) <= c["cap_r"][w.col] + d["cap_r"][w.row] + 1e-14)
