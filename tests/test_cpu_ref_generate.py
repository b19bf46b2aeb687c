"""Pins the oracle against the reference's own WeightGenerator::generate
(src/solver/weight_generator.cpp with the solver sources it calls), compiled
unchanged by oracle/build.py into oracle/_ref/libaxisref_gen.so, with
ArborX's queries replaced by an exhaustive search (oracle/ref_shim/ArborX.hpp).
Covers the dispatch of every method, the nearest-neighbour and general
bilinear paths, source and destination masks (which nearest-neighbour and
bilinear do not read), the coastal post-pass with and without NearestWet,
and user cell areas. Every array bit for bit. Skipped
where the reference checkout (and so that library) is absent."""
import numpy as np
import pytest

from axgb import grids

PAIRS = {
    "5deg->C8": lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8)),
    "C12->C8": lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8)),
    "C8->10deg": lambda: (grids.cubed_sphere(8), grids.latlon_deg(10.0)),
    "tripole->10deg": lambda: (grids.tripole(48, 36, seed=4, jitter=0.1), grids.latlon_deg(10.0)),
    "5deg->10deg": lambda: (grids.latlon_deg(5.0), grids.latlon_deg(10.0)),
    "equal-area->10deg": lambda: (grids.equal_area_latlon(36, 18, stretch=0.4), grids.latlon_deg(10.0)),
    "voronoi->10deg": lambda: (grids.voronoi(642, seed=5), grids.latlon_deg(10.0)),
    "C8->voronoi": lambda: (grids.cubed_sphere(8), grids.voronoi(642, seed=5)),
    "regional->C8": lambda: (grids.regular_latlon(20, 15, 20.0, -10.0, 2.0, 2.0), grids.cubed_sphere(8)),
    "C8->regional": lambda: (grids.cubed_sphere(8), grids.regular_latlon(20, 15, 20.0, -10.0, 2.0, 2.0)),
    "shifted 5deg->C6": lambda: (grids.regular_latlon(72, 36, -180.0, -90.0, 5.0, 5.0), grids.cubed_sphere(6)),
    "equal-area->equal-area": lambda: (grids.equal_area_latlon(36, 18, stretch=0.4),
                                       grids.equal_area_latlon(24, 12, lon_start=-90.0, stretch=0.2)),
    "tripole->voronoi": lambda: (grids.tripole(24, 18, seed=2, jitter=0.1), grids.voronoi(162, seed=3)),
}
CASES = ["cons", "cons_fracarea", "nearest", "bilinear", "cons_srcmask_nearestwet", "cons_srcmask_none",
         "cons_dstmask", "cons_both_masks", "nearest_srcmask", "bilinear_srcmask", "cons_user_areas",
         "nearest_user_areas", "bilinear_user_areas", "nearest_dstmask_ignored", "bilinear_dstmask_ignored"]


@pytest.fixture(scope="module")
def ref():
    from oracle import RefGenLib
    try:
        return RefGenLib()
    except FileNotFoundError:
        pytest.skip("reference checkout not present: reference generator library not built")


def land_mask(src):
    c = grids.cell_centroids_xyz(src)
    lat = np.degrees(np.arcsin(c[:, 2]))
    lon = np.degrees(np.arctan2(c[:, 1], c[:, 0])) % 360
    return (~((lat > -30) & (lat < 40) & (lon > 20) & (lon < 110))).astype(np.int32)


def run_case(case, ref, oracle, s, d):
    """(reference output, oracle output) of one scenario."""
    m = land_mask(s)
    if m.min() == m.max():  # a regional grid wholly inside or outside the land box
        m[::3] = 1 - m[::3]
    rng = np.random.default_rng(22)
    dm = (rng.random(d.n_cells) > 0.1).astype(np.int32)
    if case == "cons":
        return ref.generate("conservative", s, d), oracle.conservative(s, d)
    if case == "cons_fracarea":
        return ref.generate("conservative", s, d, norm_type=1), oracle.conservative(s, d, norm_type=1)
    if case == "nearest":
        return ref.generate("nearest_neighbor", s, d), oracle.nearest(s, d)
    if case == "bilinear":
        return ref.generate("bilinear", s, d), oracle.bilinear(s, d)
    if case == "cons_srcmask_nearestwet":
        return (ref.generate("conservative", s, d, src_mask=m, extrap=1),
                oracle.coastal(oracle.conservative(s, d, src_mask=m), s, d, m, nearest_wet=True))
    if case == "cons_srcmask_none":
        return (ref.generate("conservative", s, d, src_mask=m, extrap=0),
                oracle.coastal(oracle.conservative(s, d, src_mask=m), s, d, m, nearest_wet=False))
    if case == "cons_dstmask":
        return ref.generate("conservative", s, d, dst_mask=dm), oracle.conservative(s, d, dst_mask=dm)
    if case == "cons_both_masks":
        return (ref.generate("conservative", s, d, src_mask=m, dst_mask=dm),
                oracle.coastal(oracle.conservative(s, d, src_mask=m, dst_mask=dm), s, d, m))
    if case == "nearest_srcmask":
        return ref.generate("nearest_neighbor", s, d, src_mask=m), oracle.coastal(oracle.nearest(s, d), s, d, m)
    if case == "bilinear_srcmask":
        return ref.generate("bilinear", s, d, src_mask=m), oracle.coastal(oracle.bilinear(s, d), s, d, m)
    if case == "cons_user_areas":
        w0 = oracle.conservative(s, d)
        sa = w0.area_a * (1.0 + 0.01 * rng.random(s.n_cells))
        da = w0.area_b * (1.0 + 0.01 * rng.random(d.n_cells))
        da[da == 0.0] = 1.0
        return (ref.generate("conservative", s, d, src_areas=sa, dst_areas=da),
                oracle.conservative(s, d, src_areas=sa, dst_areas=da))
    if case in ("nearest_user_areas", "bilinear_user_areas"):
        sa = np.linspace(1.0, 2.0, s.n_cells)
        da = np.linspace(3.0, 4.0, d.n_cells)
        fn = oracle.nearest if case.startswith("nearest") else oracle.bilinear
        meth = "nearest_neighbor" if case.startswith("nearest") else "bilinear"
        return ref.generate(meth, s, d, src_areas=sa, dst_areas=da), fn(s, d, src_areas=sa, dst_areas=da)
    if case in ("nearest_dstmask_ignored", "bilinear_dstmask_ignored"):
        # these methods do not read destination masks
        fn = oracle.nearest if case.startswith("nearest") else oracle.bilinear
        meth = "nearest_neighbor" if case.startswith("nearest") else "bilinear"
        return ref.generate(meth, s, d, dst_mask=dm), fn(s, d)
    raise ValueError(case)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("pair", list(PAIRS))
def test_oracle_matches_reference_generate(ref, oracle, pair, case):
    s, d = PAIRS[pair]()
    r, o = run_case(case, ref, oracle, s, d)
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(r, k), getattr(o, k)), k


def test_reference_generate_unmapped_error(ref, oracle):
    """A regional source under UnmappedAction::Error: the reference throws,
    naming the unmapped destination cell; the oracle refuses too."""
    s, d = grids.regular_latlon(20, 15, 20.0, -10.0, 2.0, 2.0), grids.cubed_sphere(6)
    with pytest.raises(RuntimeError, match="[Uu]nmapped"):
        ref.generate("conservative", s, d, unmapped=0)
    with pytest.raises(RuntimeError):
        oracle.conservative(s, d, unmapped=0)


degenerate = grids.with_degenerate_cells
triangulated = grids.triangulated

ODD = {
    "degenerate C8->10deg": lambda: (degenerate(grids.cubed_sphere(8), 1), grids.latlon_deg(10.0)),
    "5deg->degenerate C8": lambda: (grids.latlon_deg(5.0), degenerate(grids.cubed_sphere(8), 2)),
    "triangulated C6->10deg": lambda: (triangulated(grids.cubed_sphere(6)), grids.latlon_deg(10.0)),
    "10deg->triangulated C6": lambda: (grids.latlon_deg(10.0), triangulated(grids.cubed_sphere(6))),
    "triangulated C6->C5": lambda: (triangulated(grids.cubed_sphere(6)), grids.cubed_sphere(5)),
}


@pytest.mark.parametrize("case", ["cons", "cons_fracarea", "nearest", "bilinear"])
@pytest.mark.parametrize("pair", list(ODD))
def test_oracle_matches_reference_generate_odd_cells(ref, oracle, pair, case):
    """Degenerate cells (repeated vertices, cells collapsed to a point) and
    triangle meshes, on either side."""
    s, d = ODD[pair]()
    r, o = run_case(case, ref, oracle, s, d)
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(r, k), getattr(o, k)), k
