"""Pins the oracle's regular / rectilinear fast paths against the reference's
own sources (src/solver/weight_generator_conservative_rect.cpp,
_conservative_rect_nonuniform.cpp, _bilinear_rect.cpp,
_bilinear_rect_nonuniform.cpp), compiled unchanged by oracle/build.py into
oracle/_ref/libaxisref_fast.so with the reference's grid detection and
to_csr. Every array bit for bit. Skipped where the reference checkout (and so
that library) is absent."""
import numpy as np
import pytest

from axgb import grids


@pytest.fixture(scope="module")
def ref():
    from oracle import RefFastLib
    try:
        return RefFastLib()
    except FileNotFoundError:
        pytest.skip("reference checkout not present: fast-path reference library not built")


def _same(r, wo):
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(r, k), getattr(wo, k)), k


REGULAR = [
    (grids.latlon_deg(1.0), grids.latlon_deg(2.0)),
    (grids.latlon_deg(2.0), grids.latlon_deg(1.0)),
    (grids.latlon_deg(0.5), grids.latlon_deg(0.75)),
    (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0), grids.latlon_deg(2.0)),
    (grids.regular_latlon(360, 180, -180.0, -90.0, 1.0, 1.0), grids.latlon_deg(3.0)),
]
RECTILINEAR = [
    (grids.equal_area_latlon(72, 36, stretch=0.4), grids.latlon_deg(2.0)),
    (grids.latlon_deg(1.0), grids.equal_area_latlon(96, 48, lon_start=-180.0, stretch=0.3)),
    (grids.equal_area_latlon(180, 90, stretch=0.2), grids.equal_area_latlon(50, 28, lon_start=-90.0, stretch=0.5)),
    # a regular pair the regular path declines (non-global, longitudes do not fit)
    (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0), grids.regular_latlon(20, 20, 10.0, -20.0, 2.0, 2.0)),
]


@pytest.mark.parametrize("i", range(len(REGULAR)))
@pytest.mark.parametrize("norm", [0, 1])
def test_conservative_regular_pinned(ref, oracle, i, norm):
    src, dst = REGULAR[i]
    _same(ref.run(ref.CONS_REGULAR, src, dst, norm), oracle.conservative(src, dst, norm_type=norm))


@pytest.mark.parametrize("i", range(len(RECTILINEAR)))
@pytest.mark.parametrize("norm", [0, 1])
def test_conservative_rectilinear_pinned(ref, oracle, i, norm):
    src, dst = RECTILINEAR[i]
    _same(ref.run(ref.CONS_RECTILINEAR, src, dst, norm), oracle.conservative(src, dst, norm_type=norm))


@pytest.mark.parametrize("i", range(len(REGULAR)))
def test_bilinear_regular_pinned(ref, oracle, i):
    src, dst = REGULAR[i]
    _same(ref.run(ref.BIL_REGULAR, src, dst), oracle.bilinear(src, dst))


@pytest.mark.parametrize("src,dst", [(grids.latlon_deg(1.0), grids.cubed_sphere(48)),
                                     (grids.equal_area_latlon(72, 36, stretch=0.4), grids.cubed_sphere(24)),
                                     (grids.latlon_deg(5.0), grids.tripole(72, 54, seed=4))])
def test_bilinear_rectilinear_source_pinned(ref, oracle, src, dst):
    _same(ref.run(ref.BIL_RECTILINEAR, src, dst), oracle.bilinear(src, dst))
