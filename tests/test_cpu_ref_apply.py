"""Pins the oracle's NaN-aware batch apply, masked apply and conservation
report against the reference's own code (include/axis/solver/apply.hpp, the
team-policy CSR paths of nan_batch_apply and the masked apply, and
src/solver/conservation.cpp), compiled unchanged by oracle/build.py into
oracle/_ref/libaxisref_apply.so. Bit for bit, NaN positions included.
Skipped where the reference checkout (and so that library) is absent."""
import numpy as np
import pytest

from axgb import grids


@pytest.fixture(scope="module")
def ref():
    from oracle import RefApplyLib
    try:
        return RefApplyLib()
    except FileNotFoundError:
        pytest.skip("reference checkout not present: reference apply library not built")


PAIRS = [(grids.latlon_deg(5.0), grids.cubed_sphere(8)), (grids.cubed_sphere(12), grids.latlon_deg(10.0)),
         (grids.tripole(48, 36, seed=4, jitter=0.1), grids.latlon_deg(10.0))]


@pytest.mark.parametrize("i", range(len(PAIRS)))
def test_nan_batch_apply_pinned(ref, oracle, i):
    w = oracle.conservative(*PAIRS[i])
    rng = np.random.default_rng(40 + i)
    x = rng.standard_normal((8, w.n_src)) * 50.0 + 280.0
    for v in range(8):
        x[v, rng.uniform(size=w.n_src) < v / 8.0] = np.nan
    x[3, :] = np.nan  # a field that is all NaN
    for thres in (0.0, 0.1, 0.5, 0.9, 1.0):
        np.testing.assert_array_equal(ref.nan_batch_apply(w, x, thres), oracle.nan_batch_apply(w, x, thres))


@pytest.mark.parametrize("i", range(len(PAIRS)))
def test_masked_apply_pinned(ref, oracle, i):
    w = oracle.conservative(*PAIRS[i])
    rng = np.random.default_rng(50 + i)
    x = rng.standard_normal(w.n_src) * 50.0 + 280.0
    y0 = rng.standard_normal(w.n_dst)
    for mask in ((rng.random(w.n_dst) > 0.3).astype(np.int32), np.ones(w.n_dst, np.int32),
                 np.zeros(w.n_dst, np.int32)):
        np.testing.assert_array_equal(ref.apply_masked(w, x, mask, y0), oracle.apply_masked(w, x, mask, y0))


@pytest.mark.parametrize("i", range(len(PAIRS)))
@pytest.mark.parametrize("norm", [0, 1])
def test_conservation_report_pinned(ref, oracle, i, norm):
    w = oracle.conservative(*PAIRS[i], norm_type=norm)
    rng = np.random.default_rng(60 + i)
    x = rng.standard_normal(w.n_src) * 50.0 + 280.0
    y = oracle.apply_csr(w, x, compensated=False)[0]
    assert ref.conservation(w, x, y, norm) == oracle.conservation(w, x, y, norm)
