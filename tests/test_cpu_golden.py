"""The oracle against golden vectors produced by the reference's own
geometry code (tests/golden, see make_golden.py): bit-for-bit."""
import numpy as np
import pytest

from golden_io import cases, load, mesh

CONS = cases("conservative")
CELL = cases("cellprep")


def test_fixtures_present():
    assert len(CONS) >= 4 and len(CELL) >= 3


@pytest.mark.parametrize("name", CONS)
def test_oracle_conservative_golden(oracle, name):
    z = load("conservative", name)
    w = oracle.conservative(mesh(z, "src"), mesh(z, "dst"))
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(w, k), z[k]), k


@pytest.mark.parametrize("name", CELL)
def test_oracle_cellprep_golden(oracle, name):
    z = load("cellprep", name)
    c = oracle.cell_prep(mesh(z, "mesh"))
    for k in ("area", "cap_c", "cap_r", "box", "degen"):
        assert np.array_equal(c[k], z[k]), k


def test_oracle_clip_golden(oracle):
    z = load("clip")
    for i in range(len(z["area"])):
        a = z["subj"][i, : z["n_subj"][i]]
        b = z["clip"][i, : z["n_clip"][i]]
        area, poly = oracle.clip(a, b)
        assert area == z["area"][i]
        assert np.array_equal(poly, z["out"][i, : z["n_out"][i]])
