"""The oracle against golden vectors produced by the reference's own
geometry code (tests/golden, see make_golden.py): bit-for-bit."""
import numpy as np
import pytest

from golden_io import cases, load, mesh

CONS = cases("conservative")
CELL = cases("cellprep")
FAST = cases("fastpath")
GEN = cases("generate")


def test_fixtures_present():
    assert len(CONS) >= 4 and len(CELL) >= 3 and len(FAST) >= 6 and len(GEN) >= 9


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


@pytest.mark.parametrize("name", FAST)
def test_oracle_fastpath_golden(oracle, name):
    """The oracle's dispatch (regular, then rectilinear, then the clipper for
    conservative; regular, then rectilinear source for bilinear) against the
    reference's own fast-path sources on the same pair: every array bit for
    bit."""
    z = load("fastpath", name)
    src, dst = mesh(z, "src"), mesh(z, "dst")
    if str(z["method"]) == "conservative":
        w = oracle.conservative(src, dst, norm_type=int(z["norm_type"]))
    else:
        w = oracle.bilinear(src, dst)
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(w, k), z[k]), k


def oracle_generate(oracle, z, src, dst):
    """The oracle's composition of one generate() fixture: the method's
    weights (masked destination rows dropped), then the coastal post-pass
    when the source has a mask."""
    method = str(z["method"])
    sm = np.asarray(z["src_mask"]) if "src_mask" in z else None
    dm = np.asarray(z["dst_mask"]) if "dst_mask" in z else None
    if method == "conservative":
        w = oracle.conservative(src, dst, src_mask=sm, dst_mask=dm)
    elif method == "bilinear":
        w = oracle.bilinear(src, dst)
    else:
        w = oracle.nearest(src, dst)
    if sm is not None:
        w = oracle.coastal(w, src, dst, sm, nearest_wet=bool(int(z["extrap"])))
    return w


@pytest.mark.parametrize("name", GEN)
def test_oracle_generate_golden(oracle, name):
    """Nearest-neighbour, general bilinear and masked / coastal weights
    against the reference's whole WeightGenerator::generate: bit for bit."""
    z = load("generate", name)
    w = oracle_generate(oracle, z, mesh(z, "src"), mesh(z, "dst"))
    for k in ("row", "col", "w", "frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(getattr(w, k), z[k]), k


def test_oracle_apply_golden(oracle):
    """NaN-aware batch apply and masked apply against the reference's own
    apply.hpp loops on the same CSR matrix: bit for bit, NaN positions
    included."""
    from oracle import Weights
    z = load("apply_nan_masked")
    n_src, n_dst = int(z["n_src"]), int(z["n_dst"])
    row = np.repeat(np.arange(n_dst), np.diff(z["row_ptr"]))
    w = Weights(n_src, n_dst, row, z["col"], z["val"], None, None, None, None)
    for t, ref in zip(z["thres"], z["y_nan"]):
        np.testing.assert_array_equal(oracle.nan_batch_apply(w, z["x"], float(t)), ref)
    np.testing.assert_array_equal(oracle.apply_masked(w, z["x_masked"], z["mask"], z["y0"]), z["y_masked"])


def test_weight_cache_blob_golden():
    """The reference's WeightCache blob of the 5 deg -> C8 matrix read with
    the layout of weight_cache.hpp:14-26 (40-byte header, then w, row, col,
    frac_a, frac_b, area_a, area_b): the same arrays as the weight fixture.
    Where the reference checkout exists, its serializer re-makes the blob
    byte for byte."""
    import struct
    blob = load("weight_cache", "5deg_to_C8")["blob"].tobytes()
    z = load("conservative", "5deg_to_C8")
    magic, version, endian = struct.unpack_from("<IIB", blob, 0)
    assert (magic, version, endian) == (0x43574841, 1, 1) and blob[9:16] == bytes(7)
    ns, nd, nz = struct.unpack_from("<QQQ", blob, 16)
    assert (ns, nd, nz) == (len(z["frac_a"]), len(z["frac_b"]), len(z["w"]))
    off = 40
    for name, n, dt in (("w", nz, "<f8"), ("row", nz, "<i8"), ("col", nz, "<i8"), ("frac_a", ns, "<f8"),
                        ("frac_b", nd, "<f8"), ("area_a", ns, "<f8"), ("area_b", nd, "<f8")):
        assert np.array_equal(np.frombuffer(blob, dtype=dt, count=n, offset=off), z[name]), name
        off += 8 * n
    assert off == len(blob)
    try:
        from oracle import RefApplyLib, ref_cache_blob
        lib = RefApplyLib()
    except FileNotFoundError:
        return
    assert ref_cache_blob(lib, ns, nd, z["row"], z["col"], z["w"], z["frac_a"], z["frac_b"], z["area_a"],
                          z["area_b"]) == blob
