"""ESMF weight files (EsmfWeightIO, src/io/esmf_weight_io.cpp:66-183) through
the host-only entry points, no device needed. scipy's NetCDF-3 reader and
writer (an independent implementation of the classic and 64-bit-offset
formats) check both directions: files axgb writes are read by scipy, and
files scipy writes, with the extra dimensions, variables, attributes and
record layouts other writers produce, are read by axgb."""
import numpy as np
import pytest

netcdf = pytest.importorskip("scipy.io").netcdf_file


def _weights(nnz, n_a=5000, n_b=3000, seed=3):
    rng = np.random.default_rng(seed)
    S = rng.random(nnz)
    col = rng.integers(1, n_a + 1, nnz).astype(np.int32)
    row = np.sort(rng.integers(1, n_b + 1, nnz)).astype(np.int32)
    return n_a, n_b, S, col, row


def test_written_file_reads_in_scipy(tmp_path):
    import axgb
    n_a, n_b, S, col, row = _weights(10007)
    p = tmp_path / "w.nc"
    axgb.esmf_write(p, n_a, n_b, S, col, row)
    with open(p, "rb") as fh:
        assert fh.read(4) == b"CDF\x02"  # 64-bit offset format
    f = netcdf(str(p), "r", mmap=False)
    try:
        assert f.version_byte == 2
        assert f.dimensions["num_wgts"] == S.size
        assert int(f.n_a) == n_a and int(f.n_b) == n_b
        assert f.variables["S"].typecode() == "d"
        assert f.variables["col_idx"].typecode() == "i" and f.variables["row_idx"].typecode() == "i"
        assert np.array_equal(f.variables["S"][:], S)
        assert np.array_equal(f.variables["col_idx"][:], col)
        assert np.array_equal(f.variables["row_idx"][:], row)
    finally:
        f.close()
    back = axgb.esmf_read(p)
    assert (back["n_a"], back["n_b"]) == (n_a, n_b)
    assert np.array_equal(back["S"], S) and np.array_equal(back["col_idx"], col)
    assert np.array_equal(back["row_idx"], row)


@pytest.mark.parametrize("version", [1, 2])
def test_reads_scipy_files_with_extra_content(tmp_path, version):
    """A classic or 64-bit-offset file with other dimensions, variables and
    attributes (as ESMF's own weight files carry) and S stored as float32."""
    import axgb
    n_a, n_b, S, col, row = _weights(777, seed=version)
    p = tmp_path / f"v{version}.nc"
    f = netcdf(str(p), "w", version=version)
    f.title = b"test weights"
    f.n_a = np.int32(n_a)
    f.n_b = np.int32(n_b)
    f.scale = np.float64(2.5)
    f.createDimension("n_a", n_a)
    f.createDimension("num_wgts", S.size)
    f.createDimension("n_b", n_b)
    xc = f.createVariable("xc_a", "d", ("n_a",))
    xc[:] = np.arange(n_a, dtype=np.float64)
    xc.units = b"degrees"
    v = f.createVariable("S", "f", ("num_wgts",))
    v[:] = S.astype(np.float32)
    v.long_name = b"weights"
    f.createVariable("col_idx", "i", ("num_wgts",))[:] = col
    f.createVariable("row_idx", "i", ("num_wgts",))[:] = row
    f.createVariable("frac_b", "d", ("n_b",))[:] = 1.0
    f.close()
    back = axgb.esmf_read(p)
    assert (back["n_a"], back["n_b"]) == (n_a, n_b)
    assert np.array_equal(back["S"], S.astype(np.float32).astype(np.float64))
    assert np.array_equal(back["col_idx"], col) and np.array_equal(back["row_idx"], row)


def test_reads_record_layout(tmp_path):
    """num_wgts as the unlimited dimension: records interleave S, col_idx,
    row_idx (and a short variable, so records are padded)."""
    import axgb
    n_a, n_b, S, col, row = _weights(501, seed=9)
    p = tmp_path / "rec.nc"
    f = netcdf(str(p), "w", version=2)
    f.n_a = np.int32(n_a)
    f.n_b = np.int32(n_b)
    f.createDimension("num_wgts", None)
    vs = f.createVariable("S", "d", ("num_wgts",))
    vc = f.createVariable("col_idx", "i", ("num_wgts",))
    vr = f.createVariable("row_idx", "i", ("num_wgts",))
    vq = f.createVariable("flag", "h", ("num_wgts",))
    vs[:] = S
    vc[:] = col
    vr[:] = row
    vq[:] = np.ones(S.size, np.int16)
    f.close()
    back = axgb.esmf_read(p)
    assert np.array_equal(back["S"], S) and np.array_equal(back["col_idx"], col)
    assert np.array_equal(back["row_idx"], row)


def test_empty_matrix_round_trip(tmp_path):
    import axgb
    p = tmp_path / "empty.nc"
    axgb.esmf_write(p, 10, 20, np.zeros(0), np.zeros(0, np.int32), np.zeros(0, np.int32))
    f = netcdf(str(p), "r", mmap=False)
    try:
        assert f.variables["S"][:].size == 0 and int(f.n_b) == 20
    finally:
        f.close()
    back = axgb.esmf_read(p)
    assert back["S"].size == 0 and (back["n_a"], back["n_b"]) == (10, 20)


def test_rejections(tmp_path):
    import axgb
    h5 = tmp_path / "h5.nc"
    h5.write_bytes(b"\x89HDF\r\n\x1a\n" + bytes(64))
    with pytest.raises(axgb.Unsupported):
        axgb.esmf_read(h5)
    p = tmp_path / "noattr.nc"
    f = netcdf(str(p), "w", version=2)
    f.createDimension("num_wgts", 3)
    for name, t in (("S", "d"), ("col_idx", "i"), ("row_idx", "i")):
        f.createVariable(name, t, ("num_wgts",))[:] = 1
    f.close()
    with pytest.raises(axgb.InvalidArgument):  # the reference reads n_a / n_b attributes
        axgb.esmf_read(p)
    n_a, n_b, S, col, row = _weights(100)
    good = tmp_path / "good.nc"
    axgb.esmf_write(good, n_a, n_b, S, col, row)
    cut = tmp_path / "cut.nc"
    cut.write_bytes(good.read_bytes()[:60])
    with pytest.raises(axgb.InvalidArgument):
        axgb.esmf_read(cut)
    with pytest.raises(axgb.InvalidArgument):
        axgb.esmf_read(tmp_path / "missing.nc")
