"""GPU parity: libaxgb (through its C ABI) against the CPU oracle on the same
seeded inputs. Index sets bit-exact after the reference's area threshold,
weights within 1e-12 relative, the FP64 apply within 1e-13 relative of a
compensated FP64 oracle, the split-FP32 apply within 1e-6 relative."""
import numpy as np
import pytest

from axgb import fields, grids

pytestmark = pytest.mark.gpu

W_RTOL = 1e-12  # weights / fractions vs the oracle
F64_RTOL = 1e-13  # FP64 apply vs compensated FP64 oracle
SPLIT_RTOL = 1e-6  # split-FP32 apply vs FP64 oracle on the same FP32 inputs


def _rows(csr, n_dst):
    return np.repeat(np.arange(n_dst), np.diff(csr["row_ptr"]))


def _mismatch_report(rows_g, cols_g, wo):
    g = set(zip(rows_g.tolist(), cols_g.tolist()))
    o = set(zip(wo.row.tolist(), wo.col.tolist()))
    only_g = sorted(g - o)[:10]
    only_o = sorted(o - g)[:10]
    return f"only GPU: {len(g - o)} {only_g}; only oracle: {len(o - g)} {only_o}"


def _check_weights(M, wo):
    csr = M.to_csr()
    rows = _rows(csr, M.n_dst)
    same = M.nnz == wo.nnz and np.array_equal(rows, wo.row) and np.array_equal(csr["col"], wo.col)
    assert same, _mismatch_report(rows, csr["col"], wo)
    rel = np.abs(csr["val"] - wo.w) / np.maximum(np.abs(wo.w), 1e-300)
    assert rel.max() < W_RTOL, rel.max()
    for k, ref in (("frac_a", wo.frac_a), ("frac_b", wo.frac_b), ("area_a", wo.area_a), ("area_b", wo.area_b)):
        d = np.abs(csr[k] - ref) / np.maximum(np.abs(ref), 1e-300)
        assert d.max() < W_RTOL, (k, d.max())
    return csr


PAIRS = [
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("5deg->C8", lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8))),
    ("C12->C8", lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8))),
    ("2deg->C96", lambda: (grids.latlon_deg(2.0), grids.cubed_sphere(96))),
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),
    ("tripole360x270->1deg", lambda: (grids.tripole(360, 270, seed=4), grids.latlon_deg(1.0))),
]


@pytest.mark.parametrize("name,make", PAIRS)
def test_conservative_parity(gpu, oracle, name, make):
    src, dst = make()
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    M = gpu.generate_weights(ms, md, {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    _check_weights(M, wo)
    st = M.stats()
    assert st["gated_pairs"] == wo.stats["cap_pass"], (st, wo.stats)


def test_conservative_fracarea_parity(gpu, oracle):
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst),
                             {"method": "conservative", "norm_type": "FracArea"})
    _check_weights(M, oracle.conservative(src, dst, norm_type=1))


def test_deterministic(gpu):
    src, dst = grids.latlon_deg(2.0), grids.cubed_sphere(24)
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    a = gpu.generate_weights(ms, md, {"method": "conservative"}).to_csr()
    b = gpu.generate_weights(ms, md, {"method": "conservative"}).to_csr()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_cell_geometry_parity(gpu, oracle):
    for g in (grids.latlon_deg(1.0), grids.cubed_sphere(48)):
        m = gpu.Mesh.from_grid(g)
        a = m.cell_geometry()
        b = oracle.cell_prep(g)
        assert np.array_equal(a["degen"], b["degen"])
        assert np.array_equal(a["cap_c"], b["cap_c"])
        assert np.max(np.abs(a["area"] - b["area"]) / b["area"]) < 1e-14
        assert np.max(np.abs(a["cap_r"] - b["cap_r"])) < 1e-15
        # float boxes: equal up to one float ulp where CUDA and libm trig differ
        assert np.max(np.abs(a["box"] - b["box"])) <= 1.2e-7
        assert np.mean(a["box"] == b["box"]) > 0.999


def test_bilinear_parity(gpu, oracle):
    src, dst = grids.latlon_deg(1.0), grids.cubed_sphere(48)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "bilinear"})
    wo = oracle.bilinear(src, dst)
    csr = M.to_csr()
    assert np.array_equal(_rows(csr, M.n_dst), wo.row)
    assert np.array_equal(csr["col"], wo.col)
    assert np.array_equal(csr["val"], wo.w)


def test_unsupported_and_unmapped(gpu, oracle):
    a = gpu.make_regular_mesh(36, 18, 0.0, -90.0, 10.0, 10.0)
    b = gpu.make_regular_mesh(18, 9, 0.0, -90.0, 20.0, 20.0)
    with pytest.raises(gpu.Unsupported):
        gpu.generate_weights(a, b, {"method": "bicubic"})
    with pytest.raises(gpu.Unsupported):
        gpu.generate_weights(a, b, {"method": "patch"})
    # a regional source leaves most of a global destination unmapped
    reg = grids.regular_latlon(20, 10, 0.0, 0.0, 2.0, 2.0)
    dst = grids.cubed_sphere(8)
    with pytest.raises(gpu.AxgbError) as e:
        gpu.generate_weights(gpu.Mesh.from_grid(reg), gpu.Mesh.from_grid(dst),
                             {"method": "conservative", "unmapped": "error"})
    assert e.value.code == gpu.ERR_UNMAPPED
    with pytest.raises(RuntimeError):
        oracle.conservative(reg, dst, unmapped=0)
    M = gpu.generate_weights(gpu.Mesh.from_grid(reg), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    _check_weights(M, oracle.conservative(reg, dst))


def test_invalid_mesh_rejected(gpu):
    g = grids.latlon_deg(10.0)
    bad = g.node_lonlat.copy()
    bad[3, 1] = np.nan
    with pytest.raises(gpu.InvalidArgument):
        gpu.Mesh.from_arrays(bad, g.conn_offsets, g.conn_indices)
    idx = g.conn_indices.copy()
    idx[5] = g.n_nodes + 3
    with pytest.raises(gpu.InvalidArgument):
        gpu.Mesh.from_arrays(g.node_lonlat, g.conn_offsets, idx)


# ─── apply ─────────────────────────────────────────────────────────────────


def test_spmv_golden_matrix(gpu):
    # tests/test_spmv_apply.cpp:33-142 of the reference
    M = gpu.Matrix.from_csr(3, 2, [0, 2, 4], [0, 1, 1, 2], [0.5, 0.3, 0.2, 1.0])
    y = gpu.apply_weights(M, np.array([2.0, 4.0, 6.0]))
    assert abs(y[0] - 2.2) < 1e-14 and abs(y[1] - 6.8) < 1e-14
    y = gpu.apply_weights(M, np.array([1.0, 1.0, 1.0]))
    assert abs(y[0] - 0.8) < 1e-14 and abs(y[1] - 1.2) < 1e-14
    with pytest.raises(gpu.InvalidArgument):
        gpu.apply_weights(M, np.ones(5))
    import ctypes
    dst = np.zeros(5)
    rc = gpu.lib().axgb_apply_c(M.handle, np.ones(3).ctypes.data_as(ctypes.c_void_p),
                                dst.ctypes.data_as(ctypes.c_void_p), 3, 5)
    assert rc == gpu.ERR_INVALID and np.all(dst == 0.0)
    out = gpu.batch_apply(M, np.array([[2.0, 1.0], [4.0, 1.0], [6.0, 1.0]]))
    assert np.allclose(out, [[2.2, 0.8], [6.8, 1.2]], atol=1e-14)


@pytest.fixture(scope="module")
def cfg1(gpu, oracle):
    src, dst = grids.latlon_deg(1.0), grids.cubed_sphere(48)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    xyz = grids.cell_centroids_xyz(src)
    f = fields.sh_field(xyz, 16, seed=1, offset=280.0).numpy()
    return src, dst, M, wo, f


def test_apply_f64_parity(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    x = torch.tensor(f, device="cuda")
    y = gpu.apply_weights(M, x).cpu().numpy()
    ref = oracle.apply_csr(wo, f, compensated=True)[0]
    assert np.max(np.abs(y - ref) / np.abs(ref)) < F64_RTOL
    yh = gpu.apply_weights(M, f)  # host path
    assert np.max(np.abs(yh - ref) / np.abs(ref)) < F64_RTOL


def test_apply_split_parity(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    rng = np.random.default_rng(3)
    X = np.stack([f * s for s in rng.lognormal(0, 1, 7)]).astype(np.float32)
    ref = oracle.apply_csr(wo, X.astype(np.float64), compensated=True)
    xs = torch.tensor(X, device="cuda")
    outs = []
    for v, fpp, u in ((0, 0, 1), (0, 0, 2), (0, 0, 4), (0, 3, 2), (0, 1, 1), (1, 0, 2), (1, 0, 4), (1, 0, 8),
                      (2, 0, 2), (2, 0, 4), (2, 0, 8), (3, 0, 4), (3, 2, 4), (4, 0, 1), (5, 0, 32)):
        y = gpu.apply_f32split(M, xs, fields_per_pass=fpp, unroll=u, variant=v).cpu().numpy()
        err = np.max(np.abs(y - ref) / np.abs(ref))
        assert err < SPLIT_RTOL, (v, fpp, u, err)
        outs.append(y)
    for y in outs[1:]:
        assert np.array_equal(y, outs[0])
    assert M.device_status() == 0
    # strided fields (ld > n)
    xp = torch.zeros((7, M.n_src + 37), dtype=torch.float32, device="cuda")
    xp[:, : M.n_src] = xs
    yp = torch.full((7, M.n_dst + 5), -1.0, dtype=torch.float32, device="cuda")
    gpu.apply_f32split(M, xp[:, : M.n_src], yp[:, : M.n_dst])
    assert np.array_equal(yp[:, : M.n_dst].cpu().numpy(), outs[0])
    assert np.all(yp[:, M.n_dst:].cpu().numpy() == -1.0)


def test_apply_split_host_path(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    X = np.stack([f, 2 * f, -f]).astype(np.float32)
    Y = np.zeros((3, M.n_dst), np.float32)
    gpu.batch_apply_host_f32split(M, X, Y)
    dev = gpu.apply_f32split(M, torch.tensor(X, device="cuda")).cpu().numpy()
    assert np.array_equal(Y, dev)


def test_autotune_and_batch(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    X = torch.tensor(np.stack([f] * 5).astype(np.float32), device="cuda")
    Y = torch.empty((5, M.n_dst), dtype=torch.float32, device="cuda")
    best = gpu.autotune_f32split(M, X, Y)
    assert best["variant"] in (0, 1, 2, 3, 4) and best["unroll"] in (1, 2, 4, 8)
    ref = gpu.apply_f32split(M, X, fields_per_pass=0, unroll=1).cpu().numpy()
    assert np.array_equal(gpu.apply_f32split(M, X).cpu().numpy(), ref)  # tuned choice, same bits
    # persistent multi-matrix batch: same matrix twice plus a reversed pair
    M2 = gpu.generate_weights(gpu.Mesh.from_grid(dst), gpu.Mesh.from_grid(src), {"method": "conservative"})
    x2 = torch.rand((3, M2.n_src), dtype=torch.float32, device="cuda")
    y2ref = gpu.apply_f32split(M2, x2, fields_per_pass=0, unroll=1).cpu().numpy()
    B = gpu.Batch([M, M2, M], [5, 3, 2])
    ya = torch.empty((5, M.n_dst), dtype=torch.float32, device="cuda")
    yb = torch.empty((3, M2.n_dst), dtype=torch.float32, device="cuda")
    yc = torch.empty((2, M.n_dst), dtype=torch.float32, device="cuda")
    for _ in range(2):  # second call replays the captured graph
        B.apply([X, x2, X[:2]], [ya, yb, yc])
        torch.cuda.synchronize()
        assert np.array_equal(ya.cpu().numpy(), ref)
        assert np.array_equal(yb.cpu().numpy(), y2ref)
        assert np.array_equal(yc.cpu().numpy(), ref[:2])


def test_conservation_parity(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    x = torch.tensor(f, device="cuda")
    y = gpu.apply_weights(M, x)
    rep = gpu.check_conservation(M, x, y)
    ro = oracle.conservation(wo, f, oracle.apply_csr(wo, f)[0])
    assert abs(rep["src_integral"] - ro["src_integral"]) / abs(ro["src_integral"]) < 1e-13
    assert rep["relative_error"] < 1e-12


def test_kernel_choice_seed_and_read(gpu, oracle, cfg1):
    import torch
    src, dst, M, wo, f = cfg1
    nrhs = 6
    assert gpu.get_kernel_choice(M, nrhs)["cached"] is False
    gpu.set_kernel_choice(M, nrhs, variant=1, fields_per_pass=4, unroll=2, stages=3)
    ch = gpu.get_kernel_choice(M, nrhs)
    assert ch == dict(variant=1, fields_per_pass=4, unroll=2, stages=3, cached=True)
    X = torch.tensor(np.stack([f * (1 + k) for k in range(nrhs)]).astype(np.float32), device="cuda")
    y = gpu.apply_f32split(M, X).cpu().numpy().astype(np.float64)
    ref = oracle.apply_csr(wo, X.cpu().numpy().astype(np.float64), compensated=True)
    assert np.max(np.abs(y - ref) / np.abs(ref)) < SPLIT_RTOL
    with pytest.raises(gpu.InvalidArgument):
        gpu.set_kernel_choice(M, nrhs, variant=2, fields_per_pass=0, unroll=4, stages=3)
    with pytest.raises(gpu.InvalidArgument):
        gpu.set_kernel_choice(M, nrhs, variant=6, fields_per_pass=0, unroll=4, stages=2)
    with pytest.raises(gpu.InvalidArgument):
        gpu.set_kernel_choice(M, nrhs, variant=3, fields_per_pass=0, unroll=4, stages=4)
    with pytest.raises(gpu.InvalidArgument):
        gpu.set_kernel_choice(M, nrhs, variant=3, fields_per_pass=0, unroll=8, stages=3)
    with pytest.raises(gpu.InvalidArgument):  # per-class ring depth is variant 3's only
        gpu.set_kernel_choice(M, nrhs, variant=1, fields_per_pass=0, unroll=4, stages=0)
    # producer-warp ring (2, 3 slots, or per row-length class), fused single launch
    for v, ns in ((3, 2), (3, 3), (3, 0), (4, 2)):
        gpu.set_kernel_choice(M, nrhs, variant=v, fields_per_pass=0, unroll=4, stages=ns)
        assert np.array_equal(gpu.apply_f32split(M, X).cpu().numpy().astype(np.float64), y)


def test_long_rows_parity(gpu, oracle):
    """Coarse destination over a fine source (rows of 50-90 entries): the
    warp-per-row kernels agree bitwise with every other split kernel and the
    batch, and meet the FP64 / split tolerances."""
    import torch
    src, dst = grids.latlon_deg(0.5), grids.cubed_sphere(24)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    _check_weights(M, wo)
    assert np.diff(wo.row_ptr()).max() > 32
    rng = np.random.default_rng(5)
    X = rng.standard_normal((37, M.n_src)).astype(np.float32)
    ref = oracle.apply_csr(wo, X.astype(np.float64), compensated=True)
    xs = torch.tensor(X, device="cuda")
    outs = [gpu.apply_f32split(M, xs, fields_per_pass=fpp, unroll=u, variant=v).cpu().numpy()
            for v, fpp, u in ((0, 0, 1), (0, 8, 4), (1, 0, 4), (1, 16, 8), (2, 0, 4), (3, 0, 4), (4, 0, 1),
                              (5, 0, 32))]
    for y in outs[1:]:
        assert np.array_equal(y, outs[0])
    scale = np.abs(ref).max()
    assert np.max(np.abs(outs[0] - ref)) / scale < 1e-6
    y64 = gpu.apply_f64(M, xs.to(torch.float64)).cpu().numpy()
    assert np.max(np.abs(y64 - ref)) / scale < 1e-13
    # one and two fields take the fused FP64 launch: the same bits per field
    for k in (1, 2):
        assert np.array_equal(gpu.apply_f64(M, xs[:k].to(torch.float64)).cpu().numpy(), y64[:k])
    B = gpu.Batch([M], [37])
    yb = torch.empty((37, M.n_dst), dtype=torch.float32, device="cuda")
    for _ in range(2):
        B.apply([xs], [yb])
        torch.cuda.synchronize()
        assert np.array_equal(yb.cpu().numpy(), outs[0])


COND_PAIRS = [
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("0.5deg->C24", lambda: (grids.latlon_deg(0.5), grids.cubed_sphere(24))),  # rows of 50-90 entries
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),
]


@pytest.mark.parametrize("name,make", COND_PAIRS)
def test_apply_condition_bound_zero_mean(gpu, oracle, name, make):
    """Per-output error bound scaled by each output's condition: with
    c_i = sum_j |w_ij x_j|, the FP64 apply satisfies |y_i - y_ref_i| <=
    1e-13 c_i and the split-FP32 apply |y_i - y_ref_i| <= 1e-6 c_i, on
    zero-mean spherical-harmonic fields (no offset), whose outputs cross
    zero, so a bound relative to |y_ref_i| alone would not hold there.
    y_ref is the compensated FP64 oracle on the same (FP32-rounded) inputs."""
    import torch
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    xyz = grids.cell_centroids_xyz(src)
    rng = np.random.default_rng(11)
    base = fields.sh_fields(xyz, 32, [21, 22, 23]).numpy()
    X = np.concatenate([base * s for s in rng.lognormal(0, 1, 3)]).astype(np.float32).astype(np.float64)
    ref = oracle.apply_csr(wo, X, compensated=True)
    cond = oracle.apply_csr(wo, np.abs(X), compensated=True)  # conservative weights are >= 0
    assert np.all(wo.w >= 0)
    assert (ref < 0).any() and (ref > 0).any()  # outputs cross zero
    xd = torch.tensor(X, device="cuda")
    y64 = gpu.apply_f64(M, xd).cpu().numpy()
    r64 = np.abs(y64 - ref) / np.maximum(cond, 1e-300)
    assert r64.max() <= F64_RTOL, r64.max()
    ys = gpu.apply_f32split(M, xd.to(torch.float32)).cpu().numpy()
    rs = np.abs(ys - ref) / np.maximum(cond, 1e-300)
    assert rs.max() <= SPLIT_RTOL, rs.max()


HILO_PAIRS = [
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("0.5deg->C24", lambda: (grids.latlon_deg(0.5), grids.cubed_sphere(24))),  # long rows
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),  # renumbered source
]


@pytest.mark.parametrize("name,make", HILO_PAIRS)
def test_apply_split_hilo(gpu, oracle, name, make):
    """hi+lo output form: y is bitwise the plain split apply's result under
    every kernel variant; y + y_lo (summed in FP64) is within 1e-13 of the
    compensated FP64 oracle relative to c_i = sum_j |w_ij x_j|, on zero-mean
    fields; and the destination integral of the conservation report
    (conservation.cpp:83-96) equals the one of the oracle's compensated apply
    within 1e-13 of the integral of c (its condition)."""
    import torch
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    xyz = grids.cell_centroids_xyz(src)
    rng = np.random.default_rng(12)
    base = fields.sh_fields(xyz, 24, [31, 32]).numpy()
    X = np.concatenate([base * s for s in rng.lognormal(0, 1, 4)]).astype(np.float32)
    nrhs = X.shape[0]
    X64 = X.astype(np.float64)
    ref = oracle.apply_csr(wo, X64, compensated=True)
    cond = oracle.apply_csr(wo, np.abs(X64), compensated=True)
    xd = torch.tensor(X, device="cuda")
    plain = gpu.apply_f32split(M, xd, fields_per_pass=0, unroll=1, variant=0).cpu().numpy()
    for v, fpp, u, ns in ((0, 0, 2, 2), (0, 3, 4, 2), (1, 0, 4, 2), (1, 4, 8, 3), (3, 0, 4, 3), (5, 0, 32, 2),
                          (5, 0, 32, 3)):
        gpu.set_kernel_choice(M, nrhs, variant=v, fields_per_pass=fpp, unroll=u, stages=ns)
        y, ylo = gpu.apply_f32split_hilo(M, xd)
        y, ylo = y.cpu().numpy(), ylo.cpu().numpy()
        assert np.array_equal(y, plain), (v, fpp, u)
        hl = y.astype(np.float64) + ylo.astype(np.float64)
        err = np.abs(hl - ref) / np.maximum(cond, 1e-300)
        assert err.max() <= 1e-13, (v, fpp, u, err.max())
    assert M.device_status() == 0
    hl_d = torch.tensor(hl, device="cuda")
    for k in range(nrhs):
        rep = gpu.check_conservation(M, xd[k].to(torch.float64), hl_d[k])
        ro = oracle.conservation(wo, X64[k], ref[k])
        scale = float(np.sum(wo.area_b * cond[k]))
        assert abs(rep["dst_integral"] - ro["dst_integral"]) <= 1e-13 * scale, (k, rep, ro)
    with pytest.raises(gpu.InvalidArgument):
        gpu.apply_f32split_hilo(M, xd, y_lo=torch.empty((nrhs, M.n_dst - 1), dtype=torch.float32, device="cuda"))


def test_batch_on_two_streams(gpu, oracle, cfg1):
    """One batch applied alternately on two streams, with different fields on
    each: the second stream's call waits for the first's work on the GPU
    (the batch's work counters and descriptors are shared), so both outputs
    equal the per-call path bit for bit."""
    import torch
    src, dst, M, wo, f = cfg1
    rng = np.random.default_rng(17)
    Xa = torch.tensor(np.stack([f * s for s in rng.lognormal(0, 1, 6)]).astype(np.float32), device="cuda")
    Xb = torch.tensor(np.stack([-f * s for s in rng.lognormal(0, 1, 6)]).astype(np.float32), device="cuda")
    ra = gpu.apply_f32split(M, Xa, fields_per_pass=0, unroll=1).cpu().numpy()
    rb = gpu.apply_f32split(M, Xb, fields_per_pass=0, unroll=1).cpu().numpy()
    B = gpu.Batch([M], [6])
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    ya = torch.empty((6, M.n_dst), dtype=torch.float32, device="cuda")
    yb = torch.empty((6, M.n_dst), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    for _ in range(3):
        B.apply([Xa], [ya], stream=s1)
        B.apply([Xb], [yb], stream=s2)
    torch.cuda.synchronize()
    assert np.array_equal(ya.cpu().numpy(), ra)
    assert np.array_equal(yb.cpu().numpy(), rb)


SEG_PAIRS = [
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("0.5deg->C24 (long rows)", lambda: (grids.latlon_deg(0.5), grids.cubed_sphere(24))),
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),
    ("0.25deg->C12 (oversize groups)", lambda: (grids.latlon_deg(0.25), grids.cubed_sphere(12))),
]


@pytest.mark.parametrize("name,make", SEG_PAIRS)
def test_segmented_variant(gpu, oracle, name, make):
    """Variant 5 (segmented, lane = field, source cells staged by their own
    ids) against the direct kernel bit for bit, for field counts that fill
    and that do not fill a 32-field tile, from unaligned field starts (an
    odd leading dimension), with and without the hi+lo output; and within
    the split tolerance of the compensated FP64 oracle."""
    import torch
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    rng = np.random.default_rng(41)
    nrhs = 45
    X = rng.standard_normal((nrhs, M.n_src)).astype(np.float32)
    ld = M.n_src + 3
    xp = torch.zeros((nrhs, ld), dtype=torch.float32, device="cuda")
    xp[:, :M.n_src] = torch.tensor(X, device="cuda")
    xs = xp[:, :M.n_src]
    ref = gpu.apply_f32split(M, xs.contiguous(), fields_per_pass=0, unroll=1, variant=0).cpu().numpy()
    for k in (nrhs, 32, 7):
        gpu.set_kernel_choice(M, k, variant=0, fields_per_pass=0, unroll=1, stages=2)
        lo_ref = gpu.apply_f32split_hilo(M, xs[:k].contiguous())[1].cpu().numpy()
        for ns in (2, 3):
            gpu.set_kernel_choice(M, k, variant=5, fields_per_pass=0, unroll=32, stages=ns)
            y = gpu.apply_f32split(M, xs[:k]).cpu().numpy()
            assert np.array_equal(y, ref[:k]), (k, ns, int(np.sum(y != ref[:k])))
            yh, yl = gpu.apply_f32split_hilo(M, xs[:k])
            assert np.array_equal(yh.cpu().numpy(), ref[:k])
            assert np.array_equal(yl.cpu().numpy(), lo_ref)
    assert M.device_status() == 0
    oref = oracle.apply_csr(wo, X.astype(np.float64), compensated=True)
    cond = oracle.apply_csr(wo, np.abs(X.astype(np.float64)), compensated=True)
    assert np.max(np.abs(ref - oref) / np.maximum(cond, 1e-300)) <= SPLIT_RTOL


def test_one_dimensional_fields(gpu, oracle, cfg1):
    """1-D x and y (one field) through the device entry points."""
    import torch
    src, dst, M, wo, f = cfg1
    x = torch.tensor(f, device="cuda")
    y = torch.empty(M.n_dst, dtype=torch.float64, device="cuda")
    gpu.apply_f64(M, x, y)
    ref = oracle.apply_csr(wo, f, compensated=True)[0]
    assert np.max(np.abs(y.cpu().numpy() - ref) / np.abs(ref)) < F64_RTOL
    y32 = torch.empty(M.n_dst, dtype=torch.float32, device="cuda")
    gpu.apply_f32split(M, x.to(torch.float32), y32)
    assert np.max(np.abs(y32.cpu().numpy() - ref) / np.abs(ref)) < SPLIT_RTOL


def test_very_long_rows_few_fields(gpu, oracle):
    """Polar destination cells over a lat-lon source: rows of hundreds of
    entries. One, three and forty fields (warp-per-row and lane-per-field
    forms of the long-row order) give the same bits per field, and match
    the oracle."""
    import torch
    src, dst = grids.latlon_deg(1.0), grids.cubed_sphere(6)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    assert np.diff(wo.row_ptr()).max() > 200
    rng = np.random.default_rng(9)
    X = (rng.standard_normal((40, M.n_src)) + 3.0).astype(np.float32)
    ref = oracle.apply_csr(wo, X.astype(np.float64), compensated=True)
    xs = torch.tensor(X, device="cuda")
    y40 = gpu.apply_f32split(M, xs).cpu().numpy()
    y1 = gpu.apply_f32split(M, xs[:1]).cpu().numpy()
    y3 = gpu.apply_f32split(M, xs[:3], variant=0, unroll=1, fields_per_pass=0).cpu().numpy()
    assert np.array_equal(y1, y40[:1]) and np.array_equal(y3, y40[:3])
    assert np.max(np.abs(y40 - ref) / np.abs(ref)) < SPLIT_RTOL
    d40 = gpu.apply_f64(M, xs.to(torch.float64)).cpu().numpy()
    d1 = gpu.apply_f64(M, xs[:1].to(torch.float64)).cpu().numpy()
    assert np.array_equal(d1, d40[:1])
    assert np.max(np.abs(d40 - ref) / np.abs(ref)) < F64_RTOL
    B = gpu.Batch([M, M], [2, 40])
    yb2 = torch.empty((2, M.n_dst), dtype=torch.float32, device="cuda")
    yb40 = torch.empty((40, M.n_dst), dtype=torch.float32, device="cuda")
    B.apply([xs[:2], xs], [yb2, yb40])
    torch.cuda.synchronize()
    assert np.array_equal(yb2.cpu().numpy(), y40[:2]) and np.array_equal(yb40.cpu().numpy(), y40)


def test_staged_kernels_partial_last_chunk(gpu, oracle):
    """n_src not a multiple of 4 (a Voronoi source): with a padded leading
    dimension the staged kernels run, the last source chunk is copied in
    part and zero-filled; results agree bitwise with the direct kernel and
    with the batch."""
    import torch
    src, dst = grids.voronoi(40962, seed=5), grids.latlon_deg(0.5)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    assert M.n_src % 4 == 2
    wo = oracle.conservative(src, dst)
    rng = np.random.default_rng(11)
    X = (rng.standard_normal((9, M.n_src)) + 2.0).astype(np.float32)
    ref = oracle.apply_csr(wo, X.astype(np.float64), compensated=True)
    ld = (M.n_src + 3) // 4 * 4
    buf = torch.zeros((9, ld), dtype=torch.float32, device="cuda")
    buf[:, : M.n_src] = torch.tensor(X, device="cuda")
    xs = buf[:, : M.n_src]
    y1 = gpu.apply_f32split(M, xs, fields_per_pass=0, unroll=4, variant=1).cpu().numpy()
    y0 = gpu.apply_f32split(M, xs, fields_per_pass=0, unroll=1, variant=0).cpu().numpy()
    assert np.array_equal(y1, y0)
    # a Voronoi mesh numbers its cells along a spiral: a 128-row strip of the
    # 0.5 deg grid touches every few cells of a latitude band
    assert M.stats()["source_renumbered"]
    assert np.max(np.abs(y1 - ref) / np.abs(ref)) < SPLIT_RTOL
    B = gpu.Batch([M], [9])
    yb = torch.empty((9, M.n_dst), dtype=torch.float32, device="cuda")
    B.apply([xs], [yb])
    torch.cuda.synchronize()
    assert np.array_equal(yb.cpu().numpy(), y1)


def _oracle_weights_of(M):
    """The GPU's own CSR as oracle weights (the two generators agree to an
    ulp on a few weights, where CUDA's and glibc's atan2 differ)."""
    from oracle import Weights
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    return Weights(M.n_src, M.n_dst, rows.astype(np.int64), csr["col"].astype(np.int64), csr["val"], csr["frac_a"],
                   csr["frac_b"], csr["area_a"], csr["area_b"])


def test_nan_batch_apply_parity(gpu, oracle):
    """NaN-aware batched apply on the GPU against the oracle on the same
    weights: NaN positions and values bit for bit (device and host entry
    points)."""
    import torch
    src, dst = grids.latlon_deg(2.0), grids.cubed_sphere(24)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = _oracle_weights_of(M)
    rng = np.random.default_rng(17)
    X = rng.standard_normal((6, M.n_src)) + 280.0
    for v, p in enumerate((0.0, 0.05, 0.3, 0.6, 0.9, 1.0)):
        X[v, rng.uniform(size=M.n_src) < p] = np.nan
    for thres in (0.0, 0.25, 0.5, 1.0):
        ref = oracle.nan_batch_apply(wo, X, thres)
        got = gpu.nan_apply_f64(M, torch.tensor(X, device="cuda"), thres).cpu().numpy()
        np.testing.assert_array_equal(got, ref)
        host = gpu.nan_batch_apply(M, X.T, thres)  # [n_src, n_vars] like axis_py.nan_batch_apply
        np.testing.assert_array_equal(host, ref.T)


def test_apply_masked_parity(gpu, oracle):
    import torch
    src, dst = grids.latlon_deg(2.0), grids.cubed_sphere(24)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = _oracle_weights_of(M)
    x = np.random.default_rng(19).standard_normal(M.n_src) + 280.0
    mask = (np.arange(M.n_dst) % 5 != 1).astype(np.int32)
    y0 = np.full(M.n_dst, -3.0)
    ref = oracle.apply_masked(wo, x, mask, y0)
    y = torch.tensor(y0, device="cuda")
    gpu.apply_masked(M, torch.tensor(x, device="cuda"), y, torch.tensor(mask, device="cuda"))
    np.testing.assert_array_equal(y.cpu().numpy(), ref)
    y2 = torch.tensor(y0, device="cuda")
    gpu.apply_masked(M, torch.tensor(x, device="cuda"), y2)  # no mask: every row
    full = oracle.apply_masked(wo, x, np.ones(M.n_dst, np.int32), y0)
    np.testing.assert_array_equal(y2.cpu().numpy(), full)


def _read_blob(blob):
    """Independent reader of the weight cache layout (weight_cache.hpp:14-26)."""
    import struct
    magic, version, endian = struct.unpack_from("<IIB", blob, 0)
    ns, nd, nz = struct.unpack_from("<QQQ", blob, 16)
    off = 40
    arrs = {}
    for name, n, dt in (("w", nz, "<f8"), ("row", nz, "<i8"), ("col", nz, "<i8"), ("frac_a", ns, "<f8"),
                        ("frac_b", nd, "<f8"), ("area_a", ns, "<f8"), ("area_b", nd, "<f8")):
        arrs[name] = np.frombuffer(blob, dtype=dt, count=n, offset=off)
        off += 8 * n
    return magic, version, endian, ns, nd, nz, off, arrs


def test_weight_cache_round_trip(gpu, oracle):
    """WeightCache blob: layout read back independently, deserialize
    reproduces the CSR bit for bit (the reference's round-trip property),
    triplets in any order accepted, and bad magic / version / truncation
    rejected (prop_weight_cache.cpp)."""
    import torch
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    blob = M.serialize()
    magic, version, endian, ns, nd, nz, size, a = _read_blob(blob)
    # the reference's magic value 0x43574841 (its comment calls it "AXWC"; the
    # little-endian bytes of the value are b"AHWC")
    assert (magic, version, endian) == (0x43574841, 1, 1) and blob[:4] == b"AHWC"
    assert (ns, nd, nz) == (M.n_src, M.n_dst, M.nnz) and size == len(blob)
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    assert np.array_equal(a["row"], rows) and np.array_equal(a["col"], csr["col"]) and np.array_equal(a["w"], csr["val"])
    M2 = gpu.Matrix.deserialize(blob)
    csr2 = M2.to_csr()
    for k in csr:
        assert np.array_equal(csr[k], csr2[k]), k
    x = torch.tensor(np.random.default_rng(2).standard_normal(M.n_src), device="cuda")
    assert torch.equal(gpu.apply_f64(M, x), gpu.apply_f64(M2, x))
    # triplets shuffled: the same matrix
    perm = np.random.default_rng(3).permutation(nz)
    b = bytearray(blob)
    for name, off in (("w", 40), ("row", 40 + 8 * nz), ("col", 40 + 16 * nz)):
        b[off:off + 8 * nz] = a[name][perm].tobytes()
    csr3 = gpu.Matrix.deserialize(bytes(b)).to_csr()
    for k in csr:
        assert np.array_equal(csr[k], csr3[k]), k
    # rejections
    for bad in (b"XXXX" + blob[4:], blob[:4] + (2).to_bytes(4, "little") + blob[8:], blob[:41], blob[:20]):
        with pytest.raises(gpu.InvalidArgument):
            gpu.Matrix.deserialize(bad)


REGULAR_PAIRS = [
    ("1deg->2deg", lambda: (grids.latlon_deg(1.0), grids.latlon_deg(2.0))),
    ("2deg->1deg", lambda: (grids.latlon_deg(2.0), grids.latlon_deg(1.0))),
    ("0.5deg->0.75deg", lambda: (grids.latlon_deg(0.5), grids.latlon_deg(0.75))),
    ("regional 1deg->global 2deg", lambda: (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0), grids.latlon_deg(2.0))),
    ("shifted global", lambda: (grids.regular_latlon(360, 180, -180.0, -90.0, 1.0, 1.0), grids.latlon_deg(3.0))),
]


@pytest.mark.parametrize("name,make", REGULAR_PAIRS)
def test_conservative_regular_fast_path(gpu, oracle, name, make):
    """Regular x regular conservative weights (the analytic fast path of
    weight_generator_conservative_rect.cpp) against the oracle's restatement:
    the index set bit-exact, values within 1e-12."""
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    wo = oracle.conservative(src, dst)
    _check_weights(M, wo)
    Mf = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst),
                              {"method": "conservative", "norm_type": "FracArea"})
    _check_weights(Mf, oracle.conservative(src, dst, norm_type=1))


def _land_mask(src):
    c = grids.cell_centroids_xyz(src)
    lat = np.degrees(np.arcsin(c[:, 2]))
    lon = np.degrees(np.arctan2(c[:, 1], c[:, 0])) % 360
    return (~((lat > -30) & (lat < 40) & (lon > 20) & (lon < 110))).astype(np.int32)


@pytest.mark.parametrize("name,make", [
    ("5deg->C8", lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8))),
    ("C24->2deg", lambda: (grids.cubed_sphere(24), grids.latlon_deg(2.0))),
])
def test_coastal_postpass_parity(gpu, oracle, name, make):
    """A masked source: generate_weights applies the coastal post-pass (wet
    renormalisation, NearestWet extrapolation) as the reference's generate()
    does; against the oracle on the same kept pairs."""
    src, dst = make()
    mask = _land_mask(src)
    ms = gpu.Mesh.from_arrays(src.node_lonlat, src.conn_offsets, src.conn_indices, mask=mask)
    md = gpu.Mesh.from_grid(dst)
    wo = oracle.conservative(src, dst, src_mask=mask)
    for extrap, nearest in (("nearest_wet", True), ("none", False)):
        M = gpu.generate_weights(ms, md, {"method": "conservative", "extrap_method": extrap})
        ref = oracle.coastal(wo, src, dst, mask, nearest_wet=nearest)
        _check_weights(M, ref)


@pytest.mark.parametrize("name,make", [
    ("C12->10deg", lambda: (grids.cubed_sphere(12), grids.latlon_deg(10.0))),
    ("C24->3deg", lambda: (grids.cubed_sphere(24), grids.latlon_deg(3.0))),
    ("5deg->shifted 2.5deg (periodic wrap)", lambda: (grids.latlon_deg(5.0),
                                                     grids.regular_latlon(144, 72, -1.0, -90.0, 2.5, 2.5))),
])
def test_coastal_sums_in_generation_order(gpu, oracle, name, make):
    """Masked bilinear weights bit for bit: the coastal pass divides each row
    by the sum of its wet weights, and the reference sums them in the order
    the generator emitted them (quad / triangle corner order on the general
    path, corner order on the regular path, where a periodic wrap puts
    column 0 after the last column), not in column order
    (weight_generator.cpp:1769-1777). The bilinear weights themselves are
    bit-exact, so every bit of the renormalised weights must match."""
    src, dst = make()
    mask = (np.random.default_rng(3).uniform(size=src.n_cells) > 0.3).astype(np.int32)
    ms = gpu.Mesh.from_arrays(src.node_lonlat, src.conn_offsets, src.conn_indices, mask=mask)
    md = gpu.Mesh.from_grid(dst)
    wo = oracle.bilinear(src, dst)
    for extrap, nearest in (("nearest_wet", True), ("none", False)):
        csr = gpu.generate_weights(ms, md, {"method": "bilinear", "extrap_method": extrap}).to_csr()
        ref = oracle.coastal(wo, src, dst, mask, nearest_wet=nearest)
        rows = _rows(csr, dst.n_cells)
        assert np.array_equal(rows, ref.row) and np.array_equal(csr["col"], ref.col)
        assert np.array_equal(csr["val"], ref.w), int(np.sum(csr["val"] != ref.w))


RECT_PAIRS = [
    ("equal-area stretched->2deg", lambda: (grids.equal_area_latlon(72, 36, stretch=0.4), grids.latlon_deg(2.0))),
    ("1deg->shifted equal-area", lambda: (grids.latlon_deg(1.0),
                                          grids.equal_area_latlon(96, 48, lon_start=-180.0, stretch=0.3))),
    ("equal-area->equal-area", lambda: (grids.equal_area_latlon(180, 90, stretch=0.2),
                                        grids.equal_area_latlon(50, 28, lon_start=-90.0, stretch=0.5))),
    ("declined regular pair", lambda: (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0),
                                       grids.regular_latlon(20, 20, 10.0, -20.0, 2.0, 2.0))),
]


@pytest.mark.parametrize("name,make", RECT_PAIRS)
def test_conservative_rectilinear_fast_path(gpu, oracle, name, make):
    """Rectilinear x rectilinear conservative weights (the non-uniform fast
    path, which also takes regular pairs the regular path declines) against
    the oracle: index set bit-exact, values within 1e-12, DstArea and
    FracArea."""
    src, dst = make()
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    _check_weights(gpu.generate_weights(ms, md, {"method": "conservative"}), oracle.conservative(src, dst))
    _check_weights(gpu.generate_weights(ms, md, {"method": "conservative", "norm_type": "FracArea"}),
                   oracle.conservative(src, dst, norm_type=1))


def test_fast_paths_return_partial_coverage_under_error(gpu, oracle):
    """The fast paths return their matrix as it is under UnmappedAction::Error
    when some rows are empty but not all: a regional source on a global
    destination raises nothing and matches the oracle."""
    src, dst = grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0), grids.latlon_deg(2.0)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst),
                             {"method": "conservative", "unmapped": "Error"})
    _check_weights(M, oracle.conservative(src, dst, unmapped=0))
    src = grids.equal_area_latlon(36, 18, stretch=0.3)
    dst = grids.rectilinear([0.0, 5.0, 12.0, 30.0], [-10.0, 0.0, 7.5])
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst),
                             {"method": "conservative", "unmapped": "Error"})
    _check_weights(M, oracle.conservative(src, dst, unmapped=0))


BILINEAR_REGULAR_PAIRS = [
    ("10deg->20deg", lambda: (grids.latlon_deg(10.0), grids.latlon_deg(20.0))),
    ("1deg->0.75deg", lambda: (grids.latlon_deg(1.0), grids.latlon_deg(0.75))),
    ("1deg->shifted 2deg", lambda: (grids.latlon_deg(1.0), grids.regular_latlon(180, 90, -180.0, -90.0, 2.0, 2.0))),
    ("regional->global", lambda: (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0), grids.latlon_deg(2.0))),
]


@pytest.mark.parametrize("name,make", BILINEAR_REGULAR_PAIRS)
def test_bilinear_regular_fast_path(gpu, oracle, name, make):
    """Regular x regular bilinear (weight_generator_bilinear_rect.cpp) against
    the oracle, bit for bit: index arithmetic and four products per row. A
    regional source leaves rows unmapped: empty under Ignore, an error under
    Error, on both sides."""
    src, dst = make()
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    M = gpu.generate_weights(ms, md, {"method": "bilinear"})
    wo = oracle.bilinear(src, dst)
    csr = _check_weights(M, wo)
    assert np.array_equal(csr["val"], wo.w)
    if name == "regional->global":
        assert wo.nnz < 4 * dst.n_cells
        with pytest.raises(gpu.AxgbError) as e:
            gpu.generate_weights(ms, md, {"method": "bilinear", "unmapped": "Error"})
        assert e.value.code == gpu.ERR_UNMAPPED
        with pytest.raises(RuntimeError):
            oracle.bilinear(src, dst, unmapped=0)
    else:
        assert wo.nnz == 4 * dst.n_cells


def test_esmf_weight_file_round_trip(gpu, oracle, tmp_path):
    """ESMF weight file of a generated matrix: scipy's NetCDF-3 reader sees S,
    1-based col_idx / row_idx in CSR order and n_a / n_b; read_esmf rebuilds
    the CSR bit for bit with frac and area arrays zero (as the reference's
    read_esmf leaves them); a shuffled file gives the same matrix."""
    import torch
    netcdf = pytest.importorskip("scipy.io").netcdf_file
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    csr = M.to_csr()
    p = tmp_path / "w.nc"
    M.write_esmf(p)
    f = netcdf(str(p), "r", mmap=False)
    try:
        assert (int(f.n_a), int(f.n_b)) == (M.n_src, M.n_dst)
        rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
        assert np.array_equal(f.variables["row_idx"][:], rows + 1)
        assert np.array_equal(f.variables["col_idx"][:], csr["col"] + 1)
        assert np.array_equal(f.variables["S"][:], csr["val"])
    finally:
        f.close()
    M2 = gpu.Matrix.read_esmf(p)
    csr2 = M2.to_csr()
    for k in ("row_ptr", "col", "val"):
        assert np.array_equal(csr[k], csr2[k]), k
    for k in ("frac_a", "frac_b", "area_a", "area_b"):
        assert not np.any(csr2[k]), k
    x = torch.tensor(np.random.default_rng(2).standard_normal(M.n_src), device="cuda")
    assert torch.equal(gpu.apply_f64(M, x), gpu.apply_f64(M2, x))
    w = gpu.esmf_read(p)
    perm = np.random.default_rng(4).permutation(w["S"].size)
    q = tmp_path / "shuffled.nc"
    gpu.esmf_write(q, w["n_a"], w["n_b"], w["S"][perm], w["col_idx"][perm], w["row_idx"][perm])
    csr3 = gpu.Matrix.read_esmf(q).to_csr()
    for k in ("row_ptr", "col", "val"):
        assert np.array_equal(csr[k], csr3[k]), k


NEAREST_PAIRS = [
    ("1deg->C48", lambda: (grids.latlon_deg(1.0), grids.cubed_sphere(48))),
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("C12->C8", lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8))),
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),
    ("regional 1deg->C24 (far queries)", lambda: (grids.regular_latlon(40, 30, 20.0, -10.0, 1.0, 1.0),
                                                  grids.cubed_sphere(24))),
    ("2deg->1deg (regular)", lambda: (grids.latlon_deg(2.0), grids.latlon_deg(1.0))),
    ("1deg->shifted 3deg (regular)", lambda: (grids.latlon_deg(1.0),
                                              grids.regular_latlon(120, 60, -180.0, -90.0, 3.0, 3.0))),
]


@pytest.mark.parametrize("name,make", NEAREST_PAIRS)
def test_nearest_neighbor_parity(gpu, oracle, name, make):
    """Nearest-neighbour weights (generate_nearest: index rounding for two
    regular grids, else the exact float nearest centroid) against the oracle:
    every (dst, src) pair identical, weights, fractions and areas as well."""
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "nearest_neighbor"})
    wo = oracle.nearest(src, dst)
    csr = _check_weights(M, wo)
    assert np.array_equal(csr["val"], wo.w)


def test_nearest_neighbor_masked_source(gpu, oracle):
    """A masked source: the nearest-neighbour matrix goes through the coastal
    post-pass like every method's (generate(), weight_generator.cpp:2014)."""
    src, dst = grids.latlon_deg(5.0), grids.cubed_sphere(8)
    mask = _land_mask(src)
    ms = gpu.Mesh.from_arrays(src.node_lonlat, src.conn_offsets, src.conn_indices, mask=mask)
    M = gpu.generate_weights(ms, gpu.Mesh.from_grid(dst), {"method": "nearest_neighbor"})
    _check_weights(M, oracle.coastal(oracle.nearest(src, dst), src, dst, mask))


PROPERTY_PAIRS = PAIRS[:5] + REGULAR_PAIRS[:3] + RECT_PAIRS[:3]


@pytest.mark.parametrize("name,make", PROPERTY_PAIRS)
def test_weight_properties(gpu, name, make):
    """prop_conservative_nonneg.cpp / prop_grid_combinations.cpp /
    prop_csr_format.cpp: weights >= 0, indices in range, row sums <= 1 + 1e-9,
    row_ptr monotone from 0 to nnz, columns strictly ascending in each row."""
    src, dst = make()
    csr = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"}).to_csr()
    rp, col, val = csr["row_ptr"], csr["col"], csr["val"]
    assert rp[0] == 0 and rp[-1] == val.size and np.all(np.diff(rp) >= 0)
    assert np.all(val >= 0.0)
    assert np.all((col >= 0) & (col < src.n_cells))
    rows = np.repeat(np.arange(dst.n_cells), np.diff(rp))
    same_row = rows[1:] == rows[:-1]
    assert np.all(col[1:][same_row] > col[:-1][same_row])
    rs = np.bincount(rows, weights=val, minlength=dst.n_cells)
    assert rs.max() <= 1.0 + 1e-9


@pytest.mark.parametrize("direction", ["C96->1deg", "1deg->C96"])
def test_constant_field_c96(gpu, direction):
    """test_c96_benchmarks.py:60-104: a constant field regrids to 1 within
    1e-12 (FP64 apply, DstArea and FracArea, great circles); the split-FP32
    apply within 1e-6."""
    import torch
    a, b = grids.cubed_sphere(96), grids.latlon_deg(1.0)
    src, dst = (a, b) if direction == "C96->1deg" else (b, a)
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    for norm in ("DstArea", "FracArea"):
        M = gpu.generate_weights(ms, md, {"method": "conservative", "norm_type": norm})
        y = gpu.apply_weights(M, np.ones(src.n_cells))
        assert np.abs(y - 1.0).max() < 1e-12, (norm, np.abs(y - 1.0).max())
        x32 = torch.ones((4, src.n_cells), dtype=torch.float32, device="cuda")
        y32 = gpu.apply_f32split(M, x32).cpu().numpy()
        assert np.abs(y32 - 1.0).max() < 1e-6


@pytest.mark.parametrize("method,budget", [("bilinear", 0.250), ("nearest_neighbor", 0.350),
                                           ("conservative", 0.400)])
def test_performance_budgets(gpu, method, budget):
    """test_axis_performance.py:47-110: 360 x 180 cells to 720 x 360 cells,
    weight generation within the reference's per-method budget and the apply
    of one field (host arrays in and out) within 80 ms."""
    import time
    src, dst = grids.latlon_deg(1.0), grids.latlon_deg(0.5)
    warm = gpu.generate_weights(gpu.Mesh.from_grid(grids.latlon_deg(30.0)), gpu.Mesh.from_grid(grids.latlon_deg(20.0)),
                                {"method": method})
    gpu.apply_weights(warm, np.ones(warm.n_src))
    ms, md = gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst)
    t0 = time.perf_counter()
    M = gpu.generate_weights(ms, md, {"method": method})
    gen = time.perf_counter() - t0
    field = grids.cell_centroids_xyz(src)[:, 0]  # cos(lat) cos(lon), the reference test's field
    t0 = time.perf_counter()
    y = gpu.apply_weights(M, field)
    app = time.perf_counter() - t0
    assert gen < budget, gen
    assert app < 0.080, app
    assert y.shape == (dst.n_cells,) and np.all(np.isfinite(y))


BILINEAR_GENERAL_PAIRS = [
    ("C24->5deg", lambda: (grids.cubed_sphere(24), grids.latlon_deg(5.0))),
    ("C48->1deg", lambda: (grids.cubed_sphere(48), grids.latlon_deg(1.0))),
    ("C12->C8", lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8))),
    ("voronoi40962->2deg", lambda: (grids.voronoi(40962, seed=5), grids.latlon_deg(2.0))),
    ("tripole360x270->1deg", lambda: (grids.tripole(360, 270, seed=4), grids.latlon_deg(1.0))),
]


@pytest.mark.parametrize("name,make", BILINEAR_GENERAL_PAIRS)
def test_bilinear_general_parity(gpu, oracle, name, make):
    """Bilinear from a non-rectilinear source (nearest centroids, then the
    reference's quad / triangle / inverse-distance stencils) against the
    oracle: every (dst, src) pair and every weight identical."""
    src, dst = make()
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "bilinear"})
    wo = oracle.bilinear(src, dst)
    csr = _check_weights(M, wo)
    # host-libm inputs and IEEE double stencils on the device: bit for bit
    assert np.array_equal(csr["val"], wo.w)


def _with(g, gpu, mask=None, areas=None):
    return gpu.Mesh.from_arrays(g.node_lonlat, g.conn_offsets, g.conn_indices, areas=areas, mask=mask)


MASK_PAIRS = [
    ("clipper C24->2deg", lambda: (grids.cubed_sphere(24), grids.latlon_deg(2.0))),
    ("regular 1deg->2deg", lambda: (grids.latlon_deg(1.0), grids.latlon_deg(2.0))),
    ("rectilinear", lambda: (grids.equal_area_latlon(72, 36, stretch=0.4), grids.latlon_deg(3.0))),
]


@pytest.mark.parametrize("name,make", MASK_PAIRS)
def test_destination_mask_and_user_areas(gpu, oracle, name, make):
    """Masked destination cells get no entries (every generation path), and
    cell areas given with the mesh replace the computed ones in weights,
    fractions and the reported areas; against the oracle on the same
    inputs."""
    src, dst = make()
    rng = np.random.default_rng(21)
    dmask = (rng.random(dst.n_cells) > 0.2).astype(np.int32)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), _with(dst, gpu, mask=dmask), {"method": "conservative"})
    wo = oracle.conservative(src, dst, dst_mask=dmask)
    _check_weights(M, wo)
    assert not np.isin(np.nonzero(dmask == 0)[0], wo.row).any()
    # user areas: the cells' own areas scaled by a seeded factor near 1
    sa = M.to_csr()["area_a"] * (1.0 + 0.01 * rng.random(src.n_cells))
    da = M.to_csr()["area_b"] * (1.0 + 0.01 * rng.random(dst.n_cells))
    da[da == 0.0] = 1.0
    Ma = gpu.generate_weights(_with(src, gpu, areas=sa), _with(dst, gpu, areas=da), {"method": "conservative"})
    _check_weights(Ma, oracle.conservative(src, dst, src_areas=sa, dst_areas=da))


@pytest.mark.parametrize("name,make", MASK_PAIRS)
def test_both_masks_with_coastal(gpu, oracle, name, make):
    """Source and destination masks together: the generator drops both, then
    the coastal post-pass renormalises and extrapolates the unmasked rows."""
    src, dst = make()
    smask = _land_mask(src)
    rng = np.random.default_rng(22)
    dmask = (rng.random(dst.n_cells) > 0.1).astype(np.int32)
    M = gpu.generate_weights(_with(src, gpu, mask=smask), _with(dst, gpu, mask=dmask), {"method": "conservative"})
    wo = oracle.conservative(src, dst, src_mask=smask, dst_mask=dmask)
    _check_weights(M, oracle.coastal(wo, src, dst, smask))
