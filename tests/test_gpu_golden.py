"""GPU weights and cell geometry against the golden vectors produced by the
reference's own geometry code (tests/golden): the (dst, src) index set
bit-exact, weights, fractions and areas within 1e-12 relative (bilinear
weights bit for bit)."""
import numpy as np
import pytest

from golden_io import cases, load, mesh

pytestmark = pytest.mark.gpu

W_RTOL = 1e-12


@pytest.mark.parametrize("name", cases("conservative"))
def test_gpu_conservative_golden(gpu, name):
    z = load("conservative", name)
    src, dst = mesh(z, "src"), mesh(z, "dst")
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    assert M.nnz == len(z["w"])
    assert np.array_equal(rows, z["row"]) and np.array_equal(csr["col"], z["col"])
    assert np.max(np.abs(csr["val"] - z["w"]) / np.abs(z["w"])) < W_RTOL
    for k in ("frac_a", "frac_b", "area_a", "area_b"):
        ref = z[k]
        assert np.max(np.abs(csr[k] - ref) / np.maximum(np.abs(ref), 1e-300)) < W_RTOL, k


@pytest.mark.parametrize("name", cases("fastpath"))
def test_gpu_fastpath_golden(gpu, name):
    """Regular and rectilinear fast paths against the reference's own
    weight_generator_{conservative,bilinear}_rect{,_nonuniform}.cpp output."""
    z = load("fastpath", name)
    method = str(z["method"])
    cfg = {"method": method, "norm_type": ("DstArea", "FracArea")[int(z["norm_type"])], "unmapped": "Ignore"}
    M = gpu.generate_weights(gpu.Mesh.from_grid(mesh(z, "src")), gpu.Mesh.from_grid(mesh(z, "dst")), cfg)
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    assert M.nnz == len(z["w"])
    assert np.array_equal(rows, z["row"]) and np.array_equal(csr["col"], z["col"])
    if method == "bilinear":
        assert np.array_equal(csr["val"], z["w"])
    else:
        assert np.max(np.abs(csr["val"] - z["w"]) / np.abs(z["w"])) < W_RTOL
    for k in ("frac_a", "frac_b", "area_a", "area_b"):
        ref = z[k]
        assert np.max(np.abs(csr[k] - ref) / np.maximum(np.abs(ref), 1e-300), initial=0.0) < W_RTOL, k


@pytest.mark.parametrize("name", cases("generate"))
def test_gpu_generate_golden(gpu, name):
    """Nearest-neighbour, general bilinear and masked / coastal weights
    against the reference's whole WeightGenerator::generate (masks on the
    meshes, the coastal post-pass inside generate_weights)."""
    z = load("generate", name)
    src, dst = mesh(z, "src"), mesh(z, "dst")
    ms = gpu.Mesh.from_arrays(src.node_lonlat, src.conn_offsets, src.conn_indices,
                              mask=np.asarray(z["src_mask"]) if "src_mask" in z else None)
    md = gpu.Mesh.from_arrays(dst.node_lonlat, dst.conn_offsets, dst.conn_indices,
                              mask=np.asarray(z["dst_mask"]) if "dst_mask" in z else None)
    cfg = {"method": str(z["method"]), "extrap_method": ("none", "nearest_wet")[int(z["extrap"])]}
    csr = gpu.generate_weights(ms, md, cfg).to_csr()
    rows = np.repeat(np.arange(len(csr["row_ptr"]) - 1), np.diff(csr["row_ptr"]))
    assert np.array_equal(rows, z["row"]) and np.array_equal(csr["col"], z["col"])
    if str(z["method"]) == "bilinear":
        # bilinear weights are bit-exact, and a masked source's coastal pass
        # sums each row's wet weights in the generator's corner order
        assert np.array_equal(csr["val"], z["w"]), int(np.sum(csr["val"] != z["w"]))
    # kept entries may carry weight 0 (clamped barycentric weights): exact there
    assert np.max(np.abs(csr["val"] - z["w"]) / np.maximum(np.abs(z["w"]), 1e-300), initial=0.0) < W_RTOL
    for k in ("frac_a", "frac_b", "area_a", "area_b"):
        ref = z[k]
        assert np.max(np.abs(csr[k] - ref) / np.maximum(np.abs(ref), 1e-300), initial=0.0) < W_RTOL, k


def test_gpu_apply_golden(gpu):
    """NaN-aware batch apply (device and host entry points) and masked apply
    against the reference's own apply.hpp loops on the same CSR matrix: bit
    for bit, NaN positions included."""
    import torch
    z = load("apply_nan_masked")
    M = gpu.Matrix.from_csr(int(z["n_src"]), int(z["n_dst"]), z["row_ptr"], z["col"], z["val"])
    X = np.asarray(z["x"])
    for t, ref in zip(z["thres"], z["y_nan"]):
        got = gpu.nan_apply_f64(M, torch.tensor(X, device="cuda"), float(t)).cpu().numpy()
        np.testing.assert_array_equal(got, ref)
        np.testing.assert_array_equal(gpu.nan_batch_apply(M, X.T, float(t)), ref.T)
    y = torch.tensor(np.asarray(z["y0"]), device="cuda")
    gpu.apply_masked(M, torch.tensor(np.asarray(z["x_masked"]), device="cuda"), y,
                     torch.tensor(np.asarray(z["mask"]), device="cuda"))
    np.testing.assert_array_equal(y.cpu().numpy(), z["y_masked"])


def test_gpu_weight_cache_golden(gpu):
    """The reference's own WeightCache blob: the device library reads it into
    the fixture's CSR arrays, and writes the same matrix back byte for byte."""
    blob = load("weight_cache", "5deg_to_C8")["blob"].tobytes()
    z = load("conservative", "5deg_to_C8")
    n_src, n_dst = len(z["frac_a"]), len(z["frac_b"])
    csr = gpu.Matrix.deserialize(blob).to_csr()
    rows = np.repeat(np.arange(n_dst), np.diff(csr["row_ptr"]))
    assert np.array_equal(rows, z["row"]) and np.array_equal(csr["col"], z["col"])
    assert np.array_equal(csr["val"], z["w"])
    for k in ("frac_a", "frac_b", "area_a", "area_b"):
        assert np.array_equal(csr[k], z[k]), k
    rp = np.concatenate([[0], np.cumsum(np.bincount(z["row"], minlength=n_dst))])
    M = gpu.Matrix.from_csr(n_src, n_dst, rp, z["col"], z["w"], z["frac_a"], z["frac_b"], z["area_a"], z["area_b"])
    assert M.serialize() == blob


@pytest.mark.parametrize("name", cases("cellprep"))
def test_gpu_cellprep_golden(gpu, name):
    z = load("cellprep", name)
    g = gpu.Mesh.from_grid(mesh(z, "mesh")).cell_geometry()
    assert np.array_equal(g["degen"], z["degen"])
    assert np.array_equal(g["cap_c"], z["cap_c"])
    assert np.max(np.abs(g["area"] - z["area"]) / z["area"]) < 1e-14
    assert np.max(np.abs(g["cap_r"] - z["cap_r"])) < 1e-15
    assert np.max(np.abs(g["box"] - z["box"])) <= 1.2e-7  # one float ulp where CUDA and libm trig differ
