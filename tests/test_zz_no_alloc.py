"""The allocation-free conservation entry point.

Some callers cannot call cudaMalloc while they run: a model whose device
memory is all owned by its own pool, or code that must stay free of
allocation between set-up and tear-down. axgb_conservation_f64_noalloc
serves them with a fixed device array for its partial sums. This file checks
it through the C ABI against axgb_conservation_f64 (the allocating entry
point) on two calls in a row, and that it refuses matrices larger than its
fixed scratch allows. It is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13  # the conservation tolerance the GPU parity tests use for integrals


def test_noalloc_conservation_matches_allocating_entry_point(gpu):
    import torch

    from axgb import fields, grids
    src, dst = grids.latlon_deg(1.0), grids.cubed_sphere(48)
    M = gpu.generate_weights(gpu.Mesh.from_grid(src), gpu.Mesh.from_grid(dst), {"method": "conservative"})
    f = fields.sh_field(grids.cell_centroids_xyz(src), 16, seed=1, offset=280.0)
    x = f.to("cuda")
    y = gpu.apply_weights(M, x)
    L = gpu.lib()
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    for norm in (0, 1):
        ref = np.zeros(4)
        assert L.axgb_conservation_f64(M.handle, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), norm,
                                       ref.ctypes.data_as(ctypes.c_void_p), stream) == 0
        for _ in range(2):  # the shared array keeps the previous call's contents
            out = np.full(4, np.nan)
            rc = L.axgb_conservation_f64_noalloc(M.handle, ctypes.c_void_p(x.data_ptr()),
                                                 ctypes.c_void_p(y.data_ptr()), norm,
                                                 out.ctypes.data_as(ctypes.c_void_p), stream)
            assert rc == 0, gpu.last_error()
            assert abs(out[0] - ref[0]) <= RTOL * abs(ref[0])
            assert abs(out[1] - ref[1]) <= RTOL * abs(ref[1])
            assert abs(out[2] - ref[2]) <= RTOL * max(abs(ref[0]), abs(ref[1]))
            assert out[3] < 1e-12 and ref[3] < 1e-12


def test_noalloc_conservation_rejects_oversized_matrix(gpu):
    import torch
    n_src = 16_777_216 + 1
    M = gpu.Matrix.from_csr(n_src, 1, [0, 1], [0], [1.0])
    x = torch.ones(n_src, dtype=torch.float64, device="cuda")
    y = torch.ones(1, dtype=torch.float64, device="cuda")
    out = np.zeros(4)
    rc = gpu.lib().axgb_conservation_f64_noalloc(M.handle, ctypes.c_void_p(x.data_ptr()),
                                                 ctypes.c_void_p(y.data_ptr()), 0,
                                                 out.ctypes.data_as(ctypes.c_void_p), None)
    assert rc == gpu.ERR_INVALID
    assert "16777216" in gpu.last_error()
