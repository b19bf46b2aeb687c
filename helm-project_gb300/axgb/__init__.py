"""Python mirror of the AXIS ``axis_py`` API over the libaxgb C ABI.

Same entry points, argument meaning and error behaviour as the reference's
nanobind module (``libs/axis/python/axis_py.cpp``): ``make_regular_mesh``,
``make_ugrid_mesh``, ``generate_weights``, ``apply_weights``, ``batch_apply``
and ``check_conservation``, plus the GPU-only entry points of this library
(device-tensor apply in FP64 and split FP32, persistent multi-matrix batches).

All computation runs in ``helm-project_gb300/axgb/lib/libaxgb.so`` (built for
sm_103a by ``helm-project_gb300/build.py``); there is no CPU fallback: if the
library is missing or no GPU is present the calls raise.
"""

from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import grids  # noqa: F401  (re-exported)

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libaxgb.so")

# return codes (include/axgb.h)
SUCCESS, ERROR, ERR_INVALID, ERR_CUDA, ERR_UNSUPPORTED, ERR_NOMEM, ERR_TIMEOUT, ERR_UNMAPPED, ERR_HANDLE = (
    0, -1, -2, -3, -4, -5, -6, -7, -8)

# enum values of regrid_config.hpp:24-72
METHODS = {"bilinear": 0, "nearest_neighbor": 1, "bicubic": 2, "patch": 3, "conservative": 4, "conservative2nd": 5}
_METHOD_ALIASES = {"Bilinear": "bilinear", "NearestNeighbor": "nearest_neighbor", "Bicubic": "bicubic",
                   "Patch": "patch", "Conservative1stOrder": "conservative", "Conservative2ndOrder": "conservative2nd"}
NORM = {"dstarea": 0, "DstArea": 0, "fracarea": 1, "FracArea": 1}
LINE = {"cartesian": 0, "Cartesian": 0, "great_circle": 1, "GreatCircle": 1}
UNMAPPED = {"error": 0, "Error": 0, "ignore": 1, "Ignore": 1}

_SYMBOLS = [
    "axgb_default_config", "axgb_init", "axgb_last_error", "axgb_version", "axgb_mesh_create",
    "axgb_mesh_create_regular", "axgb_mesh_info", "axgb_mesh_cell_geometry", "axgb_destroy_mesh",
    "axgb_generate_weights", "axgb_generate_weights_c", "axgb_matrix_stats", "axgb_matrix_info",
    "axgb_matrix_export_csr", "axgb_matrix_import_csr", "axgb_matrix_prepare", "axgb_destroy_matrix",
    "axgb_apply_f64", "axgb_apply_f32split", "axgb_apply_f32split_tuned", "axgb_autotune_f32split",
    "axgb_set_autotune", "axgb_apply_c", "axgb_batch_apply_host_f64", "axgb_batch_apply_host_f32split",
    "axgb_batch_create", "axgb_batch_apply", "axgb_destroy_batch", "axgb_conservation_f64",
    "axgb_conservation_f32", "axgb_matrix_device_status", "axgb_conservation_f64_noalloc",
    "axgb_set_kernel_choice", "axgb_get_kernel_choice", "axgb_nan_batch_apply_f64", "axgb_apply_masked_f64",
    "axgb_nan_batch_apply_host", "axgb_matrix_serialize", "axgb_matrix_deserialize", "axgb_esmf_write",
    "axgb_esmf_read", "axgb_matrix_write_esmf", "axgb_matrix_read_esmf", "axgb_apply_f32split_hilo", "axgb_probe_fp64_fma",
]


class AxgbError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"axgb error {code}: {msg}")
        self.code = code


class InvalidArgument(AxgbError, ValueError):
    """std::invalid_argument of the reference (extent/coordinate mismatch)."""


class Unsupported(AxgbError, NotImplementedError):
    pass


class RegridConfig(C.Structure):
    _fields_ = [("method", C.c_int32), ("norm_type", C.c_int32), ("line_type", C.c_int32),
                ("unmapped", C.c_int32), ("use_limiter", C.c_int32), ("extrap_method", C.c_int32)]


_L = None


def lib():
    """Load libaxgb.so (raises if it has not been built)."""
    global _L
    if _L is not None:
        return _L
    if not os.path.exists(LIB_PATH):
        raise ImportError(f"libaxgb.so not built at {LIB_PATH}; run helm-project_gb300/build.py")
    L = C.CDLL(LIB_PATH)
    i64, i32, vp, dp, fp = C.c_int64, C.c_int32, C.c_void_p, C.c_void_p, C.c_void_p
    ip = C.POINTER(C.c_int)
    L.axgb_default_config.argtypes = [C.POINTER(RegridConfig)]
    L.axgb_default_config.restype = None
    L.axgb_init.argtypes = [C.c_int]
    L.axgb_last_error.argtypes = [C.c_char_p, C.c_size_t]
    L.axgb_version.restype = C.c_char_p
    L.axgb_mesh_create.argtypes = [dp, i64, vp, vp, i64, C.c_int, dp, vp, ip]
    L.axgb_mesh_create_regular.argtypes = [i64, i64, C.c_double, C.c_double, C.c_double, C.c_double, ip]
    L.axgb_mesh_info.argtypes = [C.c_int, vp, vp, vp, vp, vp]
    L.axgb_mesh_cell_geometry.argtypes = [C.c_int, vp, vp, vp, vp, vp]
    L.axgb_destroy_mesh.argtypes = [C.c_int]
    L.axgb_generate_weights.argtypes = [C.c_int, C.c_int, C.POINTER(RegridConfig), ip]
    L.axgb_generate_weights_c.argtypes = [C.c_int, C.c_int, C.c_int, ip]
    L.axgb_matrix_stats.argtypes = [C.c_int, vp, vp]
    L.axgb_matrix_info.argtypes = [C.c_int, vp, vp, vp]
    L.axgb_matrix_export_csr.argtypes = [C.c_int, vp, vp, vp, vp, vp, vp, vp]
    L.axgb_matrix_import_csr.argtypes = [i64, i64, i64, vp, vp, vp, vp, vp, vp, vp, ip]
    L.axgb_matrix_prepare.argtypes = [C.c_int, C.c_int]
    L.axgb_destroy_matrix.argtypes = [C.c_int]
    L.axgb_matrix_device_status.argtypes = [C.c_int, vp]
    L.axgb_apply_f64.argtypes = [C.c_int, vp, i64, vp, i64, i64, vp]
    L.axgb_apply_f32split.argtypes = [C.c_int, vp, i64, vp, i64, i64, vp]
    L.axgb_apply_f32split_tuned.argtypes = [C.c_int, vp, i64, vp, i64, i64, C.c_int, C.c_int, C.c_int, vp]
    L.axgb_apply_f32split_hilo.argtypes = [C.c_int, vp, i64, vp, i64, vp, i64, i64, vp]
    L.axgb_probe_fp64_fma.argtypes = [i64, vp]
    L.axgb_autotune_f32split.argtypes = [C.c_int, vp, i64, vp, i64, i64, vp, vp]
    L.axgb_set_autotune.argtypes = [C.c_int]
    L.axgb_apply_c.argtypes = [C.c_int, vp, vp, C.c_int, C.c_int]
    L.axgb_batch_apply_host_f64.argtypes = [C.c_int, vp, i64, vp, i64, i64]
    L.axgb_batch_apply_host_f32split.argtypes = [C.c_int, vp, i64, vp, i64, i64]
    L.axgb_batch_create.argtypes = [vp, vp, C.c_int, ip]
    L.axgb_batch_apply.argtypes = [C.c_int, vp, vp, vp, vp, vp]
    L.axgb_destroy_batch.argtypes = [C.c_int]
    L.axgb_conservation_f64.argtypes = [C.c_int, vp, vp, C.c_int, vp, vp]
    L.axgb_conservation_f32.argtypes = [C.c_int, vp, vp, C.c_int, vp, vp]
    L.axgb_conservation_f64_noalloc.argtypes = [C.c_int, vp, vp, C.c_int, vp, vp]
    L.axgb_set_kernel_choice.argtypes = [C.c_int, C.c_int64, vp]
    L.axgb_nan_batch_apply_f64.argtypes = [C.c_int, vp, C.c_int64, vp, C.c_int64, C.c_int64, C.c_double, vp]
    L.axgb_apply_masked_f64.argtypes = [C.c_int, vp, vp, vp, vp]
    L.axgb_nan_batch_apply_host.argtypes = [C.c_int, vp, C.c_int64, vp, C.c_int64, C.c_int64, C.c_double]
    L.axgb_matrix_serialize.argtypes = [C.c_int, vp, C.c_int64, vp]
    L.axgb_matrix_deserialize.argtypes = [vp, C.c_int64, vp]
    L.axgb_esmf_write.argtypes = [C.c_char_p, C.c_int64, C.c_int64, C.c_int64, vp, vp, vp]
    L.axgb_esmf_read.argtypes = [C.c_char_p, vp, vp, vp, vp, vp, vp, C.c_int64]
    L.axgb_matrix_write_esmf.argtypes = [C.c_int, C.c_char_p]
    L.axgb_matrix_read_esmf.argtypes = [C.c_char_p, vp]
    L.axgb_get_kernel_choice.argtypes = [C.c_int, C.c_int64, vp, vp]
    _L = L
    return L


def last_error() -> str:
    buf = C.create_string_buffer(4096)
    lib().axgb_last_error(buf, len(buf))
    return buf.value.decode(errors="replace")


def _check(rc: int):
    if rc == SUCCESS:
        return
    msg = last_error()
    if rc == ERR_INVALID:
        raise InvalidArgument(rc, msg)
    if rc == ERR_UNSUPPORTED:
        raise Unsupported(rc, msg)
    raise AxgbError(rc, msg)


_initialised = False


def init(device: int = 0):
    """axis_init_c equivalent: select the CUDA device."""
    global _initialised
    _check(lib().axgb_init(device))
    _initialised = True


def _ensure_init():
    if not _initialised:
        init(0)


def _ptr(a):
    if a is None:
        return None
    if hasattr(a, "data_ptr"):
        return C.c_void_p(a.data_ptr())
    return a.ctypes.data_as(C.c_void_p)


def _stream(stream):
    if stream is None:
        return None
    if hasattr(stream, "cuda_stream"):
        return C.c_void_p(stream.cuda_stream)
    return C.c_void_p(int(stream))


class Mesh:
    """An UnstructuredMesh on the device (handle into libaxgb)."""

    def __init__(self, handle: int):
        self.handle = handle
        n_nodes = C.c_int64()
        n_cells = C.c_int64()
        _check(lib().axgb_mesh_info(handle, C.byref(n_nodes), C.byref(n_cells), None, None, None))
        self.n_nodes = n_nodes.value
        self.n_cells = n_cells.value

    @classmethod
    def from_arrays(cls, node_coords, conn_offsets, conn_indices, areas=None, mask=None):
        """node_coords [n_nodes, 2] (lon, lat) degrees; CSR connectivity."""
        _ensure_init()
        nc = np.asarray(node_coords, dtype=np.float64)
        if nc.ndim != 2 or nc.shape[1] < 2:
            raise InvalidArgument(ERR_INVALID, "node_coords must be [n_nodes, 2]")
        ll = np.ascontiguousarray(nc[:, :2].T)  # LayoutLeft: lons then lats
        off = np.ascontiguousarray(conn_offsets, dtype=np.int64)
        idx = np.ascontiguousarray(conn_indices, dtype=np.int64)
        ar = None if areas is None else np.ascontiguousarray(areas, dtype=np.float64)
        mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.int32)
        h = C.c_int()
        _check(lib().axgb_mesh_create(_ptr(ll), nc.shape[0], _ptr(off), _ptr(idx), off.shape[0] - 1, 0, _ptr(ar),
                                      _ptr(mk), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_grid(cls, g):
        return cls.from_arrays(g.node_lonlat, g.conn_offsets, g.conn_indices)

    def info(self):
        flags = np.zeros(2, np.int32)
        dims = np.zeros(2, np.int64)
        vals = np.zeros(4)
        _check(lib().axgb_mesh_info(self.handle, None, None, _ptr(flags), _ptr(dims), _ptr(vals)))
        return dict(regular=bool(flags[0]), rectilinear=bool(flags[1]), ni=int(dims[0]), nj=int(dims[1]),
                    lon_min=vals[0], dlon=vals[1], lat_min=vals[2], dlat=vals[3])

    def cell_geometry(self):
        n = self.n_cells
        area = np.zeros(n)
        cc = np.zeros((n, 3))
        cr = np.zeros(n)
        box = np.zeros((n, 6), np.float32)
        deg = np.zeros(n, np.int32)
        _check(lib().axgb_mesh_cell_geometry(self.handle, _ptr(area), _ptr(cc), _ptr(cr), _ptr(box), _ptr(deg)))
        return dict(area=area, cap_c=cc, cap_r=cr, box=box, degen=deg)

    def __del__(self):
        try:
            if _L is not None and self.handle:
                _L.axgb_destroy_mesh(self.handle)
        except Exception:
            pass
        self.handle = 0


def make_regular_mesh(ni, nj, lon_start, lat_start, dlon, dlat) -> Mesh:
    """make_regular_mesh (axis_py.cpp:75-103)."""
    _ensure_init()
    h = C.c_int()
    _check(lib().axgb_mesh_create_regular(ni, nj, lon_start, lat_start, dlon, dlat, C.byref(h)))
    return Mesh(h.value)


def make_ugrid_mesh(node_coords, conn_offsets, conn_indices) -> Mesh:
    """make_ugrid_mesh (axis_py.cpp:126-140)."""
    return Mesh.from_arrays(node_coords, conn_offsets, conn_indices)


def parse_regrid_config(config: dict | None) -> RegridConfig:
    """parse_regrid_config (axis_py.cpp:144-221): defaults from RegridConfig,
    string or integer values, unknown names raise ValueError."""
    cfg = RegridConfig()
    lib().axgb_default_config(C.byref(cfg))
    config = config or {}
    if "method" in config:
        m = config["method"]
        if isinstance(m, str):
            key = _METHOD_ALIASES.get(m, m)
            if key not in METHODS:
                raise ValueError("Unknown method: " + m)
            cfg.method = METHODS[key]
        else:
            cfg.method = int(m)
    for name, table, field in (("norm_type", NORM, "norm_type"), ("line_type", LINE, "line_type"),
                               ("unmapped", UNMAPPED, "unmapped")):
        if name in config:
            v = config[name]
            if isinstance(v, str):
                if v not in table:
                    raise ValueError(f"Unknown {name}: {v}")
                setattr(cfg, field, table[v])
            else:
                setattr(cfg, field, int(v))
    if "use_limiter" in config:
        cfg.use_limiter = int(bool(config["use_limiter"]))
    if "extrap_method" in config:  # ExtrapolationAction (regrid_config.hpp:65-88); not parsed by axis_py
        v = config["extrap_method"]
        table = {"none": 0, "nearest_wet": 1}
        if isinstance(v, str):
            if v not in table:
                raise ValueError(f"Unknown extrap_method: {v}")
            cfg.extrap_method = table[v]
        else:
            cfg.extrap_method = int(v)
    return cfg


class Matrix:
    """InterpolationMatrix on the device (CSR + frac/area arrays)."""

    def __init__(self, handle: int):
        self.handle = handle
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        _check(lib().axgb_matrix_info(handle, C.byref(a), C.byref(b), C.byref(c)))
        self.n_src, self.n_dst, self.nnz = a.value, b.value, c.value

    def to_csr(self):
        rp = np.zeros(self.n_dst + 1, np.int64)
        col = np.zeros(self.nnz, np.int64)
        val = np.zeros(self.nnz)
        fa = np.zeros(self.n_src)
        fb = np.zeros(self.n_dst)
        aa = np.zeros(self.n_src)
        ab = np.zeros(self.n_dst)
        _check(lib().axgb_matrix_export_csr(self.handle, _ptr(rp), _ptr(col), _ptr(val), _ptr(fa), _ptr(fb),
                                            _ptr(aa), _ptr(ab)))
        return dict(row_ptr=rp, col=col, val=val, frac_a=fa, frac_b=fb, area_a=aa, area_b=ab)

    def stats(self):
        st = np.zeros(8, np.int64)
        tm = np.zeros(8)
        _check(lib().axgb_matrix_stats(self.handle, _ptr(st), _ptr(tm)))
        return dict(bvh_candidates=int(st[0]), gated_pairs=int(st[1]), fallback_clips=int(st[2]), nnz=int(st[3]),
                    bvh_nodes=int(st[4]), source_renumbered=bool(st[7]), t_prep_ms=tm[0], t_bvh_ms=tm[1],
                    t_search_ms=tm[2], t_clip_ms=tm[3], t_assemble_ms=tm[4], t_total_ms=tm[5])

    def prepare(self, fmt: int):
        _check(lib().axgb_matrix_prepare(self.handle, fmt))

    def device_status(self) -> int:
        st = np.zeros(1, np.int32)
        _check(lib().axgb_matrix_device_status(self.handle, _ptr(st)))
        return int(st[0])

    def serialize(self) -> bytes:
        """WeightCache blob (weight_cache.hpp:49-157)."""
        n = C.c_int64()
        _check(lib().axgb_matrix_serialize(self.handle, None, 0, C.byref(n)))
        buf = C.create_string_buffer(n.value)
        _check(lib().axgb_matrix_serialize(self.handle, buf, n.value, C.byref(n)))
        return buf.raw

    @classmethod
    def deserialize(cls, blob: bytes):
        _ensure_init()
        h = C.c_int()
        _check(lib().axgb_matrix_deserialize(C.c_char_p(blob), len(blob), C.byref(h)))
        return cls(h.value)

    def write_esmf(self, path) -> None:
        """ESMF weight file (EsmfWeightIO::write_esmf, src/io/esmf_weight_io.cpp:66-113),
        as NetCDF-3 64-bit offset."""
        _check(lib().axgb_matrix_write_esmf(self.handle, os.fsencode(path)))

    @classmethod
    def read_esmf(cls, path):
        """EsmfWeightIO::read_esmf (esmf_weight_io.cpp:115-183): NetCDF-3 files;
        frac and area arrays come back zero."""
        _ensure_init()
        h = C.c_int()
        _check(lib().axgb_matrix_read_esmf(os.fsencode(path), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_csr(cls, n_src, n_dst, row_ptr, col, val, frac_a=None, frac_b=None, area_a=None, area_b=None):
        _ensure_init()
        rp = np.ascontiguousarray(row_ptr, np.int64)
        co = np.ascontiguousarray(col, np.int64)
        va = np.ascontiguousarray(val, np.float64)
        arrs = [None if a is None else np.ascontiguousarray(a, np.float64) for a in (frac_a, frac_b, area_a, area_b)]
        h = C.c_int()
        _check(lib().axgb_matrix_import_csr(n_src, n_dst, va.shape[0], _ptr(rp), _ptr(co), _ptr(va),
                                            *[_ptr(a) for a in arrs], C.byref(h)))
        return cls(h.value)

    def __del__(self):
        try:
            if _L is not None and self.handle:
                _L.axgb_destroy_matrix(self.handle)
        except Exception:
            pass
        self.handle = 0


def generate_weights(src: Mesh, dst: Mesh, config: dict | None = None) -> Matrix:
    """generate_weights (axis_py.cpp:633-652)."""
    cfg = parse_regrid_config(config)
    h = C.c_int()
    _check(lib().axgb_generate_weights(src.handle, dst.handle, C.byref(cfg), C.byref(h)))
    return Matrix(h.value)


def apply_weights(matrix: Matrix, src):
    """apply_weights (axis_py.cpp:656-686): one FP64 field. A numpy array goes
    through the host C ABI (axgb_apply_c); a CUDA tensor stays on the device."""
    if hasattr(src, "is_cuda") and src.is_cuda:
        import torch
        x = src.contiguous().to(torch.float64)
        if x.numel() != matrix.n_src:
            raise InvalidArgument(ERR_INVALID, "src extent != matrix.n_src")
        y = torch.empty(matrix.n_dst, dtype=torch.float64, device=x.device)
        _check(lib().axgb_apply_f64(matrix.handle, _ptr(x), max(1, matrix.n_src), _ptr(y), max(1, matrix.n_dst), 1,
                                    _stream(torch.cuda.current_stream())))
        return y
    x = np.ascontiguousarray(src, dtype=np.float64).reshape(-1)
    y = np.zeros(matrix.n_dst)
    _check(lib().axgb_apply_c(matrix.handle, _ptr(x), _ptr(y), x.shape[0], matrix.n_dst))
    return y


def batch_apply(matrix: Matrix, src):
    """batch_apply (axis_py.cpp:690-759): numpy src [n_src, n_vars] (C order,
    as the reference takes it) -> [n_dst, n_vars] FP64 through the host C ABI."""
    a = np.asarray(src, dtype=np.float64)
    if a.ndim != 2:
        raise InvalidArgument(ERR_INVALID, "batch_apply: src must be 2-D [n_src, n_vars]")
    n_vars = a.shape[1]
    x = np.ascontiguousarray(a.T)  # LayoutLeft [n_src, n_vars]
    y = np.zeros((n_vars, matrix.n_dst))
    _check(lib().axgb_batch_apply_host_f64(matrix.handle, _ptr(x), a.shape[0], _ptr(y), matrix.n_dst, n_vars))
    return np.ascontiguousarray(y.T)


def apply_f64(matrix: Matrix, x, y=None, stream=None):
    """Device FP64 apply: x, y CUDA tensors [nrhs, n] (field-major)."""
    import torch
    if x.dim() == 1:
        x = x.view(1, -1)
    if y is None:
        y = torch.empty((x.shape[0], matrix.n_dst), dtype=torch.float64, device=x.device)
    elif y.dim() == 1:
        y = y.view(1, -1)
    _check(lib().axgb_apply_f64(matrix.handle, _ptr(x), x.stride(0), _ptr(y), y.stride(0), x.shape[0],
                                _stream(stream if stream is not None else torch.cuda.current_stream())))
    return y


def apply_f32split(matrix: Matrix, x, y=None, stream=None, fields_per_pass=None, unroll=None, variant=None):
    """Device split-FP32 apply: x, y CUDA float32 tensors [nrhs, n].
    With no tuning arguments the matrix's tuned (or default) kernel is used;
    variant 0 = direct gathers, 1 = shared-memory staged."""
    import torch
    if x.dim() == 1:
        x = x.view(1, -1)
    if y is None:
        y = torch.empty((x.shape[0], matrix.n_dst), dtype=torch.float32, device=x.device)
    elif y.dim() == 1:
        y = y.view(1, -1)
    s = _stream(stream if stream is not None else torch.cuda.current_stream())
    if fields_per_pass is None and unroll is None and variant is None:
        _check(lib().axgb_apply_f32split(matrix.handle, _ptr(x), x.stride(0), _ptr(y), y.stride(0), x.shape[0], s))
    else:
        v = 0 if variant is None else int(variant)
        u = int(unroll) if unroll is not None else (2 if v == 0 else 4)
        _check(lib().axgb_apply_f32split_tuned(matrix.handle, _ptr(x), x.stride(0), _ptr(y), y.stride(0), x.shape[0],
                                               v, int(fields_per_pass or 0), u, s))
    return y


def apply_f32split_hilo(matrix: Matrix, x, y=None, y_lo=None, stream=None):
    """Split-FP32 apply with a low-part output: y is bitwise apply_f32split's
    result and y + y_lo (summed in FP64) carries each compensated row sum to
    about 2^-48 relative. Returns (y, y_lo), CUDA float32 [nrhs, n_dst]."""
    import torch
    if x.dim() == 1:
        x = x.view(1, -1)
    nrhs = x.shape[0]
    if y is None:
        y = torch.empty((nrhs, matrix.n_dst), dtype=torch.float32, device=x.device)
    if y_lo is None:
        y_lo = torch.empty((nrhs, matrix.n_dst), dtype=torch.float32, device=x.device)
    y2, l2 = (y.view(1, -1) if y.dim() == 1 else y), (y_lo.view(1, -1) if y_lo.dim() == 1 else y_lo)
    _check(lib().axgb_apply_f32split_hilo(matrix.handle, _ptr(x), x.stride(0), _ptr(y2), y2.stride(0), _ptr(l2),
                                          l2.stride(0), nrhs,
                                          _stream(stream if stream is not None else torch.cuda.current_stream())))
    return y, y_lo


def probe_fp64_fma(iters: int = 1 << 16) -> float:
    """FP64 FMA throughput of the current device, TFLOP/s."""
    out = np.zeros(1)
    _check(lib().axgb_probe_fp64_fma(int(iters), _ptr(out)))
    return float(out[0])


def autotune_f32split(matrix: Matrix, x, y, stream=None):
    import torch
    best = np.zeros(4, np.int32)
    _check(lib().axgb_autotune_f32split(matrix.handle, _ptr(x), x.stride(0), _ptr(y), y.stride(0), x.shape[0],
                                        _stream(stream if stream is not None else torch.cuda.current_stream()),
                                        _ptr(best)))
    return dict(variant=int(best[0]), fields_per_pass=int(best[1]), unroll=int(best[2]), stages=int(best[3]))


def set_kernel_choice(matrix: Matrix, nrhs: int, variant: int, fields_per_pass: int, unroll: int, stages: int = 2):
    """Seed the cached kernel choice that apply_f32split uses for (matrix, nrhs)."""
    ch = np.array([variant, fields_per_pass, unroll, stages], np.int32)
    _check(lib().axgb_set_kernel_choice(matrix.handle, int(nrhs), _ptr(ch)))


def get_kernel_choice(matrix: Matrix, nrhs: int):
    """The kernel choice apply_f32split would use for (matrix, nrhs), and whether it is cached."""
    ch = np.zeros(4, np.int32)
    cached = np.zeros(1, np.int32)
    _check(lib().axgb_get_kernel_choice(matrix.handle, int(nrhs), _ptr(ch), _ptr(cached)))
    return dict(variant=int(ch[0]), fields_per_pass=int(ch[1]), unroll=int(ch[2]), stages=int(ch[3]),
                cached=bool(cached[0]))


def set_autotune(enable: bool):
    lib().axgb_set_autotune(1 if enable else 0)


def batch_apply_host_f32split(matrix: Matrix, x_host, y_host):
    """Host buffers [nrhs, n] float32 (pinned for speed): copies in, applies,
    copies out (synchronous)."""
    n_vars = x_host.shape[0]
    _check(lib().axgb_batch_apply_host_f32split(matrix.handle, _ptr(x_host), matrix.n_src, _ptr(y_host),
                                                matrix.n_dst, n_vars))
    return y_host


def batch_apply_host_f64(matrix: Matrix, x_host, y_host):
    n_vars = x_host.shape[0]
    _check(lib().axgb_batch_apply_host_f64(matrix.handle, _ptr(x_host), matrix.n_src, _ptr(y_host), matrix.n_dst,
                                           n_vars))
    return y_host


def nan_batch_apply(matrix: Matrix, src, na_thres: float):
    """nan_batch_apply (python/axis_py.cpp:764-821): numpy src [n_src, n_vars]
    with NaNs -> [n_dst, n_vars], through the host C ABI."""
    a = np.asarray(src, dtype=np.float64)
    if a.ndim != 2:
        raise InvalidArgument(ERR_INVALID, "nan_batch_apply: src must be 2-D [n_src, n_vars]")
    n_vars = a.shape[1]
    x = np.ascontiguousarray(a.T)  # LayoutLeft [n_src, n_vars]
    y = np.zeros((n_vars, matrix.n_dst))
    _check(lib().axgb_nan_batch_apply_host(matrix.handle, _ptr(x), a.shape[0], _ptr(y), matrix.n_dst, n_vars,
                                           float(na_thres)))
    return np.ascontiguousarray(y.T)


def nan_apply_f64(matrix: Matrix, x, na_thres: float, y=None, stream=None):
    """Device NaN-aware FP64 apply: x, y CUDA tensors [nrhs, n]."""
    import torch
    if x.dim() == 1:
        x = x.view(1, -1)
    if y is None:
        y = torch.empty((x.shape[0], matrix.n_dst), dtype=torch.float64, device=x.device)
    elif y.dim() == 1:
        y = y.view(1, -1)
    _check(lib().axgb_nan_batch_apply_f64(matrix.handle, _ptr(x), x.stride(0), _ptr(y), y.stride(0), x.shape[0],
                                          float(na_thres),
                                          _stream(stream if stream is not None else torch.cuda.current_stream())))
    return y


def apply_masked(matrix: Matrix, x, y, dst_mask=None, stream=None):
    """Masked apply (apply.hpp:458-532) on device FP64 tensors: rows whose
    int32 mask is 0 keep y's value."""
    import torch
    _check(lib().axgb_apply_masked_f64(matrix.handle, _ptr(x), _ptr(y), _ptr(dst_mask),
                                       _stream(stream if stream is not None else torch.cuda.current_stream())))
    return y


def check_conservation(matrix: Matrix, src, dst, norm_type: int = 0, stream=None):
    """check_conservation (conservation.cpp:83-96) on device FP64/FP32 tensors."""
    import torch
    out = np.zeros(4)
    s = _stream(stream if stream is not None else torch.cuda.current_stream())
    if src.dtype == torch.float32:
        _check(lib().axgb_conservation_f32(matrix.handle, _ptr(src), _ptr(dst), norm_type, _ptr(out), s))
    else:
        _check(lib().axgb_conservation_f64(matrix.handle, _ptr(src), _ptr(dst), norm_type, _ptr(out), s))
    return dict(src_integral=out[0], dst_integral=out[1], absolute_error=out[2], relative_error=out[3])


class Batch:
    """Many (matrix, field count) pairs run by one persistent launch."""

    def __init__(self, matrices, nrhs):
        hs = np.array([m.handle for m in matrices], np.int32)
        nr = np.array(nrhs, np.int64)
        h = C.c_int()
        _check(lib().axgb_batch_create(_ptr(hs), _ptr(nr), len(matrices), C.byref(h)))
        self.handle = h.value
        self.matrices = list(matrices)
        self.nrhs = list(nrhs)

    def apply(self, xs, ys, stream=None):
        import torch
        k = len(self.matrices)
        xp = (C.c_void_p * k)(*[x.data_ptr() for x in xs])
        yp = (C.c_void_p * k)(*[y.data_ptr() for y in ys])
        lx = np.array([x.stride(0) if x.dim() > 1 else x.numel() for x in xs], np.int64)
        ly = np.array([y.stride(0) if y.dim() > 1 else y.numel() for y in ys], np.int64)
        _check(lib().axgb_batch_apply(self.handle, C.cast(xp, C.c_void_p), _ptr(lx), C.cast(yp, C.c_void_p),
                                      _ptr(ly), _stream(stream if stream is not None else torch.cuda.current_stream())))

    def __del__(self):
        try:
            if _L is not None and self.handle:
                _L.axgb_destroy_batch(self.handle)
        except Exception:
            pass
        self.handle = 0


def esmf_write(path, n_a: int, n_b: int, S, col_idx, row_idx) -> None:
    """Host-only ESMF weight file writer (no device needed): S float64, 1-based
    int32 col_idx / row_idx, global attributes n_a / n_b."""
    w = np.ascontiguousarray(S, np.float64)
    c = np.ascontiguousarray(col_idx, np.int32)
    r = np.ascontiguousarray(row_idx, np.int32)
    if not (w.shape == c.shape == r.shape and w.ndim == 1):
        raise InvalidArgument(ERR_INVALID, "esmf_write: S, col_idx, row_idx must be 1-D of one length")
    _check(lib().axgb_esmf_write(os.fsencode(path), int(n_a), int(n_b), w.size, _ptr(w), _ptr(c), _ptr(r)))


def esmf_read(path) -> dict:
    """Host-only ESMF weight file reader: dict of n_a, n_b, S, col_idx, row_idx
    (1-based, as stored)."""
    na, nb, nz = C.c_int64(), C.c_int64(), C.c_int64()
    p = os.fsencode(path)
    _check(lib().axgb_esmf_read(p, C.byref(na), C.byref(nb), C.byref(nz), None, None, None, 0))
    S = np.zeros(nz.value)
    c = np.zeros(nz.value, np.int32)
    r = np.zeros(nz.value, np.int32)
    _check(lib().axgb_esmf_read(p, C.byref(na), C.byref(nb), C.byref(nz), _ptr(S), _ptr(c), _ptr(r), S.size))
    return {"n_a": na.value, "n_b": nb.value, "S": S, "col_idx": c, "row_idx": r}
