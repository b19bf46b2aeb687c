"""ctypes bindings for the CPU oracle (test infrastructure only).

``Oracle`` wraps ``liboracle.so`` (the restatement in oracle.cpp) and
``RefLib`` wraps ``_ref/libaxisref.so`` (the reference's own geometry headers
compiled through the shim; present only where the reference checkout was
available at build time). Only tests/, ``__graft_entry__.smoke()`` and the
CPU-baseline leg of bench.py import this package.
"""

from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

_i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(np.float32, flags="C_CONTIGUOUS")
_i32p = np.ctypeslib.ndpointer(np.int32, flags="C_CONTIGUOUS")
_u64 = C.c_uint64


def _mesh_args(m):
    ll = np.ascontiguousarray(np.asarray(m.node_lonlat, dtype=np.float64).T).reshape(-1)  # LayoutLeft
    return (m.n_nodes, ll, m.n_cells, np.ascontiguousarray(m.conn_offsets, dtype=np.int64),
            np.ascontiguousarray(m.conn_indices, dtype=np.int64))


class Weights:
    """CSR weights + frac/area arrays as returned by the oracle."""

    def __init__(self, n_src, n_dst, row, col, w, frac_a, frac_b, area_a, area_b, stats=None, seconds=None):
        self.n_src, self.n_dst = n_src, n_dst
        self.row, self.col, self.w = row, col, w
        self.frac_a, self.frac_b, self.area_a, self.area_b = frac_a, frac_b, area_a, area_b
        self.stats = stats or {}
        self.seconds = seconds
        # per entry, its place in its row's generation order where that is
        # not column order (fast paths, general bilinear), else None
        self.gen = None

    @property
    def nnz(self):
        return int(self.w.shape[0])

    def row_ptr(self):
        rp = np.zeros(self.n_dst + 1, dtype=np.int64)
        np.add.at(rp, self.row + 1, 1)
        return np.cumsum(rp)


def centroid_xy(m):
    """compute_cell_centroids_xy (src/solver/weight_generator.cpp:75-138) for a
    spherical-degree mesh, as float32 (lon, lat) degrees."""
    pi = 3.14159265358979323846
    lon = m.node_lonlat[:, 0] * pi / 180.0
    lat = m.node_lonlat[:, 1] * pi / 180.0
    nv = np.diff(m.conn_offsets)
    cell = np.repeat(np.arange(m.n_cells), nv)
    idx = m.conn_indices
    sx = np.bincount(cell, weights=np.cos(lat[idx]) * np.cos(lon[idx]), minlength=m.n_cells)
    sy = np.bincount(cell, weights=np.cos(lat[idx]) * np.sin(lon[idx]), minlength=m.n_cells)
    sz = np.bincount(cell, weights=np.sin(lat[idx]), minlength=m.n_cells)
    inv = 1.0 / nv
    la = np.arcsin(sz * inv)
    lo = np.arctan2(sy * inv, sx * inv)
    lo = np.where(lo < 0.0, lo + 2.0 * pi, lo)
    return (lo * 180.0 / pi).astype(np.float32), (la * 180.0 / pi).astype(np.float32)


class Oracle:
    def __init__(self, path: str | None = None):
        if path is None:
            path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            from . import build as _b  # noqa: F401  (build recipe lives beside)
            _b.build_oracle()
        L = C.CDLL(path)
        self.L = L
        L.orc_num_threads.restype = C.c_int
        L.orc_set_threads.argtypes = [C.c_int]
        mesh = [C.c_int64, _f64p, C.c_int64, _i64p, _i64p]
        L.orc_detect.argtypes = mesh + [_i32p, _i64p, _f64p]
        L.orc_cell_prep.argtypes = mesh + [_f64p, _f64p, _f64p, _f32p, _i32p]
        L.orc_clip.restype = C.c_double
        L.orc_clip.argtypes = [_f64p, C.c_int, _f64p, C.c_int, _f64p, C.POINTER(C.c_int)]
        L.orc_poly_area.restype = C.c_double
        L.orc_poly_area.argtypes = [_f64p, C.c_int]
        L.orc_morton_encode.restype = _u64
        L.orc_morton_encode.argtypes = [C.c_uint32, C.c_uint32]
        L.orc_normalize_coord.restype = C.c_uint32
        L.orc_normalize_coord.argtypes = [C.c_double, C.c_double, C.c_double]
        L.orc_morton_order.argtypes = mesh + [_i64p]
        L.orc_conservative.restype = C.c_int
        L.orc_conservative.argtypes = (mesh + [C.c_void_p, C.c_void_p] + mesh + [C.c_void_p, C.c_void_p]
                                       + [C.c_int, C.c_int, C.c_int, C.POINTER(C.c_void_p)])
        L.orc_bilinear.restype = C.c_int
        L.orc_bilinear.argtypes = mesh + mesh + [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.orc_nearest.restype = C.c_int
        L.orc_nearest.argtypes = mesh + mesh + [C.c_void_p, C.c_void_p, C.c_int, C.POINTER(C.c_void_p)]
        L.orc_result_nnz.restype = C.c_int64
        L.orc_result_nnz.argtypes = [C.c_void_p]
        L.orc_result_stats.argtypes = [C.c_void_p, _i64p]
        L.orc_result_copy.argtypes = [C.c_void_p, _i64p, _i64p, _f64p, _f64p, _f64p, _f64p, _f64p]
        L.orc_result_free.argtypes = [C.c_void_p]
        L.orc_result_gen.restype = C.c_int
        L.orc_result_gen.argtypes = [C.c_void_p, _i64p]
        L.orc_nan_batch_apply.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, C.c_int64, _f64p, C.c_int64,
                                          C.c_int64, C.c_double]
        L.orc_apply_masked.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, C.c_void_p, _f64p]
        L.orc_apply_csr.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, C.c_int64, _f64p, C.c_int64, C.c_int64,
                                    C.c_int]
        L.orc_apply_coo_atomic.argtypes = [C.c_int64, _i64p, _i64p, _f64p, _f64p, C.c_int64, _f64p, C.c_int64,
                                           C.c_int64, C.c_int64]
        L.orc_conservation.argtypes = [C.c_int64, _f64p, _f64p, _f64p, C.c_int64, _f64p, _f64p, _f64p, C.c_int,
                                       _f64p]

    def threads(self, n: int | None = None) -> int:
        if n is not None:
            self.L.orc_set_threads(int(n))
        return self.L.orc_num_threads()

    def detect(self, m):
        f = np.zeros(2, np.int32)
        d = np.zeros(2, np.int64)
        v = np.zeros(4, np.float64)
        self.L.orc_detect(*_mesh_args(m), f, d, v)
        return dict(regular=bool(f[0]), rectilinear=bool(f[1]), ni=int(d[0]), nj=int(d[1]), lon_min=v[0],
                    dlon=v[1], lat_min=v[2], dlat=v[3])

    def cell_prep(self, m):
        n = m.n_cells
        area = np.zeros(n)
        cc = np.zeros(3 * n)
        cr = np.zeros(n)
        box = np.zeros(6 * n, np.float32)
        deg = np.zeros(n, np.int32)
        self.L.orc_cell_prep(*_mesh_args(m), area, cc, cr, box, deg)
        return dict(area=area, cap_c=cc.reshape(n, 3), cap_r=cr, box=box.reshape(n, 6), degen=deg)

    def clip(self, subj, clipp):
        s = np.ascontiguousarray(subj, np.float64).reshape(-1)
        c = np.ascontiguousarray(clipp, np.float64).reshape(-1)
        out = np.zeros(32 * 3)
        n = C.c_int(0)
        a = self.L.orc_clip(s, len(s) // 3, c, len(c) // 3, out, C.byref(n))
        return a, out[: 3 * n.value].reshape(-1, 3)

    def poly_area(self, xyz):
        x = np.ascontiguousarray(xyz, np.float64).reshape(-1)
        return self.L.orc_poly_area(x, len(x) // 3)

    def morton_encode(self, x, y):
        return int(self.L.orc_morton_encode(x, y))

    def normalize_coord(self, v, lo, hi):
        return int(self.L.orc_normalize_coord(v, lo, hi))

    def morton_order(self, m):
        p = np.zeros(m.n_cells, np.int64)
        self.L.orc_morton_order(*_mesh_args(m), p)
        return p

    def _result(self, h, seconds):
        nnz = self.L.orc_result_nnz(h)
        st = np.zeros(3, np.int64)
        self.L.orc_result_stats(h, st)
        return nnz, st

    def conservative(self, src, dst, norm_type: int = 0, unmapped: int = 1, faithful: bool = False,
                     src_mask=None, dst_mask=None, src_areas=None, dst_areas=None) -> Weights:
        """Conservative weights; masks (int32, 0 = masked) and cell areas
        (float64, replacing the computed ones) as the meshes may carry them."""
        h = C.c_void_p()
        t0 = time.perf_counter()

        def opt(a, dt):
            return None if a is None else np.ascontiguousarray(a, dt)
        sm, dm = opt(src_mask, np.int32), opt(dst_mask, np.int32)
        sa, da = opt(src_areas, np.float64), opt(dst_areas, np.float64)

        def ptr(a):
            return None if a is None else a.ctypes.data_as(C.c_void_p)
        rc = self.L.orc_conservative(*_mesh_args(src), ptr(sa), ptr(sm), *_mesh_args(dst), ptr(da), ptr(dm),
                                     norm_type, unmapped, int(faithful), C.byref(h))
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"oracle conservative failed rc={rc}")
        return self._collect(h, src.n_cells, dst.n_cells, dt)

    def coastal(self, w: Weights, src, dst, src_mask, nearest_wet: bool = True) -> Weights:
        """coastal_renormalize_and_extrapolate (src/solver/weight_generator.cpp:
        1736-1881) on CSR-ordered weights: wet entries (mask > 0) kept, a row
        whose wet weights sum to s in (0, 1) divided by s, and with NearestWet
        every row left empty given the wet source (mask != 0) whose float
        (lon, lat) centroid (compute_cell_centroids_xy, :75-138) is nearest,
        weight 1, ties to the lower index. Brute-force search. The row sums
        run in the order the generator emitted the entries (w.gen where the
        weights carry it, else column order), as the reference's COO loop."""
        mask = np.asarray(src_mask)
        keep = mask[w.col] > 0
        s = np.zeros(w.n_dst)
        seq = np.arange(w.nnz)
        if w.gen is not None:  # within each row, generation order
            seq = np.lexsort((w.gen, w.row))
        for k in seq:
            if keep[k]:
                s[w.row[k]] += w.w[k]
        row, col, val = w.row[keep], w.col[keep], w.w[keep].copy()
        ren = (s[row] > 0.0) & (s[row] < 1.0)
        val[ren] = val[ren] / s[row][ren]
        if nearest_wet:
            wet = np.nonzero(mask != 0)[0]
            dry = np.setdiff1d(np.arange(w.n_dst), np.unique(row))
            if len(wet) and len(dry):
                sx, sy = centroid_xy(src)
                dx, dy = centroid_xy(dst)
                px, py = sx[wet], sy[wet]
                add_c = []
                for j in dry:
                    ex = np.float32(dx[j]) - px
                    ey = np.float32(dy[j]) - py
                    d = ex * ex + ey * ey  # float32, no fused multiply-add
                    add_c.append(wet[int(np.argmin(d))])
                row = np.concatenate([row, dry])
                col = np.concatenate([col, np.array(add_c, np.int64)])
                val = np.concatenate([val, np.ones(len(dry))])
        order = np.lexsort((col, row))
        return Weights(w.n_src, w.n_dst, row[order], col[order], val[order], w.frac_a, w.frac_b, w.area_a, w.area_b)

    @staticmethod
    def _areas(a, n):
        """(keep-alive array, pointer) of optional per-cell areas."""
        if a is None:
            return None, None
        a = np.ascontiguousarray(a, np.float64)
        assert a.shape == (n,)
        return a, a.ctypes.data_as(C.c_void_p)

    def bilinear(self, src, dst, unmapped: int = 1, src_areas=None, dst_areas=None) -> Weights:
        """Bilinear weights; cell areas given with the meshes replace the
        computed ones where the path reports areas (get_cell_areas)."""
        h = C.c_void_p()
        sa, sp = self._areas(src_areas, src.n_cells)
        da, dp = self._areas(dst_areas, dst.n_cells)
        t0 = time.perf_counter()
        rc = self.L.orc_bilinear(*_mesh_args(src), *_mesh_args(dst), sp, dp, unmapped, C.byref(h))
        del sa, da
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"oracle bilinear failed rc={rc}")
        return self._collect(h, src.n_cells, dst.n_cells, dt)

    def nearest(self, src, dst, unmapped: int = 1, src_areas=None, dst_areas=None) -> Weights:
        """Nearest-neighbour weights; areas as for bilinear."""
        h = C.c_void_p()
        sa, sp = self._areas(src_areas, src.n_cells)
        da, dp = self._areas(dst_areas, dst.n_cells)
        t0 = time.perf_counter()
        rc = self.L.orc_nearest(*_mesh_args(src), *_mesh_args(dst), sp, dp, unmapped, C.byref(h))
        del sa, da
        dt = time.perf_counter() - t0
        if rc != 0:
            raise RuntimeError(f"oracle nearest failed rc={rc}")
        return self._collect(h, src.n_cells, dst.n_cells, dt)

    def _collect(self, h, n_src, n_dst, dt):
        nnz = self.L.orc_result_nnz(h)
        st = np.zeros(3, np.int64)
        self.L.orc_result_stats(h, st)
        row = np.zeros(nnz, np.int64)
        col = np.zeros(nnz, np.int64)
        w = np.zeros(nnz)
        fa = np.zeros(n_src)
        fb = np.zeros(n_dst)
        aa = np.zeros(n_src)
        ab = np.zeros(n_dst)
        self.L.orc_result_copy(h, row, col, w, fa, fb, aa, ab)
        gen = np.zeros(nnz, np.int64)
        has_gen = self.L.orc_result_gen(h, gen)
        self.L.orc_result_free(h)
        out = Weights(n_src, n_dst, row, col, w, fa, fb, aa, ab,
                      stats=dict(box_pairs=int(st[0]), cap_pass=int(st[1]), clipped=int(st[2])), seconds=dt)
        out.gen = gen if has_gen else None
        return out

    def apply_csr(self, wts: Weights, x, compensated: bool = True):
        """x: [nrhs, n_src] float64 (row-major = one field per row)."""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        nrhs = x.shape[0]
        y = np.zeros((nrhs, wts.n_dst))
        self.L.orc_apply_csr(wts.n_dst, wts.row_ptr(), np.ascontiguousarray(wts.col), np.ascontiguousarray(wts.w),
                             x.reshape(-1), x.shape[1], y.reshape(-1), wts.n_dst, nrhs, int(compensated))
        return y

    def nan_batch_apply(self, wts: Weights, x, na_thres: float):
        """x: [nrhs, n_src] float64 with NaNs; returns [nrhs, n_dst]."""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        nrhs = x.shape[0]
        y = np.zeros((nrhs, wts.n_dst))
        self.L.orc_nan_batch_apply(wts.n_dst, wts.row_ptr(), np.ascontiguousarray(wts.col),
                                   np.ascontiguousarray(wts.w), x.reshape(-1), x.shape[1], y.reshape(-1), wts.n_dst,
                                   nrhs, float(na_thres))
        return y

    def apply_masked(self, wts: Weights, x, mask, y0):
        """One field; rows with mask 0 keep y0's value."""
        y = np.array(y0, np.float64, copy=True)
        m = np.ascontiguousarray(mask, np.int32)
        self.L.orc_apply_masked(wts.n_dst, wts.row_ptr(), np.ascontiguousarray(wts.col), np.ascontiguousarray(wts.w),
                                np.ascontiguousarray(x, np.float64), m.ctypes.data_as(C.c_void_p), y)
        return y

    def apply_coo_atomic(self, wts: Weights, x):
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        nrhs = x.shape[0]
        y = np.zeros((nrhs, wts.n_dst))
        self.L.orc_apply_coo_atomic(wts.nnz, np.ascontiguousarray(wts.row), np.ascontiguousarray(wts.col),
                                    np.ascontiguousarray(wts.w), x.reshape(-1), x.shape[1], y.reshape(-1), wts.n_dst,
                                    wts.n_dst, nrhs)
        return y

    def conservation(self, wts: Weights, src, dst, norm_type: int = 0):
        out = np.zeros(4)
        self.L.orc_conservation(wts.n_src, np.ascontiguousarray(src, np.float64), wts.area_a, wts.frac_a, wts.n_dst,
                                np.ascontiguousarray(dst, np.float64), wts.area_b, wts.frac_b, norm_type, out)
        return dict(src_integral=out[0], dst_integral=out[1], absolute_error=out[2], relative_error=out[3])


class RefLib:
    """The reference's geometry headers compiled through the shim."""

    def __init__(self, path: str | None = None):
        if path is None:
            path = os.path.join(HERE, "_ref", "libaxisref.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        self.L = L
        mesh = [C.c_int64, _f64p, C.c_int64, _i64p, _i64p]
        L.ref_cell_prep.argtypes = mesh + [_f64p, _f64p, _f64p, _f32p, _i32p]
        L.ref_detect.argtypes = mesh + [_i32p, _i64p, _f64p]
        L.ref_morton_order.argtypes = mesh + [_i64p]
        L.ref_morton_encode.restype = _u64
        L.ref_morton_encode.argtypes = [C.c_uint32, C.c_uint32]
        L.ref_normalize_coord.restype = C.c_uint32
        L.ref_normalize_coord.argtypes = [C.c_double, C.c_double, C.c_double]
        L.ref_clip.restype = C.c_double
        L.ref_clip.argtypes = [_f64p, C.c_int, _f64p, C.c_int, _f64p, C.POINTER(C.c_int)]
        L.ref_conservative.argtypes = mesh + mesh + [C.c_int64, C.POINTER(C.c_int64), _i64p, _i64p, _f64p, _f64p,
                                                     _f64p, _f64p, _f64p]

    def cell_prep(self, m):
        n = m.n_cells
        area = np.zeros(n)
        cc = np.zeros(3 * n)
        cr = np.zeros(n)
        box = np.zeros(6 * n, np.float32)
        deg = np.zeros(n, np.int32)
        self.L.ref_cell_prep(*_mesh_args(m), area, cc, cr, box, deg)
        return dict(area=area, cap_c=cc.reshape(n, 3), cap_r=cr, box=box.reshape(n, 6), degen=deg)

    def detect(self, m):
        f = np.zeros(2, np.int32)
        d = np.zeros(2, np.int64)
        v = np.zeros(4, np.float64)
        self.L.ref_detect(*_mesh_args(m), f, d, v)
        return dict(regular=bool(f[0]), rectilinear=bool(f[1]), ni=int(d[0]), nj=int(d[1]), lon_min=v[0],
                    dlon=v[1], lat_min=v[2], dlat=v[3])

    def morton_order(self, m):
        p = np.zeros(m.n_cells, np.int64)
        self.L.ref_morton_order(*_mesh_args(m), p)
        return p

    def morton_encode(self, x, y):
        return int(self.L.ref_morton_encode(x, y))

    def normalize_coord(self, v, lo, hi):
        return int(self.L.ref_normalize_coord(v, lo, hi))

    def clip(self, subj, clipp):
        s = np.ascontiguousarray(subj, np.float64).reshape(-1)
        c = np.ascontiguousarray(clipp, np.float64).reshape(-1)
        out = np.zeros(32 * 3)
        n = C.c_int(0)
        a = self.L.ref_clip(s, len(s) // 3, c, len(c) // 3, out, C.byref(n))
        return a, out[: 3 * n.value].reshape(-1, 3)

    def conservative(self, src, dst) -> Weights:
        cap = 64 * dst.n_cells + 1024
        nnz = C.c_int64(0)
        row = np.zeros(cap, np.int64)
        col = np.zeros(cap, np.int64)
        w = np.zeros(cap)
        fa = np.zeros(src.n_cells)
        fb = np.zeros(dst.n_cells)
        aa = np.zeros(src.n_cells)
        ab = np.zeros(dst.n_cells)
        self.L.ref_conservative(*_mesh_args(src), *_mesh_args(dst), cap, C.byref(nnz), row, col, w, fa, fb, aa, ab)
        n = nnz.value
        if n > cap:
            raise RuntimeError("reference result larger than buffer")
        return Weights(src.n_cells, dst.n_cells, row[:n], col[:n], w[:n], fa, fb, aa, ab)


class RefFastLib:
    """The reference's regular / rectilinear fast-path sources compiled
    through the shim (oracle/_ref/libaxisref_fast.so, oracle/ref_fast.cpp).
    run(kind, src, dst): kind 0 generate_conservative_rect, 1
    generate_conservative_rect_nonuniform, 2 generate_bilinear_rect, 3
    generate_bilinear_rect_nonuniform; returns Weights in to_csr order."""

    CONS_REGULAR, CONS_RECTILINEAR, BIL_REGULAR, BIL_RECTILINEAR = 0, 1, 2, 3

    def __init__(self, path: str | None = None):
        if path is None:
            path = os.path.join(HERE, "_ref", "libaxisref_fast.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        mesh = [C.c_int64, _f64p, C.c_int64, _i64p, _i64p]
        L.ref_fast.argtypes = ([C.c_int] + mesh + mesh + [C.c_int, C.c_int, C.c_int64, C.POINTER(C.c_int64), _i64p,
                                                          _i64p, _f64p, _f64p, _f64p, _f64p, _f64p])
        L.ref_fast.restype = C.c_int
        self.L = L

    def run(self, kind: int, src, dst, norm_type: int = 0, unmapped: int = 1) -> Weights:
        cap = 64 * dst.n_cells + 64
        nnz = C.c_int64(0)
        row, col, w = np.zeros(cap, np.int64), np.zeros(cap, np.int64), np.zeros(cap)
        fa, fb = np.zeros(src.n_cells), np.zeros(dst.n_cells)
        aa, ab = np.zeros(src.n_cells), np.zeros(dst.n_cells)
        rc = self.L.ref_fast(kind, *_mesh_args(src), *_mesh_args(dst), norm_type, unmapped, cap, C.byref(nnz), row,
                             col, w, fa, fb, aa, ab)
        if rc != 0 or nnz.value > cap:
            raise RuntimeError(f"reference fast path failed rc={rc}")
        n = nnz.value
        return Weights(src.n_cells, dst.n_cells, row[:n].copy(), col[:n].copy(), w[:n].copy(), fa, fb, aa, ab)


class RefGenLib:
    """The reference's whole WeightGenerator::generate (weight_generator.cpp
    and the sources it calls) compiled through the shims, ArborX's queries by
    exhaustive search (oracle/_ref/libaxisref_gen.so, oracle/ref_generate.cpp).
    generate(method, src, dst, ...) returns Weights in to_csr order or raises
    RuntimeError with the reference's message. Quadratic searches: small
    grids only."""

    METHODS = {"bilinear": 0, "nearest_neighbor": 1, "conservative": 4}

    def __init__(self, path: str | None = None):
        if path is None:
            path = os.path.join(HERE, "_ref", "libaxisref_gen.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        mesh = [C.c_int64, _f64p, C.c_int64, _i64p, _i64p, C.c_void_p, C.c_void_p]
        L.ref_generate.argtypes = ([C.c_int] + mesh + mesh + [C.c_int] * 4 + [C.c_int64, C.POINTER(C.c_int64), _i64p,
                                                                               _i64p, _f64p, _f64p, _f64p, _f64p, _f64p])
        L.ref_generate.restype = C.c_int
        L.ref_generate_error.restype = C.c_char_p
        self.L = L

    def generate(self, method, src, dst, norm_type=0, line_type=1, unmapped=1, extrap=1, src_mask=None,
                 dst_mask=None, src_areas=None, dst_areas=None) -> Weights:
        m = self.METHODS[method] if isinstance(method, str) else int(method)
        keep = []

        def opt(a, dt):
            if a is None:
                return None
            a = np.ascontiguousarray(a, dt)
            keep.append(a)
            return a.ctypes.data_as(C.c_void_p)

        cap = 64 * dst.n_cells + 64
        nnz = C.c_int64(0)
        row, col, w = np.zeros(cap, np.int64), np.zeros(cap, np.int64), np.zeros(cap)
        fa, fb = np.zeros(src.n_cells), np.zeros(dst.n_cells)
        aa, ab = np.zeros(src.n_cells), np.zeros(dst.n_cells)
        rc = self.L.ref_generate(m, *_mesh_args(src), opt(src_mask, np.int32), opt(src_areas, np.float64),
                                 *_mesh_args(dst), opt(dst_mask, np.int32), opt(dst_areas, np.float64), norm_type,
                                 line_type, unmapped, extrap, cap, C.byref(nnz), row, col, w, fa, fb, aa, ab)
        if rc != 0:
            raise RuntimeError(self.L.ref_generate_error().decode())
        if nnz.value > cap:
            raise RuntimeError("reference generate: output above capacity")
        n = nnz.value
        return Weights(src.n_cells, dst.n_cells, row[:n].copy(), col[:n].copy(), w[:n].copy(), fa, fb, aa, ab)


class RefApplyLib:
    """The reference's NaN-aware batch apply and masked apply
    (include/axis/solver/apply.hpp, team-policy CSR paths) compiled through
    the shims (oracle/_ref/libaxisref_apply.so, oracle/ref_apply.cpp). Same
    calling conventions as Oracle.nan_batch_apply / Oracle.apply_masked."""

    def __init__(self, path: str | None = None):
        if path is None:
            path = os.path.join(HERE, "_ref", "libaxisref_apply.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        L = C.CDLL(path)
        csr = [C.c_int64, C.c_int64, C.c_int64, _i64p, _i64p, _f64p]
        L.ref_nan_batch_apply.argtypes = csr + [_f64p, _f64p, C.c_int64, C.c_double]
        L.ref_nan_batch_apply.restype = C.c_int
        L.ref_apply_masked.argtypes = csr + [_f64p, _f64p, C.c_void_p]
        L.ref_apply_masked.restype = C.c_int
        self.L = L

    def _csr(self, wts: Weights):
        return (wts.n_src, wts.n_dst, wts.nnz, np.ascontiguousarray(wts.row), np.ascontiguousarray(wts.col),
                np.ascontiguousarray(wts.w))

    def nan_batch_apply(self, wts: Weights, x, na_thres: float):
        """x: [nrhs, n_src] (each field contiguous = LayoutLeft [n_src, nrhs]); returns [nrhs, n_dst]."""
        x = np.ascontiguousarray(np.atleast_2d(x), np.float64)
        y = np.zeros((x.shape[0], wts.n_dst))
        if self.L.ref_nan_batch_apply(*self._csr(wts), x.reshape(-1), y.reshape(-1), x.shape[0], float(na_thres)):
            raise RuntimeError("reference nan_batch_apply threw")
        return y

    def conservation(self, wts: Weights, src, dst, norm_type: int = 0):
        """check_conservation (src/solver/conservation.cpp); same keys as
        Oracle.conservation."""
        L = self.L
        L.ref_conservation.argtypes = [C.c_int64, _f64p, _f64p, _f64p, C.c_int64, _f64p, _f64p, _f64p, C.c_int,
                                       _f64p]
        L.ref_conservation.restype = C.c_int
        out = np.zeros(4)
        f = [np.ascontiguousarray(a, np.float64) for a in (src, wts.area_a, wts.frac_a, dst, wts.area_b, wts.frac_b)]
        if L.ref_conservation(wts.n_src, f[0], f[1], f[2], wts.n_dst, f[3], f[4], f[5], norm_type, out):
            raise RuntimeError("reference check_conservation threw")
        return dict(src_integral=out[0], dst_integral=out[1], absolute_error=out[2], relative_error=out[3])

    def apply_masked(self, wts: Weights, x, mask, y0):
        y = np.array(y0, np.float64, copy=True)
        m = np.ascontiguousarray(mask, np.int32)
        if self.L.ref_apply_masked(*self._csr(wts), np.ascontiguousarray(x, np.float64), y,
                                   m.ctypes.data_as(C.c_void_p)):
            raise RuntimeError("reference masked apply threw")
        return y


def ref_cache_blob(lib: RefApplyLib, n_src, n_dst, row, col, val, frac_a, frac_b, area_a, area_b) -> bytes:
    """The reference's WeightCache::serialize blob of a COO matrix (entries in
    the given order) with its frac/area arrays."""
    L = lib.L
    L.ref_cache_serialize.argtypes = [C.c_int64, C.c_int64, C.c_int64, _i64p, _i64p, _f64p, _f64p, _f64p, _f64p,
                                      _f64p, C.c_void_p, C.c_int64, C.POINTER(C.c_int64)]
    L.ref_cache_serialize.restype = C.c_int
    arrs = [np.ascontiguousarray(a, dt) for a, dt in ((row, np.int64), (col, np.int64), (val, np.float64),
                                                      (frac_a, np.float64), (frac_b, np.float64),
                                                      (area_a, np.float64), (area_b, np.float64))]
    size = C.c_int64(0)
    if L.ref_cache_serialize(n_src, n_dst, len(arrs[2]), *arrs, None, 0, C.byref(size)):
        raise RuntimeError("reference serialize failed")
    buf = C.create_string_buffer(size.value)
    if L.ref_cache_serialize(n_src, n_dst, len(arrs[2]), *arrs, buf, size.value, C.byref(size)):
        raise RuntimeError("reference serialize failed")
    return buf.raw
