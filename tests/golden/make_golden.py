"""Generate the golden fixtures in this folder from the reference's own code.

Run where the reference checkout is present (it is not on the GPU machines):

    python tests/golden/make_golden.py

The reference's geometry headers (spherical clipper, cap filter, Morton
order, degenerate-cell handler, grid detector, trig cache) are compiled
unmodified through the host shim by ``oracle/build.py`` into
``oracle/_ref/libaxisref.so``; its ``ref_conservative`` glue runs the
reference's first-order conservative algorithm around them. Every fixture
stores its input meshes as well, so the tests need neither the reference
nor the grid generators to reproduce the inputs:

* ``conservative_<case>.npz``: src/dst meshes, and the reference's CSR
  (row, col, w), frac_a/b and area_a/b;
* ``clip.npz``: 200 random spherical polygon pairs and the reference
  clipper's overlap area and output polygon;
* ``cellprep_<grid>.npz``: a mesh and the reference's cell areas, bounding
  caps, float AABBs and degenerate flags;
* ``fastpath_<case>.npz``: src/dst meshes, the method ("conservative" or
  "bilinear"), the normalisation and the reference's own regular /
  rectilinear fast-path output (row, col, w, frac and area arrays). These
  come from ``oracle/_ref/libaxisref_fast.so``: the reference's
  weight_generator_{conservative,bilinear}_rect{,_nonuniform}.cpp compiled
  unchanged through the same shim, with its grid detection and to_csr;
* ``generate_<case>.npz``: src/dst meshes, source/destination masks where
  the case has them, the method and extrapolation, and the output of the
  reference's whole WeightGenerator::generate (``oracle/_ref/
  libaxisref_gen.so``: weight_generator.cpp and the solver sources it calls,
  compiled unchanged, ArborX's queries by exhaustive search) for the
  nearest-neighbour, general bilinear and masked / coastal paths;
  Six of them put meshes with degenerate cells (a repeated vertex, cells
  collapsed to a point) or triangle meshes on either side;
* ``apply_nan_masked.npz``: a CSR matrix (the 5 deg -> C8 conservative
  fixture's), fields with NaNs and the reference's own nan_batch_apply at
  four thresholds, and a masked apply (``oracle/_ref/libaxisref_apply.so``:
  include/axis/solver/apply.hpp compiled unchanged through the shim);
* ``weight_cache_5deg_to_C8.npz``: the reference's own WeightCache::serialize
  blob (as bytes) (include/axis/solver/weight_cache.hpp, same library) of the 5 deg ->
  C8 conservative fixture's matrix, entries in CSR order.
"""

from __future__ import annotations

import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
for p in (ROOT, os.path.join(ROOT, "helm-project_gb300")):
    if p not in sys.path:
        sys.path.insert(0, p)

from axgb import grids  # noqa: E402
from oracle import RefApplyLib, RefFastLib, RefGenLib, RefLib, Weights, ref_cache_blob  # noqa: E402
from oracle import build as obuild  # noqa: E402

CONSERVATIVE = {
    "5deg_to_C8": lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8)),
    "C12_to_C8": lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8)),
    "C8_to_10deg": lambda: (grids.cubed_sphere(8), grids.latlon_deg(10.0)),
    "tripole48x36_to_10deg": lambda: (grids.tripole(48, 36, seed=4, jitter=0.1), grids.latlon_deg(10.0)),
}
CELLPREP = {
    "C8": lambda: grids.cubed_sphere(8),
    "5deg": lambda: grids.latlon_deg(5.0),
    "tripole48x36": lambda: grids.tripole(48, 36, seed=4, jitter=0.1),
}

# name -> (make, reference fast-path kind, method, norm_type). Each pair is
# one the reference's dispatch sends to that fast path.
FASTPATH = {
    "cons_regular_5deg_to_10deg": (lambda: (grids.latlon_deg(5.0), grids.latlon_deg(10.0)),
                                   RefFastLib.CONS_REGULAR, "conservative", 0),
    "cons_regular_10deg_to_7p5deg_fracarea": (lambda: (grids.latlon_deg(10.0), grids.latlon_deg(7.5)),
                                              RefFastLib.CONS_REGULAR, "conservative", 1),
    "cons_rectilinear_ea36x18_to_10deg": (lambda: (grids.equal_area_latlon(36, 18, stretch=0.4),
                                                   grids.latlon_deg(10.0)),
                                          RefFastLib.CONS_RECTILINEAR, "conservative", 0),
    "cons_rectilinear_declined_regional": (lambda: (grids.regular_latlon(20, 15, 20.0, -10.0, 2.0, 2.0),
                                                    grids.regular_latlon(10, 10, 10.0, -20.0, 4.0, 4.0)),
                                           RefFastLib.CONS_RECTILINEAR, "conservative", 1),
    "bil_regular_5deg_to_12deg": (lambda: (grids.latlon_deg(5.0), grids.latlon_deg(12.0)),
                                  RefFastLib.BIL_REGULAR, "bilinear", 0),
    "bil_rectilinear_ea36x18_to_C6": (lambda: (grids.equal_area_latlon(36, 18, stretch=0.4), grids.cubed_sphere(6)),
                                    RefFastLib.BIL_RECTILINEAR, "bilinear", 0),
}



def land_mask(src):
    """1 = wet: every cell whose centroid lies outside a 30S-40N, 20E-110E box."""
    c = grids.cell_centroids_xyz(src)
    lat = np.degrees(np.arcsin(c[:, 2]))
    lon = np.degrees(np.arctan2(c[:, 1], c[:, 0])) % 360
    return (~((lat > -30) & (lat < 40) & (lon > 20) & (lon < 110))).astype(np.int32)


def dst_mask(dst, seed=22, dry=0.1):
    return (np.random.default_rng(seed).random(dst.n_cells) > dry).astype(np.int32)


# name -> (make, method, source mask?, destination mask?, extrapolation 0 None / 1 NearestWet)
GENERATE = {
    "nearest_C12_to_C8": (lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8)), "nearest_neighbor", False, False, 1),
    "nearest_voronoi642_to_10deg": (lambda: (grids.voronoi(642, seed=5), grids.latlon_deg(10.0)), "nearest_neighbor",
                                    False, False, 1),
    "bilinear_C12_to_C8": (lambda: (grids.cubed_sphere(12), grids.cubed_sphere(8)), "bilinear", False, False, 1),
    "bilinear_tripole48x36_to_10deg": (lambda: (grids.tripole(48, 36, seed=4, jitter=0.1), grids.latlon_deg(10.0)),
                                       "bilinear", False, False, 1),
    "cons_5deg_to_C8_srcmask_nearestwet": (lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8)), "conservative",
                                           True, False, 1),
    "cons_C8_to_10deg_srcmask_none": (lambda: (grids.cubed_sphere(8), grids.latlon_deg(10.0)), "conservative",
                                      True, False, 0),
    "cons_C8_to_10deg_both_masks": (lambda: (grids.cubed_sphere(8), grids.latlon_deg(10.0)), "conservative", True,
                                    True, 1),
    "nearest_5deg_to_C8_srcmask": (lambda: (grids.latlon_deg(5.0), grids.cubed_sphere(8)), "nearest_neighbor", True,
                                   False, 1),
    "bilinear_C8_to_10deg_srcmask": (lambda: (grids.cubed_sphere(8), grids.latlon_deg(10.0)), "bilinear", True,
                                     False, 1),
    # degenerate cells (repeated vertices, cells collapsed to a point) and triangle meshes
    "cons_degenerateC8_to_10deg": (lambda: (grids.with_degenerate_cells(grids.cubed_sphere(8), 1),
                                            grids.latlon_deg(10.0)), "conservative", False, False, 1),
    "cons_5deg_to_degenerateC8": (lambda: (grids.latlon_deg(5.0),
                                           grids.with_degenerate_cells(grids.cubed_sphere(8), 2)),
                                  "conservative", False, False, 1),
    "cons_triangulatedC6_to_C5": (lambda: (grids.triangulated(grids.cubed_sphere(6)), grids.cubed_sphere(5)),
                                  "conservative", False, False, 1),
    "cons_10deg_to_triangulatedC6": (lambda: (grids.latlon_deg(10.0), grids.triangulated(grids.cubed_sphere(6))),
                                     "conservative", False, False, 1),
    "bilinear_triangulatedC6_to_10deg": (lambda: (grids.triangulated(grids.cubed_sphere(6)),
                                                  grids.latlon_deg(10.0)), "bilinear", False, False, 1),
    "nearest_degenerateC8_to_10deg": (lambda: (grids.with_degenerate_cells(grids.cubed_sphere(8), 1),
                                               grids.latlon_deg(10.0)), "nearest_neighbor", False, False, 1),
}


def mesh_dict(prefix, m):
    return {f"{prefix}_lonlat": m.node_lonlat, f"{prefix}_off": m.conn_offsets, f"{prefix}_idx": m.conn_indices}


def cap_poly(center, radius, nv, rng):
    """Convex spherical polygon: nv points on a small circle, CCW seen from outside."""
    c = center / np.linalg.norm(center)
    a = np.cross(c, [0.0, 0.0, 1.0] if abs(c[2]) < 0.9 else [1.0, 0.0, 0.0])
    a /= np.linalg.norm(a)
    b = np.cross(c, a)
    th = np.sort(rng.uniform(0, 2 * np.pi, nv))
    pts = [np.cos(radius) * c + np.sin(radius) * (np.cos(t) * a + np.sin(t) * b) for t in th]
    return np.array(pts)


def main():
    path = obuild.build_ref()
    if path is None:
        raise SystemExit("the reference checkout is needed to generate the golden fixtures")
    ref = RefLib(path)
    for name, make in CONSERVATIVE.items():
        src, dst = make()
        w = ref.conservative(src, dst)
        np.savez_compressed(os.path.join(HERE, f"conservative_{name}.npz"), **mesh_dict("src", src),
                            **mesh_dict("dst", dst), row=w.row, col=w.col, w=w.w, frac_a=w.frac_a, frac_b=w.frac_b,
                            area_a=w.area_a, area_b=w.area_b)
        print(name, "nnz", w.nnz)
    for name, make in CELLPREP.items():
        m = make()
        c = ref.cell_prep(m)
        np.savez_compressed(os.path.join(HERE, f"cellprep_{name}.npz"), **mesh_dict("mesh", m), **c)
        print("cellprep", name, m.n_cells)
    if obuild.build_ref_fast() is None:
        raise SystemExit("the reference checkout is needed to generate the fast-path fixtures")
    fast = RefFastLib()
    for name, (make, kind, method, norm) in FASTPATH.items():
        src, dst = make()
        w = fast.run(kind, src, dst, norm)
        np.savez_compressed(os.path.join(HERE, f"fastpath_{name}.npz"), **mesh_dict("src", src),
                            **mesh_dict("dst", dst), method=method, norm_type=norm, row=w.row, col=w.col, w=w.w,
                            frac_a=w.frac_a, frac_b=w.frac_b, area_a=w.area_a, area_b=w.area_b)
        print("fastpath", name, "nnz", w.nnz)
    make_generate(GENERATE)
    make_apply()


def make_generate(cases):
    if obuild.build_ref_gen() is None:
        raise SystemExit("the reference checkout is needed to generate the generate() fixtures")
    gen = RefGenLib()
    for name, (make, method, smask, dmask, extrap) in cases.items():
        src, dst = make()
        sm = land_mask(src) if smask else None
        dm = dst_mask(dst) if dmask else None
        w = gen.generate(method, src, dst, extrap=extrap, src_mask=sm, dst_mask=dm)
        extra = {}
        if sm is not None:
            extra["src_mask"] = sm
        if dm is not None:
            extra["dst_mask"] = dm
        np.savez_compressed(os.path.join(HERE, f"generate_{name}.npz"), **mesh_dict("src", src),
                            **mesh_dict("dst", dst), **extra, method=method, extrap=extrap, row=w.row, col=w.col,
                            w=w.w, frac_a=w.frac_a, frac_b=w.frac_b, area_a=w.area_a, area_b=w.area_b)
        print("generate", name, "nnz", w.nnz)


def make_apply():
    if obuild.build_ref_apply() is None:
        raise SystemExit("the reference checkout is needed to generate the apply fixture")
    app = RefApplyLib()
    z = np.load(os.path.join(HERE, "conservative_5deg_to_C8.npz"))
    n_src, n_dst = len(z["frac_a"]), len(z["frac_b"])
    w = Weights(n_src, n_dst, z["row"], z["col"], z["w"], z["frac_a"], z["frac_b"], z["area_a"], z["area_b"])
    rng = np.random.default_rng(31)
    x = rng.standard_normal((6, n_src)) + 280.0
    for v, p in enumerate((0.0, 0.05, 0.3, 0.6, 0.9, 1.0)):
        x[v, rng.uniform(size=n_src) < p] = np.nan
    thres = np.array([0.0, 0.25, 0.5, 1.0])
    y_nan = np.stack([app.nan_batch_apply(w, x, t) for t in thres])
    xm = rng.standard_normal(n_src) + 280.0
    mask = (np.arange(n_dst) % 5 != 1).astype(np.int32)
    y0 = np.full(n_dst, -3.0)
    y_masked = app.apply_masked(w, xm, mask, y0)
    np.savez_compressed(os.path.join(HERE, "apply_nan_masked.npz"), n_src=n_src, n_dst=n_dst,
                        row_ptr=w.row_ptr(), col=w.col, val=w.w, x=x, thres=thres, y_nan=y_nan, x_masked=xm,
                        mask=mask, y0=y0, y_masked=y_masked)
    print("apply fixture: NaN outputs", int(np.isnan(y_nan).sum()))
    blob = ref_cache_blob(app, n_src, n_dst, z["row"], z["col"], z["w"], z["frac_a"], z["frac_b"], z["area_a"],
                          z["area_b"])
    np.savez_compressed(os.path.join(HERE, "weight_cache_5deg_to_C8.npz"), blob=np.frombuffer(blob, np.uint8))
    print("weight cache blob", len(blob), "bytes")
    rng = np.random.default_rng(20240)
    subj, clipp, nsub, ncl, area, nout, outp = [], [], [], [], [], [], []
    for _ in range(200):
        def ll(lo, la):
            return np.array([np.cos(la) * np.cos(lo), np.cos(la) * np.sin(lo), np.sin(la)])
        a = cap_poly(ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 0.5), rng.integers(3, 12), rng)
        b = cap_poly(ll(rng.uniform(-3, 3), rng.uniform(-1.5, 1.5)), rng.uniform(0.001, 0.5), rng.integers(3, 12), rng)
        if rng.uniform() < 0.5:  # overlapping pair: move b onto a
            b = cap_poly(a.mean(0), rng.uniform(0.001, 0.5), rng.integers(3, 12), rng)
        ar, poly = ref.clip(a, b)
        pad = lambda p: np.concatenate([p, np.zeros((32 - len(p), 3))])
        subj.append(pad(a)); clipp.append(pad(b)); nsub.append(len(a)); ncl.append(len(b))
        area.append(ar); nout.append(len(poly)); outp.append(pad(poly))
    np.savez_compressed(os.path.join(HERE, "clip.npz"), subj=np.array(subj), clip=np.array(clipp),
                        n_subj=np.array(nsub), n_clip=np.array(ncl), area=np.array(area), n_out=np.array(nout),
                        out=np.array(outp))
    print("clip pairs", len(area), "overlapping", int(np.sum(np.array(area) > 0)))


if __name__ == "__main__":
    # --generate NAME ...: (re)make only those generate_<NAME>.npz fixtures
    if len(sys.argv) > 2 and sys.argv[1] == "--generate":
        make_generate({k: GENERATE[k] for k in sys.argv[2:]})
    else:
        main()
