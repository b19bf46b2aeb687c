#!/usr/bin/env python
"""Benchmark of the AXIS regridding hot path on one GB300.

Headline workload (one "step" = one pass of the batched apply over the whole
batch): C768 gnomonic cubed sphere (3,538,944 cells) -> 0.25 deg lat-lon
(1,036,800 cells), first-order conservative weights generated on the GPU,
1016 right-hand sides (8 tracers x 127 levels) of FP32 fields laid out
[field][level][cell], each a seeded spherical-harmonic field (l <= 128) times
a seeded lognormal(0,1) per-level scale. The apply is the split-FP32
(hi+lo weights, compensated) SpMM; the plain FP64 SpMM on FP64 copies of the
same fields is timed beside it. Inputs are 14.4 GB per step, larger than L2.

Also reported on the same line: max/RMS relative error of both applies
against the CPU oracle on sampled fields, the conservation errors, the
roofline fraction against the measured HBM copy bandwidth, the end-to-end
throughput through the host-buffer C ABI (pinned host -> device -> host every
step), weight generation for 0.25 deg -> C384 (pairs/s), and the CPU oracle
apply timed on this host's cores.

--impl reference times the reference's CPU algorithm (the oracle port of the
CSR apply, all host threads) on a bounded sample of fields of the same
workload and prints the same metric.
"""

from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "helm-project_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "regrid apply dst-vals/s (split-FP32 SpMM, C768->0.25deg, 1016 RHS)"
UNIT = "dst-vals/s"
N_TRACERS, N_LEVELS = 8, 127
NRHS = N_TRACERS * N_LEVELS
WORKLOAD = "C768->0.25deg conservative, batched split-FP32 SpMM, 1016 RHS (8 tracers x 127 levels)"


def log(*a):
    print(*a, file=sys.stderr, flush=True)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while running."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.lines = []
        self.proc = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                          "-i", str(self.index), "-lms", "50"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except FileNotFoundError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "samples": 0}
        time.sleep(0.12)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def make_fields(xyz_t, nrhs: int = NRHS, seed: int = 2024):
    """[nrhs, n] float32 on the device: the first nrhs of the 1016 fields
    [tracer][level][cell], 8 SH(l<=128) tracers x lognormal level scales."""
    import torch

    from axgb import fields
    n_tr = (nrhs + N_LEVELS - 1) // N_LEVELS
    base = fields.sh_fields(xyz_t, 128, [seed + t for t in range(n_tr)])
    rng = np.random.default_rng(seed)
    scales = rng.lognormal(0.0, 1.0, size=(N_TRACERS, N_LEVELS))
    X = torch.empty((nrhs, xyz_t.shape[0]), dtype=torch.float32, device=xyz_t.device)
    for t in range(n_tr):
        nl = min(N_LEVELS, nrhs - t * N_LEVELS)
        sc = torch.tensor(scales[t][:nl], dtype=torch.float64, device=xyz_t.device)
        X[t * N_LEVELS:t * N_LEVELS + nl] = (base[t][None, :] * sc[:, None]).to(torch.float32)
    del base
    return X, scales


def rel_errors(y, ref):
    d = np.abs(y.astype(np.float64) - ref)
    scale = np.maximum(np.abs(ref), 1e-30)
    return {"max_rel": float(np.max(d / scale)),
            "max_rel_normwise": float(np.max(d) / np.max(np.abs(ref))),
            "rms_rel": float(np.sqrt(np.mean(d ** 2)) / np.sqrt(np.mean(ref ** 2)))}


def cond_errors(y, ref, cond):
    """Error of each output scaled by its condition c_i = sum_j |w_ij x_j|
    (outputs that cross zero keep a meaningful bound), max over outputs."""
    d = np.abs(y.astype(np.float64) - ref)
    return float(np.max(d / np.maximum(cond, 1e-300)))


def weight_parity(M, wo):
    """Index set and weights of a GPU matrix against the oracle's."""
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    same = bool(M.nnz == wo.nnz and np.array_equal(rows, wo.row) and np.array_equal(csr["col"], wo.col))
    wrel = float(np.max(np.abs(csr["val"] - wo.w) / np.maximum(np.abs(wo.w), 1e-300))) if same and M.nnz else None
    return {"index_set_identical": same, "weights_max_rel": wrel, "nnz": int(M.nnz), "oracle_nnz": int(wo.nnz)}


def cpu_apply_rate(oracle, wo, X_cpu):
    """dst-vals/s of the oracle's CSR FP64 apply (OpenMP rows) on X_cpu."""
    t0 = time.perf_counter()
    oracle.apply_csr(wo, X_cpu, compensated=False)
    dt = time.perf_counter() - t0
    return X_cpu.shape[0] * wo.n_dst / dt, dt


def cpu_coo_rate(oracle, wo, X_cpu, budget_s=5.0):
    """dst-vals/s of the COO scatter-add with OpenMP atomics (the path the
    reference's Python batch_apply takes, include/axis/solver/apply.hpp:315-330),
    repeated for about budget_s seconds."""
    oracle.apply_coo_atomic(wo, X_cpu[:1])
    reps, total = 0, 0.0
    while total < budget_s and reps < 100:
        t0 = time.perf_counter()
        oracle.apply_coo_atomic(wo, X_cpu)
        total += time.perf_counter() - t0
        reps += 1
    return reps * X_cpu.shape[0] * wo.n_dst / total, reps, total


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from axgb import fields, grids
    from oracle import Oracle
    from oracle import build as obuild
    obuild.build_oracle()
    o = Oracle()
    cores = os.cpu_count() or 1
    o.threads(cores)
    src, dst = grids.cubed_sphere(768), grids.latlon_deg(0.25)
    t0 = time.perf_counter()
    wo = o.conservative(src, dst)
    gen_s = time.perf_counter() - t0
    xyz = grids.cell_centroids_xyz(src)
    base = fields.sh_fields(xyz, 32, [2024]).numpy()[0]
    sample = 64
    rng = np.random.default_rng(2024)
    X = np.stack([base * s for s in rng.lognormal(0, 1, sample)]).astype(np.float32).astype(np.float64)
    for _ in range(args.warmup):
        cpu_apply_rate(o, wo, X)
    times = []
    for _ in range(args.steps):
        _, dt = cpu_apply_rate(o, wo, X)
        times.append(dt)
    ms = 1e3 * statistics.mean(times)
    value = sample * wo.n_dst / (ms / 1e3)
    coo, coo_reps, coo_s = cpu_coo_rate(o, wo, X[:16])
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": WORKLOAD, "n_src": wo.n_src, "n_dst": wo.n_dst, "nnz": wo.nnz,
                      "nrhs_sampled": sample, "parallelism": "host threads"},
           "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                            "sample": f"{sample} of {NRHS} RHS per step, FP64 CSR row loop (OpenMP), "
                                      f"oracle weights generated in {gen_s:.1f} s",
                            "coo_atomic_value": coo,
                            "coo_atomic_sample": f"16 RHS x {coo_reps} repeats, FP64 COO scatter-add with OpenMP "
                                                 f"atomics, {coo_s:.1f} s"},
           "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="axgb", choices=["axgb", "reference"])
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-voronoi", action="store_true",
                    help="skip the 2,621,442-cell Voronoi -> 0.1 deg case of the default run (its mesh is generated "
                         "on the host in a background process while the headline is measured)")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--nrhs", type=int, default=NRHS,
                    help="fields per step (default 1016 = 8 tracers x 127 levels; smaller values make "
                         "profiling cases of the same kernel; the first nrhs fields of the workload)")
    ap.add_argument("--kernel", default=None,
                    help="fixed kernel choice variant,fields_per_pass,unroll,stages instead of the autotuner")
    ap.add_argument("--workload", default="c768", choices=["c768", "voronoi"],
                    help="c768: the headline C768 -> 0.25 deg, 1016-field workload; voronoi: 2,621,442-cell "
                         "spherical Voronoi mesh -> 0.1 deg, 64 fields (mesh generation takes minutes on the host)")
    ap.add_argument("--apply-only", action="store_true",
                    help="time only the split apply (no FP64 apply, oracle parity, e2e, weight generation "
                         "or CPU baseline reports); for profiler captures")
    ap.add_argument("--batch-only", action="store_true",
                    help="only run the 17-pair persistent batch (weights, graph-captured batch apply, per-pair "
                         "calls) and print its report; for profiler captures of the batch kernels")
    ap.add_argument("--weightgen-only", action="store_true",
                    help="only generate the 0.25 deg -> C384 conservative weights (three times) and print their "
                         "timing; for profiler captures of the weight-generation kernels")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return reference_arm(args)
    if args.batch_only:
        import axgb
        axgb.init(0)
        print(json.dumps({"batch_17_pairs": batch_pairs(args)}))
        return 0
    if args.weightgen_only:
        import axgb
        from axgb import grids
        axgb.init(0)
        md = axgb.Mesh.from_grid(grids.latlon_deg(0.25))
        print(json.dumps({"weightgen_0p25_to_c384": weightgen_c384(md, None)}))
        return 0
    if args.workload == "voronoi":
        return voronoi_main(args)

    import torch

    import axgb
    from axgb import grids, replicas

    rank, world, local = replicas.world_info()
    torch.cuda.set_device(local)
    replicas.init()  # NCCL process group when launched with more than one rank
    axgb.init(local)
    dev = torch.device("cuda", local)

    barrier = replicas.barrier

    # the Voronoi mesh of the large unstructured case takes a minute or two of
    # host time: generate it in a spawned process while the GPU works
    vor_job = vor_path = None
    if rank == 0 and not args.apply_only and not args.no_voronoi:
        import multiprocessing as mp
        import tempfile
        vor_path = os.path.join(tempfile.mkdtemp(prefix="axgb_vor_"), "mesh.npz")
        vor_job = mp.get_context("spawn").Process(target=voronoi_mesh_job, args=(vor_path,), daemon=True)
        vor_job.start()

    # ── weights for the headline workload ──
    t0 = time.perf_counter()
    src_g, dst_g = grids.cubed_sphere(768), grids.latlon_deg(0.25)
    t_grid = time.perf_counter() - t0
    t0 = time.perf_counter()
    ms, md = axgb.Mesh.from_grid(src_g), axgb.Mesh.from_grid(dst_g)
    t_ingest = time.perf_counter() - t0
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M = axgb.generate_weights(ms, md, {"method": "conservative"})
    t_gen3 = time.perf_counter() - t0
    st3 = M.stats()
    log(f"grids {t_grid:.1f}s ingest {t_ingest:.2f}s gen C768->0.25 {t_gen3:.3f}s nnz={M.nnz} {st3}")

    # ── fields ──
    xyz = torch.tensor(grids.cell_centroids_xyz(src_g), device=dev)
    t0 = time.perf_counter()
    nrhs = max(1, min(args.nrhs, NRHS))
    X, scales = make_fields(xyz, nrhs)
    torch.cuda.synchronize()
    e2e_bufs = e2e_alloc(M, X) if rank == 0 and not args.apply_only and not args.no_e2e else None
    log(f"fields {time.perf_counter() - t0:.1f}s")
    Y = torch.empty((nrhs, M.n_dst), dtype=torch.float32, device=dev)
    t0 = time.perf_counter()
    M.prepare(2)
    log(f"apply layouts built in {time.perf_counter() - t0:.2f}s")
    if args.kernel:
        v, fpp, un, stg = (int(t) for t in args.kernel.split(","))
        tuned = {"variant": v, "fields_per_pass": fpp, "unroll": un, "stages": stg}
        axgb.set_kernel_choice(M, nrhs, **tuned)
    else:
        tuned = axgb.autotune_f32split(M, X, Y)
    launches_per_step = axgb_launches(M, tuned["variant"])
    log(f"kernel: {tuned} launches/step={launches_per_step}")

    stream = torch.cuda.current_stream()

    def run_split():
        axgb.apply_f32split(M, X, Y, stream=stream)  # the tuned (or fixed) kernel

    for _ in range(args.warmup):
        run_split()
    torch.cuda.synchronize()
    barrier()
    clk = ClockSampler(local)
    clk.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    barrier()
    e0.record(stream)
    for _ in range(args.steps):
        run_split()
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    clocks = clk.stop()
    ms_step = replicas.max_over_ranks(e0.elapsed_time(e1) / args.steps)
    dst_vals = M.n_dst * nrhs
    value = replicas.aggregate_rate(dst_vals, ms_step / 1e3, world)
    bytes_split = 4 * M.n_src * nrhs + 4 * M.n_dst * nrhs + 12 * M.nnz + 4 * (M.n_dst + 1)
    peak, peak_kind = peaks()
    achieved = bytes_split / (ms_step / 1e3) / 1e9
    log(f"split: {ms_step:.3f} ms/step  {achieved:.0f} GB/s ({achieved / peak:.2%} of {peak_kind} {peak:.0f})")

    traffic, traffic_src = profiled_traffic(tuned) if nrhs == NRHS else (None, "not the 1016-field workload")
    workload = WORKLOAD if nrhs == NRHS else f"C768->0.25deg conservative, batched split-FP32 SpMM, {nrhs} RHS"
    result = {
        "metric": METRIC if nrhs == NRHS else METRIC.replace("1016 RHS", f"{nrhs} RHS"), "value": value,
        "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": workload, "n_src": M.n_src, "n_dst": M.n_dst, "nnz": M.nnz, "nrhs": nrhs,
                   "kernel": tuned, "source_renumbered": M.stats()["source_renumbered"], "l2": f"inputs {4 * M.n_src * nrhs / 1e9:.1f} GB per step > L2",
                   "parallelism": "replicas" if world > 1 else "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic, "traffic_source": traffic_src,
                     "peak_kind": peak_kind, "bytes_per_step": bytes_split,
                     "unit_note": "achieved = algorithmic bytes per step / CUDA-event time per step; a step's "
                                  "class launches run concurrently, so the step is the timed unit"},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
        "weightgen_c768_to_0p25": {"seconds": t_gen3, "nnz": M.nnz, "pairs_per_s": M.nnz / t_gen3,
                                   "candidates": st3["bvh_candidates"], "gated": st3["gated_pairs"],
                                   "stages_ms": {k: st3[k] for k in st3 if k.startswith("t_")}},
    }
    if args.apply_only:
        if rank == 0:
            print(json.dumps(result), flush=True)
        replicas.finalize()
        return 0

    # ── plain FP64 SpMM on FP64 copies of the same fields ──
    X64 = X.to(torch.float64)
    Y64 = torch.empty((nrhs, M.n_dst), dtype=torch.float64, device=dev)
    M.prepare(0)
    for _ in range(args.warmup):
        axgb.apply_f64(M, X64, Y64, stream=stream)
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.steps):
        axgb.apply_f64(M, X64, Y64, stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    ms64 = e0.elapsed_time(e1) / args.steps
    bytes_f64 = 8 * M.n_src * nrhs + 8 * M.n_dst * nrhs + 12 * M.nnz + 4 * (M.n_dst + 1)
    log(f"fp64: {ms64:.3f} ms/step  {bytes_f64 / ms64 / 1e6:.0f} GB/s; split speed-up {ms64 / ms_step:.2f}x")

    fp64_peak = axgb.probe_fp64_fma(1 << 16)  # TFLOP/s of dependent-FMA chains on every SM
    fp64_tflops = 2.0 * M.nnz * nrhs / (ms64 / 1e3) / 1e12
    result["fp64_apply"] = {"ms_per_step": ms64, "GBps": bytes_f64 / ms64 / 1e6, "split_speedup": ms64 / ms_step,
                            "tflops": fp64_tflops, "fp64_fma_peak_tflops": fp64_peak,
                            "frac_of_fp64_fma_peak": fp64_tflops / fp64_peak,
                            "note": "one FP64 FMA per entry and field (2 flops); peak measured on this GPU by "
                                    "axgb_probe_fp64_fma"}

    if rank == 0:
        # ── errors and conservation against the CPU oracle ──
        from oracle import Oracle
        o = Oracle()
        o.threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        wo = o.conservative(src_g, dst_g)
        t_oracle = time.perf_counter() - t0
        csr = M.to_csr()
        rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
        same = M.nnz == wo.nnz and np.array_equal(rows, wo.row) and np.array_equal(csr["col"], wo.col)
        wrel = float(np.max(np.abs(csr["val"] - wo.w) / wo.w)) if same else None
        sample = sorted({0, 1, min(500, nrhs - 1), nrhs - 1})
        Xs = X[sample].to(torch.float64).cpu().numpy()
        ref = o.apply_csr(wo, Xs, compensated=True)
        cond = o.apply_csr(wo, np.abs(Xs), compensated=True)
        e_split = rel_errors(Y[sample].cpu().numpy(), ref)
        e_f64 = rel_errors(Y64[sample].cpu().numpy(), ref)
        e_split["max_err_over_cond"] = cond_errors(Y[sample].cpu().numpy(), ref, cond)
        e_f64["max_err_over_cond"] = cond_errors(Y64[sample].cpu().numpy(), ref, cond)
        cons_split = axgb.check_conservation(M, X[0], Y[0])
        cons_f64 = axgb.check_conservation(M, X64[0], Y64[0])
        # hi+lo output of the split apply (y + y_lo in FP64) and the oracle's own compensated apply, same field
        yh, yl = axgb.apply_f32split_hilo(M, X[:1])
        hilo = yh[0].to(torch.float64) + yl[0].to(torch.float64)
        cons_hilo = axgb.check_conservation(M, X64[0], hilo)
        cons_exact = o.conservation(wo, Xs[0], ref[0])
        e_hilo = cond_errors(hilo.cpu().numpy()[None], ref[:1], cond[:1])
        del yh, yl, hilo
        # operator conservation: sum_j w_ij area_b_j = area_a_i frac_a_i
        colsum = np.bincount(csr["col"], weights=csr["val"] * csr["area_b"][rows], minlength=M.n_src)
        rhs = csr["area_a"] * csr["frac_a"]
        op_cons = float(np.max(np.abs(colsum - rhs) / rhs))
        result["parity"] = {"index_set_identical": bool(same), "weights_max_rel": wrel,
                            "oracle_weightgen_s": t_oracle, "split": e_split, "fp64": e_f64,
                            "sampled_rhs": sample}
        result["conservation"] = {"split_field_rel": cons_split["relative_error"],
                                  "split_hilo_field_rel": cons_hilo["relative_error"],
                                  "fp64_field_rel": cons_f64["relative_error"],
                                  "oracle_exact_field_rel": cons_exact["relative_error"],
                                  "operator_max_rel": op_cons, "split_hilo_max_err_over_cond": e_hilo,
                                  "field": "field 0 (tracer 0, level 0)",
                                  "note": "oracle_exact_field_rel is the compensated FP64 oracle apply of the same "
                                          "field: the floor the reference's own weights and areas set"}
        log("parity", result["parity"])
        log("conservation", result["conservation"])
        del X64, Y64
        torch.cuda.empty_cache()

        # the background mesh job must not share the host with the end-to-end timing
        if vor_job is not None:
            vor_job.join(timeout=1200)
        # ── end to end through the host-buffer C ABI ──
        if e2e_bufs is not None:
            result["e2e"] = e2e_run(M, e2e_bufs, args)
            del e2e_bufs
        # ── weight generation for 0.25 deg -> C384 ──
        result["weightgen_0p25_to_c384"] = weightgen_c384(md, dst_g)
        # ── single-field configurations (1 deg -> C48, 0.25 deg -> C384) ──
        result["single_field_configs"] = small_configs(o)
        log("single-field", result["single_field_configs"])
        # ── uneven batch of 17 grid pairs in one persistent launch ──
        result["batch_17_pairs"] = batch_pairs(args, o)
        log("batch", {k: v for k, v in result["batch_17_pairs"].items() if k not in ("pairs", "nrhs")})
        # ── large unstructured case: Voronoi 2,621,442 cells -> 0.1 deg ──
        if vor_job is not None:
            if vor_job.exitcode == 0:
                src_v, t_mesh = load_voronoi_mesh(vor_path)
                result["voronoi_2p6M_to_0p1deg"] = voronoi_case(args, src_v, o, t_mesh)
                del src_v
                log("voronoi", {k: result["voronoi_2p6M_to_0p1deg"].get(k) for k in ("ms_per_step", "parity")})
            else:
                if vor_job.is_alive():
                    vor_job.terminate()
                result["voronoi_2p6M_to_0p1deg"] = {"error": f"mesh generation exit code {vor_job.exitcode}"}
        # ── CPU baseline: oracle CSR apply on this host ──
        if not args.no_cpu:
            ns = min(64, nrhs)
            xs = X[:ns].to(torch.float64).cpu().numpy()
            reps, total = 0, 0.0
            while total < 10.0 and reps < 1000:  # about 10 s of CPU work
                _, dt = cpu_apply_rate(o, wo, xs)
                reps += 1
                total += dt
            rate = reps * ns * wo.n_dst / total
            coo, coo_reps, coo_s = cpu_coo_rate(o, wo, xs[:16])
            result["cpu_baseline"] = {"value": rate, "unit": UNIT, "cores": os.cpu_count(), "kind": "port",
                                      "sample": f"{ns} of {nrhs} RHS x {reps} repeats, FP64 CSR row loop "
                                                f"(OpenMP, oracle port), {total:.1f} s",
                                      "coo_atomic_value": coo,
                                      "coo_atomic_sample": f"{min(16, ns)} RHS x {coo_reps} repeats, FP64 COO "
                                                           f"scatter-add with OpenMP atomics, {coo_s:.1f} s"}
        print(json.dumps(result), flush=True)
    replicas.finalize()
    return 0


def axgb_launches(M, variant):
    # one launch per non-empty length class of the chosen layout
    st = np.zeros(8, np.int64)
    import ctypes

    import axgb
    axgb._check(axgb.lib().axgb_matrix_stats(M.handle, st.ctypes.data_as(ctypes.c_void_p), None))
    n = int(st[6] if variant >= 1 else st[5])
    return n if n > 0 else 1


def profiled_traffic(tuned):
    """Per-step DRAM bytes of the apply from the committed ncu captures
    (profiles/apply_split_ws_c768_0p25.md: the launches of a 128- or
    256-field step, scaled to 1016 fields, one line per kernel choice), used
    only when a capture of the kernel choice this run uses is there; else
    None. Returns (bytes, source)."""
    p = os.path.join(ROOT, "profiles", "apply_split_ws_c768_0p25.md")
    if not os.path.exists(p):
        return None, "no capture"
    vals = {}
    for line in open(p):
        if line.startswith("traffic_bytes_per_step[") and "]:" in line:
            k, v = line[len("traffic_bytes_per_step["):].split("]:", 1)
            vals[k.strip()] = v.strip()
    want = ",".join(str(tuned[k]) for k in ("variant", "fields_per_pass", "unroll", "stages"))
    if want not in vals:
        return None, f"the committed captures are of kernels {sorted(vals)}, this run uses {want}"
    return float(vals[want]), ("ncu dram__bytes_read.sum + dram__bytes_write.sum of a 128- or 256-field step "
                               "of the same kernel choice, scaled to 1016 fields "
                               "(profiles/apply_split_ws_c768_0p25.md)")

def e2e_alloc(M, X):
    """Pinned host copies of the headline fields and outputs, made before the
    oracle and the other host work of the run allocate host memory."""
    import torch
    nrhs = X.shape[0]
    need = 4 * (M.n_src + M.n_dst) * nrhs
    avail = 0
    try:
        for ln in open("/proc/meminfo"):
            if ln.startswith("MemAvailable:"):
                avail = int(ln.split()[1]) * 1024
    except OSError:
        pass
    if avail and need > 0.6 * avail:
        nrhs = max(8, int(nrhs * 0.6 * avail / need))
    Xh = torch.empty((nrhs, M.n_src), dtype=torch.float32, pin_memory=True)
    Yh = torch.empty((nrhs, M.n_dst), dtype=torch.float32, pin_memory=True)
    Xh.copy_(X[:nrhs])
    return Xh, Yh, nrhs


def link_floor_ms(M, Xh, Yh, reps=3):
    """The same bytes as one host-buffer apply moved by plain copies alone:
    host->device chunks on one stream and device->host chunks on another,
    concurrently (the floor the host link sets for the end-to-end step)."""
    import torch
    nrhs = Xh.shape[0]
    per = max(1, (1 << 26) // (M.n_src + M.n_dst))
    dx = torch.empty((2, per, M.n_src), dtype=torch.float32, device="cuda")
    dy = torch.zeros((2, per, M.n_dst), dtype=torch.float32, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    best = 1e30
    for _ in range(reps + 1):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        with torch.cuda.stream(s1):
            for c, v0 in enumerate(range(0, nrhs, per)):
                nv = min(per, nrhs - v0)
                dx[c % 2, :nv].copy_(Xh[v0:v0 + nv], non_blocking=True)
        with torch.cuda.stream(s2):
            for c, v0 in enumerate(range(0, nrhs, per)):
                nv = min(per, nrhs - v0)
                Yh[v0:v0 + nv].copy_(dy[c % 2, :nv], non_blocking=True)
        torch.cuda.synchronize()
        best = min(best, time.perf_counter() - t0)
    del dx, dy
    return 1e3 * best


def e2e_run(M, bufs, args):
    import axgb
    Xh, Yh, nrhs = bufs
    steps = max(7, min(args.steps, 9))
    for _ in range(1):
        axgb.batch_apply_host_f32split(M, Xh, Yh)
    t = []
    for _ in range(steps):
        t0 = time.perf_counter()
        axgb.batch_apply_host_f32split(M, Xh, Yh)
        t.append(time.perf_counter() - t0)
    s = statistics.median(t)
    floor = link_floor_ms(M, Xh, Yh)
    return {"value": M.n_dst * nrhs / s, "unit": UNIT, "h2d_bytes_per_step": 4 * M.n_src * nrhs,
            "d2h_bytes_per_step": 4 * M.n_dst * nrhs, "ms_per_step": 1e3 * s, "ms_min": 1e3 * min(t),
            "ms_samples": [round(1e3 * v, 2) for v in t], "nrhs": nrhs,
            "link_floor_ms": floor, "frac_of_link_floor": floor / (1e3 * s),
            "link_floor": "the same bytes by plain chunked copies, host->device and device->host concurrently "
                          "(best of 4)",
            "timing": "median of the timed calls (the host link is shared with other jobs on the machine: "
                      "single calls vary; ms_min is the fastest)",
            "api": "axgb_batch_apply_host_f32split (pinned host buffers)"}


VORONOI = dict(n=2621442, seed=5, jitter=0.2, lloyd=5)


def voronoi_mesh_job(path):
    """Generate the config-5 Voronoi mesh and save it (run in a spawned
    process while the GPU measures the headline workload)."""
    from axgb import grids
    t0 = time.perf_counter()
    g = grids.voronoi(**VORONOI)
    np.savez(path, node=g.node_lonlat, off=g.conn_offsets, idx=g.conn_indices, seconds=time.perf_counter() - t0)


def load_voronoi_mesh(path):
    from axgb import grids
    d = np.load(path)
    return grids.MeshArrays(d["node"], d["off"], d["idx"], name=f"voronoi{VORONOI['n']}"), float(d["seconds"])


def voronoi_case(args, src_g, o, t_mesh, timed_steps=None):
    """Large unstructured case: a 2,621,442-cell spherical Voronoi mesh
    (seeded jittered Fibonacci generators, 5 Lloyd iterations) -> 0.1 deg
    lat-lon (6,480,000 cells). Conservative weights generated on the GPU
    (pairs/s), then the split-FP32 apply of 64 FP32 fields (8 seeded
    spherical-harmonic fields with l <= 256, each at 8 seeded lognormal
    scales) against the plain FP64 apply, with the whole weight set, sampled
    field errors and the conservation errors checked against the CPU oracle
    (o; None skips the oracle checks)."""
    import torch

    import axgb
    from axgb import fields, grids
    dev = torch.device("cuda", 0)
    steps = timed_steps or args.steps
    dst_g = grids.latlon_deg(0.1)
    ms, md = axgb.Mesh.from_grid(src_g), axgb.Mesh.from_grid(dst_g)
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        M = axgb.generate_weights(ms, md, {"method": "conservative"})
        times.append(time.perf_counter() - t0)
    st = M.stats()
    log(f"voronoi weights {min(times):.3f}s nnz={M.nnz} {st}")
    nrhs = 64
    xyz = torch.tensor(grids.cell_centroids_xyz(src_g), device=dev)
    base = fields.sh_fields(xyz, 256, [7000 + k for k in range(8)], chunk=1 << 20)
    scales = np.random.default_rng(7000).lognormal(0.0, 1.0, size=(8, 8))
    # leading dimension padded to a multiple of 4 floats (16-byte aligned field
    # starts, which the shared-memory staged kernels need; n_src = 2,621,442)
    ld = (M.n_src + 3) // 4 * 4
    X = torch.empty((nrhs, ld), dtype=torch.float32, device=dev)[:, :M.n_src]
    for k in range(8):
        sc = torch.tensor(scales[k], dtype=torch.float64, device=dev)
        X[8 * k:8 * k + 8] = (base[k][None, :] * sc[:, None]).to(torch.float32)
    del base, xyz
    Y = torch.empty((nrhs, M.n_dst), dtype=torch.float32, device=dev)
    M.prepare(2)
    if args.kernel:
        v, fpp, un, stg = (int(t) for t in args.kernel.split(","))
        tuned = {"variant": v, "fields_per_pass": fpp, "unroll": un, "stages": stg}
        axgb.set_kernel_choice(M, nrhs, **tuned)
    else:
        tuned = axgb.autotune_f32split(M, X, Y)
    log(f"voronoi kernel: {tuned}")
    stream = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def timed(fn):
        for _ in range(args.warmup):
            fn()
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(steps):
            fn()
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / steps

    clk = ClockSampler(0)
    clk.start()
    ms_split = timed(lambda: axgb.apply_f32split(M, X, Y, stream=stream))
    clocks = clk.stop()
    bytes_split = 4 * (M.n_src + M.n_dst) * nrhs + 12 * M.nnz + 4 * (M.n_dst + 1)
    peak, peak_kind = peaks()
    achieved = bytes_split / (ms_split / 1e3) / 1e9
    result = {
        "metric": "regrid apply dst-vals/s (split-FP32 SpMM, Voronoi 2.6M -> 0.1deg, 64 RHS)",
        "value": M.n_dst * nrhs / (ms_split / 1e3), "unit": UNIT, "n_gpus": 1, "steps": steps,
        "warmup": args.warmup, "ms_per_step": ms_split, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "spherical Voronoi 2,621,442 cells (5 Lloyd iterations) -> 0.1deg lat-lon "
                               "6,480,000 cells, conservative, split-FP32 SpMM, 64 RHS",
                   "n_src": M.n_src, "n_dst": M.n_dst, "nnz": M.nnz, "nrhs": nrhs, "kernel": tuned,
                   "source_renumbered": M.stats()["source_renumbered"],
                   "l2": f"inputs {4 * M.n_src * nrhs / 1e9:.2f} GB per step > L2", "parallelism": "single GPU"},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": None, "peak_kind": peak_kind, "bytes_per_step": bytes_split},
        "clocks": clocks,
        "mesh_generation_s": t_mesh,
        "weightgen": {"seconds_best": min(times), "seconds_first": times[0], "nnz": M.nnz,
                      "pairs_per_s": M.nnz / min(times), "candidates": st["bvh_candidates"],
                      "gated": st["gated_pairs"], "fallback_clips": st["fallback_clips"],
                      "stages_ms": {k: st[k] for k in st if k.startswith("t_")}},
    }
    if not args.apply_only:
        X64 = X.to(torch.float64)
        Y64 = torch.empty((nrhs, M.n_dst), dtype=torch.float64, device=dev)
        M.prepare(0)
        ms64 = timed(lambda: axgb.apply_f64(M, X64, Y64, stream=stream))
        result["fp64_apply"] = {"ms_per_step": ms64, "split_speedup": ms64 / ms_split}
        log(f"voronoi split {ms_split:.3f} ms ({achieved:.0f} GB/s), fp64 {ms64:.3f} ms")
        if o is not None:
            t0 = time.perf_counter()
            wo = o.conservative(src_g, dst_g)
            t_oracle = time.perf_counter() - t0
            sample = [0, 9, 35, 63]
            Xs = X[sample].to(torch.float64).cpu().numpy()
            ref = o.apply_csr(wo, Xs, compensated=True)
            cond = o.apply_csr(wo, np.abs(Xs), compensated=True)
            e_s, e_d = rel_errors(Y[sample].cpu().numpy(), ref), rel_errors(Y64[sample].cpu().numpy(), ref)
            e_s["max_err_over_cond"] = cond_errors(Y[sample].cpu().numpy(), ref, cond)
            e_d["max_err_over_cond"] = cond_errors(Y64[sample].cpu().numpy(), ref, cond)
            result["parity"] = dict(weight_parity(M, wo), oracle_weightgen_s=t_oracle, split=e_s, fp64=e_d,
                                    sampled_rhs=sample)
            result["conservation"] = {
                "split_field_rel": axgb.check_conservation(M, X[0], Y[0])["relative_error"],
                "fp64_field_rel": axgb.check_conservation(M, X64[0], Y64[0])["relative_error"],
                "oracle_exact_field_rel": o.conservation(wo, Xs[0], ref[0])["relative_error"]}
        del X64, Y64
    del X, Y, M
    torch.cuda.empty_cache()
    return result


def voronoi_main(args):
    """--workload voronoi: the config-5 case on its own, one JSON line."""
    import axgb
    from axgb import grids
    axgb.init(0)
    t0 = time.perf_counter()
    src_g = grids.voronoi(**VORONOI)
    t_mesh = time.perf_counter() - t0
    log(f"voronoi mesh {t_mesh:.1f}s")
    o = None
    if not args.apply_only:
        from oracle import Oracle
        o = Oracle()
        o.threads(os.cpu_count() or 1)
    print(json.dumps(voronoi_case(args, src_g, o, t_mesh)), flush=True)
    return 0


def batch_pairs(args, o=None):
    """Uneven batch of grid pairs in one persistent, graph-captured launch:
    every cubed-sphere (C48, C96, C192, C384) x lat-lon (2, 1, 0.5, 0.25 deg)
    combination, the direction alternating with the parity of the two grid
    indices so each grid is source and destination, plus a 1440 x 1080
    tripole-style grid -> 0.5 deg (17 pairs). Each pair carries a seeded
    uniform 1..64 FP32 fields. Reports weight generation of all pairs, the
    batch apply (dst-vals/s, algorithmic GB/s) and the same work as one
    tuned apply call per pair, and checks the batch bitwise against them."""
    import torch

    import axgb
    from axgb import grids
    cs = {n: grids.cubed_sphere(n) for n in (48, 96, 192, 384)}
    ll = {d: grids.latlon_deg(d) for d in (2.0, 1.0, 0.5, 0.25)}
    meshes = {}

    def mesh(key, g):
        if key not in meshes:
            meshes[key] = axgb.Mesh.from_grid(g)
        return meshes[key]

    pairs = []
    for a, n in enumerate(cs):
        for b, d in enumerate(ll):
            if (a + b) % 2 == 0:
                pairs.append((f"C{n}->{d}deg", ("cs", n), cs[n], ("ll", d), ll[d]))
            else:
                pairs.append((f"{d}deg->C{n}", ("ll", d), ll[d], ("cs", n), cs[n]))
    pairs.append(("tripole1440x1080->0.5deg", ("tp",), grids.tripole(1440, 1080, seed=4, jitter=0.1), ("ll", 0.5),
                  ll[0.5]))
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    mats = [axgb.generate_weights(mesh(ks, gs), mesh(kd, gd), {"method": "conservative"}) for _, ks, gs, kd, gd in pairs]
    torch.cuda.synchronize()
    t_gen = time.perf_counter() - t0
    rng = np.random.default_rng(404)
    nrhs = [int(v) for v in rng.integers(1, 65, len(pairs))]
    gen = torch.Generator(device="cuda").manual_seed(404)
    xs = [torch.rand((k, M.n_src), device="cuda", generator=gen, dtype=torch.float32) for k, M in zip(nrhs, mats)]
    ys = [torch.empty((k, M.n_dst), device="cuda", dtype=torch.float32) for k, M in zip(nrhs, mats)]
    B = axgb.Batch(mats, nrhs)
    for _ in range(args.warmup):
        B.apply(xs, ys)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(args.steps):
        B.apply(xs, ys)
    e1.record()
    torch.cuda.synchronize()
    ms_b = e0.elapsed_time(e1) / args.steps
    # the same work as one tuned call per pair
    for M, x, y in zip(mats, xs, ys):
        M.prepare(2)
        axgb.autotune_f32split(M, x, y)
    yp = [torch.empty_like(y) for y in ys]
    for _ in range(args.warmup):
        for M, x, y in zip(mats, xs, yp):
            axgb.apply_f32split(M, x, y)
    torch.cuda.synchronize()
    e0.record()
    for _ in range(args.steps):
        for M, x, y in zip(mats, xs, yp):
            axgb.apply_f32split(M, x, y)
    e1.record()
    torch.cuda.synchronize()
    ms_p = e0.elapsed_time(e1) / args.steps
    same = all(torch.equal(a, b) for a, b in zip(ys, yp))
    oracle_parity = None
    if o is not None:
        # every pair's weights against the oracle, and the batch outputs of up
        # to two fields per pair against the compensated FP64 oracle apply
        oracle_parity = {"pairs_index_set_identical": 0, "weights_max_rel": 0.0, "apply_max_err_over_cond": 0.0,
                         "mismatched": []}
        for (name, _, gs, _, gd), M, x, y in zip(pairs, mats, xs, ys):
            wo = o.conservative(gs, gd)
            wp = weight_parity(M, wo)
            if wp["index_set_identical"]:
                oracle_parity["pairs_index_set_identical"] += 1
                oracle_parity["weights_max_rel"] = max(oracle_parity["weights_max_rel"], wp["weights_max_rel"] or 0.0)
                k = min(2, x.shape[0])
                xf = x[:k].to(torch.float64).cpu().numpy()
                ref = o.apply_csr(wo, xf, compensated=True)
                cond = o.apply_csr(wo, np.abs(xf), compensated=True)
                oracle_parity["apply_max_err_over_cond"] = max(oracle_parity["apply_max_err_over_cond"],
                                                               cond_errors(y[:k].cpu().numpy(), ref, cond))
            else:
                oracle_parity["mismatched"].append({name: wp})
        oracle_parity["pairs"] = len(pairs)
    dst_vals = sum(k * M.n_dst for k, M in zip(nrhs, mats))
    nbytes = sum(4 * k * (M.n_src + M.n_dst) + 12 * M.nnz + 4 * (M.n_dst + 1) for k, M in zip(nrhs, mats))
    return {"pairs": [p[0] for p in pairs], "nrhs": nrhs, "nnz_total": int(sum(M.nnz for M in mats)),
            "weightgen_s": t_gen, "batch_ms": ms_b, "batch_dst_vals_per_s": dst_vals / (ms_b / 1e3),
            "batch_GBps": nbytes / ms_b / 1e6, "per_pair_calls_ms": ms_p, "bitwise_equal_to_per_pair": bool(same),
            "oracle_parity": oracle_parity,
            "launches": "one CUDA graph per batch apply: a persistent staged kernel per row-length class "
                        "(work queue over the blocks of all pairs) and one persistent direct kernel for "
                        "the slices the staged layout leaves out and the rows of more than 32 entries"}


def small_configs(o):
    """The single-field configurations: 1 deg -> C48 (weights + one FP64
    SpMV, against the oracle's weights and output) and 0.25 deg -> C384 (one
    FP32 field with l <= 64: plain FP64 apply vs split-FP32 apply, errors
    against the FP64 oracle and conservation). Also times the oracle's
    faithful (serial, as the reference's loop) weight generation for
    1 deg -> C48 on one host core."""
    import torch

    import axgb
    from axgb import fields, grids
    out = {}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def dev_time(fn, reps=20):
        for _ in range(3):
            fn()
        torch.cuda.synchronize()
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    flush = None

    def cold_time(fn, reps=20):
        """Device time per call with L2 flushed before each call (a 256 MB
        write), events around the call alone."""
        nonlocal flush
        if flush is None:
            flush = torch.empty(64 << 20, dtype=torch.float32, device="cuda")
        for _ in range(3):
            fn()
        tot = 0.0
        for _ in range(reps):
            flush.fill_(1.0)
            e0.record()
            fn()
            e1.record()
            torch.cuda.synchronize()
            tot += e0.elapsed_time(e1)
        return tot / reps

    def graph_time(fn, reps=20):
        """Device time per call of fn with the host out of the loop: reps
        calls captured in one CUDA graph, replayed."""
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            for _ in range(3):
                fn()
        torch.cuda.current_stream().wait_stream(side)
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for _ in range(reps):
                fn()
        g.replay()
        torch.cuda.synchronize()
        e0.record()
        g.replay()
        e1.record()
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / reps

    # config 1
    src, dst = grids.latlon_deg(1.0), grids.cubed_sphere(48)
    ms, md = axgb.Mesh.from_grid(src), axgb.Mesh.from_grid(dst)
    M = axgb.generate_weights(ms, md, {"method": "conservative"})
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    M = axgb.generate_weights(ms, md, {"method": "conservative"})
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    wf = o.conservative(src, dst, faithful=True)
    t_faithful = time.perf_counter() - t0
    f = fields.sh_field(grids.cell_centroids_xyz(src), 16, seed=1, offset=280.0).numpy()
    x = torch.tensor(f, device="cuda")
    y = torch.empty(M.n_dst, dtype=torch.float64, device="cuda")
    ms1 = dev_time(lambda: axgb.apply_f64(M, x, y))
    ref = o.apply_csr(wf, f, compensated=True)[0]
    csr = M.to_csr()
    rows = np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"]))
    out["c1_1deg_to_C48"] = {
        "nnz": M.nnz, "weightgen_s": t_gen, "pairs_per_s": M.nnz / t_gen,
        "oracle_faithful_weightgen_s_1core": t_faithful,
        "index_set_identical": bool(M.nnz == wf.nnz and np.array_equal(rows, wf.row)
                                    and np.array_equal(csr["col"], wf.col)),
        "spmv_fp64_ms": ms1, "spmv_dst_vals_per_s": M.n_dst / (ms1 / 1e3),
        "fp64": rel_errors(y.cpu().numpy()[None], ref[None]),
        "conservation_fp64": axgb.check_conservation(M, x, y)["relative_error"]}
    # config 2
    src, dst = grids.latlon_deg(0.25), grids.cubed_sphere(384)
    M = axgb.generate_weights(axgb.Mesh.from_grid(src), axgb.Mesh.from_grid(dst), {"method": "conservative"})
    f32 = fields.sh_field(torch.tensor(grids.cell_centroids_xyz(src), device="cuda"), 64, seed=2).to(torch.float32)
    x32 = f32.view(1, -1).contiguous()
    x64 = x32.to(torch.float64)
    y32 = torch.empty((1, M.n_dst), dtype=torch.float32, device="cuda")
    y64 = torch.empty((1, M.n_dst), dtype=torch.float64, device="cuda")
    M.prepare(2)
    axgb.autotune_f32split(M, x32, y32)
    ms_s = dev_time(lambda: axgb.apply_f32split(M, x32, y32))
    ms_d = dev_time(lambda: axgb.apply_f64(M, x64, y64))
    ms_s_g = graph_time(lambda: axgb.apply_f32split(M, x32, y32))
    ms_d_g = graph_time(lambda: axgb.apply_f64(M, x64, y64))
    ms_s_c = cold_time(lambda: axgb.apply_f32split(M, x32, y32))
    ms_d_c = cold_time(lambda: axgb.apply_f64(M, x64, y64))
    wo = o.conservative(src, dst)
    ref = o.apply_csr(wo, x64.cpu().numpy(), compensated=True)
    cond = o.apply_csr(wo, np.abs(x64.cpu().numpy()), compensated=True)
    cons_par = weight_parity(M, wo)
    # bilinear 0.25 deg -> C384 against the oracle at full size
    Mbil = axgb.generate_weights(axgb.Mesh.from_grid(src), axgb.Mesh.from_grid(dst), {"method": "bilinear"})
    wb = o.bilinear(src, dst)
    bil_par = weight_parity(Mbil, wb)
    if bil_par["index_set_identical"]:
        bil_par["bitwise"] = bool(np.array_equal(Mbil.to_csr()["val"], wb.w))
    del Mbil
    # NaN-aware batched FP64 apply (skipna) on the same matrix: 16 fields, 5% NaN sources
    nf = 16
    gen = torch.Generator(device="cuda").manual_seed(77)
    xn = 280.0 + torch.randn((nf, M.n_src), device="cuda", dtype=torch.float64, generator=gen)
    xn[torch.rand((nf, M.n_src), device="cuda", generator=gen) < 0.05] = float("nan")
    yn = torch.empty((nf, M.n_dst), device="cuda", dtype=torch.float64)
    ms_nan = dev_time(lambda: axgb.nan_apply_f64(M, xn, 0.5, yn))
    xs = xn[:2].cpu().numpy()
    from oracle import Weights
    csr = M.to_csr()
    wg = Weights(M.n_src, M.n_dst, np.repeat(np.arange(M.n_dst), np.diff(csr["row_ptr"])).astype(np.int64),
                 csr["col"].astype(np.int64), csr["val"], csr["frac_a"], csr["frac_b"], csr["area_a"], csr["area_b"])
    ref_nan = o.nan_batch_apply(wg, xs, 0.5)  # the oracle's loop on the GPU's weights
    nan_bytes = 8 * (M.n_src + M.n_dst) * nf + 12 * M.nnz + 4 * (M.n_dst + 1)
    out["c2_nan_batch_apply_16_fields"] = {
        "ms": ms_nan, "GBps": nan_bytes / ms_nan / 1e6,
        "bitwise_equal_to_oracle_loop": bool(np.array_equal(yn[:2].cpu().numpy(), ref_nan, equal_nan=True)),
        "nan_outputs": int(torch.isnan(yn).sum().item())}
    e_s, e_d = rel_errors(y32.cpu().numpy(), ref), rel_errors(y64.cpu().numpy(), ref)
    e_s["max_err_over_cond"] = cond_errors(y32.cpu().numpy(), ref, cond)
    e_d["max_err_over_cond"] = cond_errors(y64.cpu().numpy(), ref, cond)
    bytes_1 = 12 * M.nnz + 4 * (M.n_dst + 1) + 4 * M.n_src + 4 * M.n_dst
    out["c2_0p25deg_to_C384_one_field"] = {
        "nnz": M.nnz, "conservative_weights_vs_oracle": cons_par, "bilinear_weights_vs_oracle": bil_par,
        "split_ms": ms_s, "fp64_ms": ms_d, "split_speedup": ms_d / ms_s,
        "split_ms_graph": ms_s_g, "fp64_ms_graph": ms_d_g, "split_speedup_graph": ms_d_g / ms_s_g,
        "split_GBps_graph": bytes_1 / ms_s_g / 1e6,
        "split_ms_cold": ms_s_c, "fp64_ms_cold": ms_d_c, "split_GBps_cold": bytes_1 / ms_s_c / 1e6,
        "split_frac_cold": bytes_1 / ms_s_c / 1e6 / peaks()[0],
        "timing": "split_ms / fp64_ms: one Python call each, back to back (host call overhead included); "
                  "*_graph: the same calls captured in a CUDA graph and replayed (device time per call; the "
                  f"{bytes_1 / 1e6:.1f} MB working set stays in L2 across calls); *_cold: one call after a 256 MB "
                  "write that flushes L2, events around the call alone",
        "split_kernel": axgb.get_kernel_choice(M, 1),
        "split": e_s, "fp64": e_d,
        "conservation_split": axgb.check_conservation(M, x32[0], y32[0])["relative_error"],
        "conservation_fp64": axgb.check_conservation(M, x64[0], y64[0])["relative_error"]}
    return out


def weightgen_c384(md_0p25, latlon_g):
    import torch

    import axgb
    from axgb import grids
    c384 = grids.cubed_sphere(384)
    # cold: both meshes ingested and prepared from host arrays, then generated once
    ll = latlon_g if latlon_g is not None else grids.latlon_deg(0.25)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    m_src, m_dst = axgb.Mesh.from_grid(ll), axgb.Mesh.from_grid(c384)
    axgb.generate_weights(m_src, m_dst, {"method": "conservative"})
    t_cold = time.perf_counter() - t0
    del m_src, m_dst
    t0 = time.perf_counter()
    mc = axgb.Mesh.from_grid(c384)
    t_ingest = time.perf_counter() - t0
    times = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        Mc = axgb.generate_weights(md_0p25, mc, {"method": "conservative"})
        times.append(time.perf_counter() - t0)
        st = Mc.stats()
    tb = time.perf_counter()
    Mb = axgb.generate_weights(md_0p25, mc, {"method": "bilinear"})
    t_bil = time.perf_counter() - tb
    best = min(times)
    return {"seconds_best": best, "seconds_first": times[0], "ingest_s": t_ingest, "nnz": Mc.nnz,
            "seconds_cold": t_cold, "cold": "both meshes ingested from host arrays (node vectors, cell prep) "
                                            "and one generation, timed together",
            "pairs_per_s": Mc.nnz / best, "candidates_per_s": st["gated_pairs"] / best,
            "bvh_candidates": st["bvh_candidates"], "gated": st["gated_pairs"],
            "stages_ms": {k: st[k] for k in st if k.startswith("t_")}, "bilinear_s": t_bil, "bilinear_nnz": Mb.nnz}


if __name__ == "__main__":
    sys.exit(main())
