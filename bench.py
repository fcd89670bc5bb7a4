"""Benchmark: Mcell-iter/s of the LU-SGS pseudo-iteration on one GB300.

A step is one pseudo-iteration (update%timeinteg + resi%residual of kwonhwi1/3dcode,
src/solve_module.f90:134-136) over the whole synthetic workload.  The default workload is
the large turbulent cavitating case: 384x192x192 cells (14.16 M), stretched wall grid,
k-omega SST, IAPWS water/vapour with Merkle cavitation, BDF2 dual time.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
                  [--case large] [--impl gb300|reference]

value      device-resident throughput: K graph replays timed with CUDA events on the
           engine's stream; the working set (~20 GB) is far larger than L2, so no flush.
e2e        the same metric through the C ABI as a Fortran caller that owns its arrays would
           use it: each step uploads pv/dv/tv/qq from pinned host buffers, iterates, and
           downloads pv/dv/tv (host<->device copies inside the timed region).
roofline   algorithmic bytes per cell-iteration (persisted pv/dv/tv, metrics, LU-SGS
           intermediates, BDF history, rcav; 1040 B for this case) x cells / time, against
           the measured HBM copy bandwidth; per-stage times come from an event-instrumented
           iteration.
cpu_baseline  the CPU oracle (C++ FP64 restatement of the reference) on a bounded sample
           of the same workload (the case at 1/2 resolution), cut into one block per host
           thread -- the reference's MPI decomposition, one rank per core.
N > 1      replicas: one independent engine per GPU (the case does not shard without
           changing the block-Jacobi operator); barrier + max over ranks; value is the sum.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-iter/s per GB300, mixed vs FP64 form at stated error; % HBM peak"
UNIT = "Mcell-iter/s"


def algorithmic_bytes(cfg):
    """Bytes per cell-iteration of the persisted-state model (FP64 words)."""
    from cfd3d_gb300.abi import sizes
    npv, ntv, nqq, ngrd = sizes(cfg)
    ndv = 18
    words = 2 * (npv + ndv + ntv) + (9 + ngrd) + 4 * npv + nqq * npv + (2 if cfg.get("ncav", 0) else 0)
    return 8 * words


def rhs_bytes(cfg, mixed):
    """Algorithmic bytes per cell of the residual kernel k_rhs (each datum once per cell):
    reads -- the cell's + face fluxes (inviscid and viscous), pv (and the FP32 shadow of
    the SST gradients), dv, tv, its + face vectors, volume and wall distance (and their FP32
    copy), the BDF history, dt; writes -- residual, the sweep record (66 FP64 values, and 34
    FP32 in the mixed form), icav, itt, the omega bound, rcav."""
    from cfd3d_gb300.abi import sizes
    npv, ntv, nqq, ngrd = sizes(cfg)
    vis = cfg.get("iturb", 0) != -3
    fw = 4 if mixed else 8
    rd = 3 * (2 if vis else 1) * npv * fw + 8 * npv + 8 * 18 + 8 * ntv + 8 * (9 + 2) + 8 * nqq * npv + 8
    if mixed:
        rd += 4 * 5 + 4 * (9 + 2)
    wr = 8 * npv + 8 * 66 + (4 * 34 if mixed else 0) + 8 * (4 + 4 + 1 + 2)
    return rd + wr


# DRAM traffic of k_rhs per cell measured by ncu (dram__bytes_read.sum + dram__bytes_write.sum)
# on the large case at 1/2 resolution, mixed form: 2.300 GB + 3.389 GB over 1769472 cells
# (profiles/k_rhs_large_half_mixed.md); it grows with the cell count
RHS_TRAFFIC_PER_CELL = (2.300200e9 + 3.388917e9) / 1769472


def measured_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        self.lines = []
        if self.proc is not None:
            self.proc.terminate()
            try:
                out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()
                out = ""
            self.lines = [l for l in out.splitlines() if l.strip()]

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for l in getattr(self, "lines", []):
            f = [x.strip() for x in l.split(",")]
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except Exception:
                continue
            for n, v in zip(names, f[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def host_threads():
    """host cores this process may run on"""
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def reference_sample(case_name, scale, threads):
    """The CPU oracle on the workload at 1/scale resolution, cut into `threads` blocks
    along i and run one block per thread: the reference's MPI decomposition, one rank per
    host core."""
    from cfd3d_gb300 import cases
    from oracle import oracle_py
    c = cases.make(case_name, scale=scale)
    c["cfg"]["fix_cav_clamp"] = 1
    if threads > 1 and len(c["blocks"]) == 1:
        c = cases.split_i(c, threads)
    nb = len(c["blocks"])
    o = oracle_py.Oracle(c, threads=min(threads, nb))
    o.initialize(c["pv0"])
    return o, cases.total_cells(c), nb


def cpu_baseline(case_name, scale, threads, iters=2):
    """Oracle throughput on a bounded sample of the same workload."""
    o, ncell, nb = reference_sample(case_name, scale, threads)
    o.iterate(1, 1, 0.0)
    t0 = time.perf_counter()
    for it in range(iters):
        o.iterate(1, it + 2, 0.0)
    dt = time.perf_counter() - t0
    return {"value": ncell * iters / dt / 1e6, "unit": UNIT, "cores": min(threads, nb), "kind": "port",
            "sample": f"{case_name} at 1/{scale} resolution ({ncell} cells) in {nb} blocks, {iters} "
                      f"pseudo-iterations, CPU oracle (C++ FP64 restatement of the reference), one block "
                      f"per thread, {dt:.2f} s"}


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores (CPU oracle), the
    workload at 1/ref_scale resolution decomposed over all host threads."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    threads = args.ref_threads or host_threads()
    o, ncell, nb = reference_sample(args.case, args.ref_scale, threads)
    for w in range(args.warmup):
        o.iterate(1, w + 1, 0.0)
    t0 = time.perf_counter()
    for s in range(args.steps):
        o.iterate(1, args.warmup + s + 1, 0.0)
    dt = time.perf_counter() - t0
    value = ncell * args.steps / dt / 1e6
    cores = min(threads, nb)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"{args.case} at 1/{args.ref_scale} resolution ({ncell} cells) in {nb} blocks",
                   "cells": ncell},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"{args.case} at 1/{args.ref_scale} resolution, {nb} blocks along i, "
                                   f"{args.steps} pseudo-iterations per run, CPU oracle (C++ FP64 restatement), "
                                   f"one block per thread = one reference MPI rank per core"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def fp64_form(case, res_mixed, steps, ncell, ws):
    """The plain all-FP64 form on the same workload: its throughput, and the error of the
    mixed form's residual on the initial state, max over cells of |R_mixed - R_fp64|
    divided by the largest |R_fp64| of the same variable and block."""
    from cfd3d_gb300 import abi, native
    e64 = native.Engine(case, precision=abi.FP64)
    e64.initialize(case["pv0"])
    err = 0.0
    per_var = None
    for n, rm in enumerate(res_mixed):
        r64 = e64.residual(n)["res"]
        sc = np.maximum(np.abs(r64).max(axis=(0, 1, 2)), 1e-300)
        ev = (np.abs(rm - r64) / sc).max(axis=(0, 1, 2))
        per_var = ev if per_var is None else np.maximum(per_var, ev)
    err = float(per_var.max())
    for w in range(2):
        e64.iterate(1, w + 1, 0.0)
    ms = e64.time_iterate(steps) / steps
    e64.close()
    return {"fp64_form": {"value": ws * ncell / ms / 1e3, "ms_per_step": ms, "steps": steps},
            "mixed_residual_error": {"max": err, "per_variable": [float(x) for x in per_var],
                                     "definition": "max over cells of |R_mixed - R_fp64| / max |R_fp64|, "
                                                   "per variable and block, initial state"}}


def combine_ranks(ms_step, ncell, dist=None):
    """Replicas: the slowest rank's time per step, and the whole job's throughput
    (every rank advances its own copy of the workload) in Mcell-iter/s."""
    ws = 1
    if dist is not None:
        import torch
        t = torch.tensor([ms_step], dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        ms_step = float(t.item())
        ws = dist.get_world_size()
    return ms_step, ws * ncell / ms_step / 1e3


def pinned(shape):
    import torch
    t = torch.empty(int(np.prod(shape)), dtype=torch.float64, pin_memory=True)
    return t, t.numpy().reshape(shape)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--case", default="large")
    ap.add_argument("--scale", type=int, default=1)
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=5,
                    help="iterations of the plain FP64 form timed beside the mixed form (0 skips)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-scale", type=int, default=2,
                    help="the CPU samples run the workload at 1/ref-scale resolution")
    ap.add_argument("--ref-threads", type=int, default=0, help="host threads of the CPU samples (0: all)")
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch shapes")
    args = ap.parse_args()

    if args.impl == "reference":
        return run_reference(args)

    ws, rank, local = dist_env()
    dist = None
    if ws > 1:
        import torch.distributed as dist_mod
        dist = dist_mod
        dist.init_process_group("gloo")
    from cfd3d_gb300 import abi, cases, native
    native.set_device(local)
    case = cases.make(args.case, scale=args.scale)
    case["cfg"]["fix_cav_clamp"] = 1
    cfg = case["cfg"]
    prec = abi.MIXED if args.precision == "mixed" else abi.FP64
    eng = native.Engine(case, precision=prec)
    eng.initialize(case["pv0"])
    ncell = cases.total_cells(case)
    res0 = [eng.residual(n)["res"] for n in range(len(case["blocks"]))] if prec == abi.MIXED else None
    for w in range(args.warmup):
        eng.iterate(1, w + 1, 0.0)
    shapes = eng.autotune(3) if not args.no_autotune else None
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms = eng.time_iterate(args.steps)
    ms_step, value = combine_ranks(ms / args.steps, ncell, dist)
    stats = eng.stats()
    prof = eng.profile_iterate()
    # ---- end to end through the C ABI with pinned host buffers
    blocks = case["blocks"]
    bufs = []
    h2d = d2h = 0
    for n, b in enumerate(blocks):
        st = eng.download(n)
        keep = {}
        for k in ("pv", "dv", "tv", "qq"):
            if k == "qq" and not eng.nqq:
                continue
            arr = st[k] if k != "tv" else st["tv"]
            if k == "tv" and eng.ntv == 0:
                continue
            t, a = pinned(np.ascontiguousarray(arr).shape)
            a[...] = arr
            keep[k] = (t, a)
            h2d += a.nbytes
            if k != "qq":
                d2h += a.nbytes
        bufs.append(keep)
    d2h += 8 * eng.npv
    import torch

    def e2e_step(s):
        for n, keep in enumerate(bufs):
            eng.upload(n, pv=keep["pv"][1], dv=keep["dv"][1], tv=keep["tv"][1] if "tv" in keep else None,
                       qq=keep["qq"][1] if "qq" in keep else None)
        eng.iterate(1, args.warmup + s + 1, 0.0)
        for n, keep in enumerate(bufs):
            eng.download_arrays(n, pv=keep["pv"][1], dv=keep["dv"][1], tv=keep["tv"][1] if "tv" in keep else None)

    e2e_step(0)                                   # untimed: first touch of the pinned pages
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(args.e2e_steps):
        e2e_step(s + 1)
    e2e_ms, e2e_value = combine_ranks((time.perf_counter() - t0) / args.e2e_steps * 1e3, ncell, dist)
    if rank != 0:
        dist.barrier()
        return 0
    peak, peak_kind = measured_peaks()
    bpc = algorithmic_bytes(cfg)
    achieved_it = ncell * bpc / (ms_step * 1e-3) / 1e9
    # the dominant kernel: k_rhs (the 'residual' stage is that one launch), timed with CUDA
    # events on the engine's stream by profile_iterate
    rb = rhs_bytes(cfg, prec == abi.MIXED)
    rhs_ms = prof["residual"]
    achieved = ncell * rb / (rhs_ms * 1e-3) / 1e9
    total_stage = sum(prof.values())
    dominant = max(prof, key=prof.get)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == abi.FP64 else "f32+f64", "data": "synthetic",
        "config": {"workload": f"{args.case}: {ncell} cells, SST + IAPWS + Merkle, BDF2, LU-SGS",
                   "cells": ncell, "precision": args.precision, "blocks": len(blocks),
                   "l2": "working set >> 129 MB L2 (no flush needed)", "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "launch_shapes": None if shapes is None else {"face_threads": shapes[0], "rhs_threads": shapes[1],
                                                                 "sweep_ctas_per_sm": shapes[2]}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": peak_kind,
                     "traffic": RHS_TRAFFIC_PER_CELL * ncell if prec == abi.MIXED else None,
                     "kernel": "k_rhs (residual, sources, sweep records)", "kernel_ms": rhs_ms,
                     "algorithmic_bytes_per_cell": rb,
                     "note": "FP64-pipe bound, not HBM bound: see the ncu summaries",
                     "iteration": {"achieved": achieved_it, "frac": achieved_it / peak,
                                   "bytes_per_cell": bpc, "dominant_stage": dominant,
                                   "dominant_share": prof[dominant] / total_stage, "stage_ms": prof}},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "gpu_launches": stats["launches_per_iter"] * args.steps,
        "clocks": clk.summary(),
    }
    if prec == abi.MIXED and args.fp64_steps > 0:
        line.update(fp64_form(case, res0, args.fp64_steps, ncell, ws))
        line["speedup_vs_fp64"] = value / line["fp64_form"]["value"]
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(args.case, args.ref_scale, args.ref_threads or host_threads())
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
