"""Benchmark: Mcell-iter/s of the LU-SGS pseudo-iteration on one GB300.

A step is one pseudo-iteration (update%timeinteg + resi%residual of kwonhwi1/3dcode,
src/solve_module.f90:134-136) over the whole synthetic workload.  The default workload is
the large turbulent cavitating case as stated: 384x192x192 cells (14.16 M), stretched wall
grid, k-omega SST, IAPWS water/vapour with Merkle cavitation, BDF2 dual time, decomposed
along i into 16 blocks -- the
reference's MPI decomposition with one block per rank (src/grid_module.f90:95-116), which
the CPU arm runs with one block per host thread.  Both arms run the same blocks, so the
same block-Jacobi LU-SGS operator.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--precision fp64|mixed]
                  [--case large] [--blocks 16] [--impl gb300|reference]

value      device-resident throughput: K graph replays timed with CUDA events on the
           engine's stream; the working set (~20 GB) is far larger than L2, so no flush.
e2e        the same metric through the C ABI as a Fortran caller that keeps the state on
           the host would use it: each step uploads pv and the BDF history qq from pinned
           host buffers for all blocks in one call (dv and tv follow on the device from
           the EOS and the eddy viscosity, cfd3d_upload_primitives_all), iterates, and
           downloads pv, dv and tv of all blocks (cfd3d_download_state_all); the
           host<->device copies are inside the timed region.
roofline   the whole pseudo-iteration: algorithmic bytes per cell-iteration (persisted
           pv/dv/tv, metrics, LU-SGS intermediates, BDF history, rcav; 1040 B for this
           case) x cells / time, against the measured HBM copy bandwidth; beside it the
           residual kernel k_rhs alone and the measured FP64 peak (cfd3d_fp64_peak).
cpu_baseline  the CPU oracle (C++ FP64 restatement of the reference, its speed build) on a
           bounded sample of the same workload: the same 16 blocks, two iterations, one
           block per host thread.
N > 1      replicas: one independent engine per GPU (the case does not shard without
           changing the block-Jacobi operator); barrier + max over ranks; value is the sum.
"""
import argparse
import concurrent.futures as cf
import json
import os
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mcell-iter/s per GB300, mixed vs FP64 form at stated error; % HBM peak"
UNIT = "Mcell-iter/s"


# DRAM bytes per cell of one k_rhs launch, dram__bytes_read.sum + dram__bytes_write.sum
# of a one-pass ncu capture of the mixed form on the large case itself (14155776 cells, the
# launch list of one pseudo-iteration), divided by the cells
RHS_TRAFFIC_PER_CELL = (19.984210e9 + 11.177800e9) / 14155776
# the same for the whole pseudo-iteration: dram read + write summed over its 22 launches
ITER_TRAFFIC_PER_CELL = (72.270140e9 + 33.714040e9) / 14155776


def algorithmic_bytes(cfg):
    """Bytes per cell-iteration of the persisted-state model (FP64 words)."""
    from cfd3d_gb300.abi import sizes
    npv, ntv, nqq, ngrd = sizes(cfg)
    ndv = 18
    words = 2 * (npv + ndv + ntv) + (9 + ngrd) + 4 * npv + nqq * npv + (2 if cfg.get("ncav", 0) else 0)
    return 8 * words


def rhs_bytes(cfg, mixed):
    """Algorithmic bytes per cell of the residual kernel k_rhs in the LU-SGS iteration (each
    datum once per cell).  FP64 form -- reads: the cell's + face fluxes (inviscid and
    viscous), pv, dv, tv, its + face vectors, volume and wall distance, the BDF history, dt;
    writes: the residual, icav, itt, the omega bound, rcav and the 66-value FP64 sweep
    record.  Mixed form -- reads: the FP32 fluxes, pv, dv, tv, the volume, the BDF history,
    dt, the free-stream closure, the FP32 shadow of the SST variables and the FP32 metrics
    (+ face vectors, volume, wall distance); writes: the omega bound, rcav, the 74-value FP32
    tile record and the FP32 own part x0 (the residual, icav and itt stay in registers)."""
    from cfd3d_gb300.abi import sizes
    npv, ntv, nqq, ngrd = sizes(cfg)
    vis = cfg.get("iturb", 0) != -3
    sst = cfg.get("iturb", 0) == 0
    cav = cfg.get("ncav", 0) != 0
    ndv = 18
    if not mixed:
        rd = 3 * (2 if vis else 1) * npv * 8 + 8 * npv + 8 * ndv + 8 * ntv + 8 * (9 + 2) + 8 * nqq * npv + 8
        wr = 8 * npv + 8 * (4 + 4 + 1 + 2) + 8 * 66
        return rd + wr
    rd = (3 * (2 if vis else 1) * npv * 4 + 8 * npv + 8 * ndv + 8 * ntv + 8 + 8 * nqq * npv + 8 + 8 * npv
          + (4 * 5 if sst else 0) + 4 * (9 + 2))
    wr = (8 if sst else 0) + (16 if cav else 0) + 4 * 74 + 4 * npv
    return rd + wr


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


def workload(name, scale=1, blocks=1, cfl=None, prec=None):
    """The benchmark case: the named configuration (the intended cavitation clamp; the
    reference's temperature-indexed one diverges from a cavitating start), cut along i
    into `blocks` blocks."""
    from cfd3d_gb300 import cases
    c = cases.make(name, scale=scale)
    c["cfg"]["fix_cav_clamp"] = 1
    if cfl is not None:
        c["cfg"]["cfl"] = cfl
    if prec is not None:
        c["cfg"]["prec"] = prec
    if blocks > 1 and len(c["blocks"]) == 1:
        c = cases.split_i(c, blocks)
    return c


def describe(c, ncell):
    cfg = c["cfg"]
    return (f"{c['name']}: {ncell} cells in {len(c['blocks'])} blocks, prec={cfg.get('prec')}, cfl={cfg.get('cfl')}, "
            f"nsteady={cfg.get('nsteady', 0)}, iturb={cfg.get('iturb')}, ncav={cfg.get('ncav', 0)}")


def oracle_sample(c, threads):
    """The CPU oracle's speed build on the case, one block per host thread (the reference's
    MPI ranks); the blocks are initialised in parallel (ctypes releases the interpreter)."""
    from oracle import oracle_py
    nb = len(c["blocks"])
    o = oracle_py.Oracle(c, threads=min(threads, nb), fast=True)

    def init(n):
        o._L.orc_initialize(o.h, n, oracle_py._p(np.ascontiguousarray(c["pv0"][n], dtype=np.float64)))

    with cf.ThreadPoolExecutor(max(1, min(threads, nb))) as ex:
        list(ex.map(init, range(nb)))
    return o


def cpu_baseline(c, ncell, threads, iters=2):
    """Oracle throughput on a bounded sample of the same workload: the same blocks, a few
    pseudo-iterations."""
    o = oracle_sample(c, threads)
    o.iterate(1, 1, 0.0)
    t0 = time.perf_counter()
    for it in range(iters):
        o.iterate(1, it + 2, 0.0)
    dt = time.perf_counter() - t0
    nb = len(c["blocks"])
    return {"value": ncell * iters / dt / 1e6, "unit": UNIT, "cores": min(threads, nb), "kind": "port",
            "sample": f"{describe(c, ncell)}; {iters} pseudo-iterations after 1 untimed, CPU oracle (C++ FP64 "
                      f"restatement of the reference, -O3 build), one block per thread, {dt:.2f} s"}


def run_reference(args):
    """--impl reference: the reference's algorithm on the host cores (the CPU oracle's
    speed build) on the GPU arm's workload, one block per host thread; one untimed
    iteration warms the caches (the GPU arm's warm-up iterations build graphs and tune
    launch shapes, which the CPU has no counterpart of)."""
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from cfd3d_gb300 import cases
    threads = args.ref_threads or host_threads()
    c = workload(args.case, args.scale, args.blocks, args.cfl, args.prec)
    ncell = cases.total_cells(c)
    o = oracle_sample(c, threads)
    for w in range(min(args.warmup, 1)):
        o.iterate(1, w + 1, 0.0)
    t0 = time.perf_counter()
    for s in range(args.steps):
        o.iterate(1, s + 2, 0.0)
    dt = time.perf_counter() - t0
    value = ncell * args.steps / dt / 1e6
    cores = min(threads, len(c["blocks"]))
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": min(args.warmup, 1), "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": describe(c, ncell), "cells": ncell, "blocks": len(c["blocks"])},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                         "sample": f"the whole workload every step ({args.steps} pseudo-iterations after "
                                   f"{min(args.warmup, 1)} untimed), CPU oracle (C++ FP64 restatement, -O3 "
                                   f"build), one block per thread = one reference MPI rank per core"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def residual_error(res_a, res_b):
    """max over cells of |R_a - R_b| / max |R_b|, per variable (max over blocks)"""
    per = None
    for ra, rb in zip(res_a, res_b):
        sc = np.maximum(np.abs(rb).max(axis=(0, 1, 2)), 1e-300)
        ev = (np.abs(ra - rb) / sc).max(axis=(0, 1, 2))
        per = ev if per is None else np.maximum(per, ev)
    return per


def field_error(emx, e64, nblocks):
    """max over interior cells of |pv_mixed - pv_fp64| / max |pv_fp64|, per variable"""
    per = None
    for n in range(nblocks):
        a = emx.download(n)["pv"][3:-3, 3:-3, 3:-3]
        b = e64.download(n)["pv"][3:-3, 3:-3, 3:-3]
        sc = np.maximum(np.abs(b).max(axis=(0, 1, 2)), 1e-300)
        ev = (np.abs(a - b) / sc).max(axis=(0, 1, 2))
        per = ev if per is None else np.maximum(per, ev)
    return per


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


def run_e2e(eng, case, steps, it0):
    """The drop-in mode: per step, pv and qq up from pinned host memory (dv, tv derived on
    the device), one iteration, pv, dv, tv down.  Returns (ms per step, H2D, D2H bytes).
    The host arrays are carved from one pinned arena (2 MiB-aligned views): on a host whose
    memory is fragmented, dozens of separately pinned arrays measured the device-to-host
    copies 40 % slower than one pinned allocation."""
    import torch
    states = [eng.download(n) for n in range(len(case["blocks"]))]
    keys = [k for k in ("pv", "dv", "tv", "qq")
            if not ((k == "qq" and not eng.nqq) or (k == "tv" and eng.ntv == 0))]
    align = (2 << 20) // 8
    words = sum(-(-st[k].size // align) * align for st in states for k in keys)
    arena_t = torch.empty(words, dtype=torch.float64, pin_memory=True)
    arena = arena_t.numpy()
    bufs = []
    h2d = d2h = 0
    off = 0
    for st in states:
        keep = {}
        for k in keys:
            src = np.ascontiguousarray(st[k])
            a = arena[off:off + src.size].reshape(src.shape)
            off += -(-src.size // align) * align
            a[...] = src
            keep[k] = (arena_t, a)
            if k in ("pv", "qq"):
                h2d += a.nbytes
            if k != "qq":
                d2h += a.nbytes
        bufs.append(keep)
    d2h += 8 * eng.npv   # the residual norms

    pv_l = [keep["pv"][1] for keep in bufs]
    qq_l = [keep["qq"][1] for keep in bufs] if eng.nqq else None
    dv_l = [keep["dv"][1] for keep in bufs]
    tv_l = [keep["tv"][1] for keep in bufs] if eng.ntv else None

    def step(s):
        eng.upload_primitives_all(pv_l, qq_l)
        eng.iterate(1, it0 + s, 0.0)
        eng.download_state_all(pv_l, dv_l, tv_l)

    step(0)                                   # untimed: first touch of the pinned pages
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in range(steps):
        step(s + 1)
    return (time.perf_counter() - t0) / steps * 1e3, h2d, d2h


def batched_leg(args):
    """The 24 uneven blocks (~12 M cells) of the batched configuration in one launch per
    stage: mixed form, its per-iteration roofline, and the plain FP64 form beside it."""
    from cfd3d_gb300 import abi, cases, native
    c = workload("batched")
    ncell = cases.total_cells(c)
    eng = native.Engine(c, precision=abi.MIXED)
    eng.initialize(c["pv0"])
    for w in range(3):
        eng.iterate(1, w + 1, 0.0)
    shapes = eng.autotune(3) if not args.no_autotune else None
    ms = eng.time_iterate(args.batched_steps) / args.batched_steps
    eng.close()
    e64 = native.Engine(c, precision=abi.FP64)
    e64.initialize(c["pv0"])
    for w in range(2):
        e64.iterate(1, w + 1, 0.0)
    ms64 = e64.time_iterate(3) / 3
    e64.close()
    peak, _ = measured_peaks()
    bpc = algorithmic_bytes(c["cfg"])
    gbs = ncell * bpc / (ms * 1e-3) / 1e9
    return {"workload": describe(c, ncell), "cells": ncell, "blocks": len(c["blocks"]),
            "value": ncell / ms / 1e3, "ms_per_step": ms, "steps": args.batched_steps,
            "roofline": {"achieved": gbs, "peak": peak, "unit": "GB/s", "frac": gbs / peak, "bytes_per_cell": bpc},
            "fp64_form": {"value": ncell / ms64 / 1e3, "ms_per_step": ms64, "steps": 3},
            "launch_shapes": None if shapes is None else list(shapes)}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--case", default="large")
    ap.add_argument("--scale", type=int, default=1)
    ap.add_argument("--blocks", type=int, default=16,
                    help="blocks along i (the reference's MPI decomposition); both arms run them")
    ap.add_argument("--cfl", type=float, default=None)
    ap.add_argument("--prec", type=int, default=None, help="preconditioning speed (the case's own by default)")
    ap.add_argument("--precision", default="mixed", choices=["fp64", "mixed"])
    ap.add_argument("--fp64-steps", type=int, default=3,
                    help="iterations of the plain FP64 form timed beside the mixed form (0 skips)")
    ap.add_argument("--field-iters", type=int, default=20,
                    help="iterations after which the mixed form's state is compared with the FP64 form's (0 skips)")
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--ref-threads", type=int, default=0, help="host threads of the CPU samples (0: all)")
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--batched-steps", type=int, default=10, help="timed iterations of the 24-block leg (0 skips)")
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
    case = workload(args.case, args.scale, args.blocks, args.cfl, args.prec)
    cfg = case["cfg"]
    nb = len(case["blocks"])
    prec = abi.MIXED if args.precision == "mixed" else abi.FP64
    import torch
    free0 = torch.cuda.mem_get_info(local)[0]
    t_setup = time.perf_counter()
    eng = native.Engine(case, precision=prec)
    t_create = time.perf_counter()
    device_gb = (free0 - torch.cuda.mem_get_info(local)[0]) / 1e9
    eng.initialize(case["pv0"])
    t_init = time.perf_counter()
    ncell = cases.total_cells(case)
    res0 = [eng.residual(n)["res"] for n in range(nb)] if prec == abi.MIXED else None
    for w in range(args.warmup):
        eng.iterate(1, w + 1, 0.0)
    if not args.no_autotune:
        eng.autotune(3)
    shapes = eng.launch_shapes()
    if dist:
        dist.barrier()
    with ClockSampler(local) as clk:
        ms = eng.time_iterate(args.steps)
    ms_step, value = combine_ranks(ms / args.steps, ncell, dist)
    stats = eng.stats()
    prof = eng.profile_iterate()
    it_next = args.warmup + args.steps + 2
    e2e = None
    if args.e2e_steps > 0:
        e2e_ms, h2d, d2h = run_e2e(eng, case, args.e2e_steps, it_next)
        e2e_ms, e2e_value = combine_ranks(e2e_ms, ncell, dist)
        e2e = {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
               "ms_per_step": e2e_ms, "steps": args.e2e_steps}
    if rank != 0:
        dist.barrier()
        return 0
    fp64_tflops = native.fp64_peak(1.0)
    conv = native.convert_rate()
    peak, peak_kind = measured_peaks()
    bpc = algorithmic_bytes(cfg)
    achieved_it = ncell * bpc / (ms_step * 1e-3) / 1e9
    # the residual kernel k_rhs (the 'residual' stage is that one launch), timed with CUDA
    # events on the engine's stream by profile_iterate
    rb = rhs_bytes(cfg, prec == abi.MIXED)
    rhs_ms = prof["residual"]
    achieved_rhs = ncell * rb / (rhs_ms * 1e-3) / 1e9
    total_stage = sum(prof.values())
    dominant = max(prof, key=prof.get)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if prec == abi.FP64 else "f32+f64", "data": "synthetic",
        "config": {"workload": describe(case, ncell), "cells": ncell, "precision": args.precision, "blocks": nb,
                   "l2": "working set >> 129 MB L2 (no flush needed)", "parallelism": "replicas" if ws > 1 else "1 GPU",
                   "launch_shapes": {"face_threads": shapes[0], "rhs_threads": shapes[1],
                                     "sweep_ctas_per_sm": shapes[2], "face_residual_pipeline_groups": shapes[3],
                                     "autotuned": not args.no_autotune}},
        "roofline": {"bound": "hbm", "achieved": achieved_it, "peak": peak, "unit": "GB/s", "frac": achieved_it / peak,
                     "peak_kind": peak_kind,
                     "traffic": ITER_TRAFFIC_PER_CELL * ncell if (prec == abi.MIXED and args.case == "large") else None,
                     "scope": "whole pseudo-iteration: algorithmic bytes per cell-iteration x cells / ms_per_step",
                     "bytes_per_cell": bpc, "dominant_stage": dominant,
                     "dominant_share": prof[dominant] / total_stage, "stage_ms": prof,
                     "kernel": {"name": "k_rhs (residual, sources, sweep records)", "achieved": achieved_rhs,
                                "frac": achieved_rhs / peak, "kernel_ms": rhs_ms, "algorithmic_bytes_per_cell": rb,
                                "traffic": RHS_TRAFFIC_PER_CELL * ncell if (prec == abi.MIXED and args.case == "large") else None},
                     "fp64": {"peak_tflops": fp64_tflops,
                              "peak_kind": "measured: cfd3d_fp64_peak, independent DFMA chains, 1 s",
                              "conversions_gps": {k: round(v, 1) for k, v in conv.items()},
                              "conversions_kind": "measured: cfd3d_convert_rate, float <-> double by the "
                                                  "hardware (FP64 pipe) and on the integer pipes"}},
        "e2e": e2e,
        "gpu_launches": stats["launches_per_iter"] * args.steps,
        "setup_s": {"create": t_create - t_setup, "initialize": t_init - t_create,
                    "what": "cfd3d_create (metrics, wall distance, boundary program, tiles, device buffers) "
                            "and cfd3d_initialize (state upload and EOS) of the mixed engine",
                    "device_gb": device_gb},
        "clocks": clk.summary(),
    }
    if prec == abi.MIXED and (args.fp64_steps > 0 or args.field_iters > 0):
        e64 = native.Engine(case, precision=abi.FP64)
        e64.initialize(case["pv0"])
        err = residual_error(res0, [e64.residual(n)["res"] for n in range(nb)])
        line["mixed_residual_error"] = {
            "max": float(err.max()), "per_variable": [float(x) for x in err],
            "definition": "max over cells of |R_mixed - R_fp64| / max |R_fp64|, per variable and block, initial state"}
        if args.fp64_steps > 0:
            for w in range(2):
                e64.iterate(1, w + 1, 0.0)
            ms64 = e64.time_iterate(args.fp64_steps) / args.fp64_steps
            line["fp64_form"] = {"value": ws * ncell / ms64 / 1e3, "ms_per_step": ms64, "steps": args.fp64_steps}
            line["speedup_vs_fp64"] = value / line["fp64_form"]["value"]
        if args.field_iters > 0:
            eng.initialize(case["pv0"])
            e64.initialize(case["pv0"])
            for it in range(args.field_iters):
                eng.iterate(1, it + 1, 0.0)
                e64.iterate(1, it + 1, 0.0)
            ferr = field_error(eng, e64, nb)
            line["mixed_field_error"] = {
                "max": float(ferr.max()), "per_variable": [float(x) for x in ferr], "iterations": args.field_iters,
                "definition": "max over interior cells of |pv_mixed - pv_fp64| / max |pv_fp64|, per variable, "
                              "after the stated pseudo-iterations from the same initial state"}
        e64.close()
    eng.close()
    if args.batched_steps > 0 and args.case == "large" and args.scale == 1:
        line["batched"] = batched_leg(args)
    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(case, ncell, args.ref_threads or host_threads())
    print(json.dumps(line), flush=True)
    if dist:
        dist.barrier()
    return 0


if __name__ == "__main__":
    sys.exit(main())
