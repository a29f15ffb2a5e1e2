#!/usr/bin/env python3
"""Benchmark of the matrix-free SIPG DG operator on GB300.

Headline workload (one "step" = one FP64 jacobian_apply over the whole
grid): 3D SIPG diffusion, QkDG degree 2 (27 DoF/cell) on a 64^3 structured
grid (7,077,888 DoF), cellwise log-normal K = exp(g), g ~ N(0,1) seeded,
Dirichlet boundary, alpha = 3 (sigma = 3 k (k+d-1)).  Metric: GDoF/s.

Also reported on the same line: the end-to-end number through the C ABI
with host buffers (H2D input, D2H result every step), the roofline of the
operator kernel (FP64 pipe; measured DFMA peak), the CPU baseline (the
oracle restating the reference's loop structure, one core), the solve
metrics of the same problem (time to 1e-10 relative residual for the FP64
CG + cell-block-Jacobi solve and for the FP32-apply / FP64-defect-correction
solve, and the adjoint gradient cost relative to one forward solve), and the
same two solves on the 96^3 Q3 grid (56.6M DoF, box-filtered log-normal K)
with the errors of the mixed solution against the FP64 one.

``--impl reference`` times the reference's CPU algorithm (the oracle port:
PDELab itself cannot be built here) on all host cores for the same
workload and metric.
"""
from __future__ import annotations

import argparse
import ctypes
import functools
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "dune-pdelab_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "GDoF/s matrix-free SIPG apply; time-to-1e-10 solve, mixed vs FP64 on GB300; grad/solve"
WORKLOAD = dict(dim=3, degree=2, cells=64, alpha=3.0, seed=2)
DATA = "synthetic (seeded log-normal K per cell, x ~ U(-1,1))"


def flops_per_cell(dim, N, mass_factored=False):
    """FP64/FP32 arithmetic of one cell in the operator kernel as written:
    d-direction 1D operators + tangential mass contractions (8 N^4 MAC in
    3D, 4 N^3 in 2D; 6 N^4 in the mass-factored 3D FP64 kernel, three
    directional applies of Mhat^-1 A'_dir and one Mhat (x) Mhat (x) Mhat)
    plus neighbour traces and face expansions (4 d N^d MAC); one MAC =
    2 flops."""
    if dim == 3:
        mac = (6 if mass_factored else 8) * N ** 4 + 12 * N ** 3
    else:
        mac = 4 * N ** 3 + 8 * N ** 2
    return 2 * mac


def quadrature_flops_per_dof(dim, N):
    """Sum-factorised count of the reference algorithm (volume at quadrature
    points + both-sided face quadrature): 8 d N^{d+1} + 16 d^2 N^d per cell."""
    return (8 * dim * N ** (dim + 1) + 16 * dim * dim * N ** dim) / N ** dim


class ClockSampler:
    """nvidia-smi clock/throttle sampling during the timed region."""

    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index, period_ms=50):
        self.index, self.period_ms = index, period_ms
        self.proc = None
        self.f = None

    def __enter__(self):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", str(self.period_ms)],
                stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *exc):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
        self.f.close()

    def summary(self):
        rows = []
        try:
            for line in open(self.f.name):
                parts = [p.strip() for p in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        finally:
            os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None, "reasons": reasons,
                "samples": len(rows),
                "power_w_max": max((float(r[3]) for r in rows
                                    if r[3].replace(".", "").isdigit()), default=None)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


# ---- replicas on N GPUs: host logic shared by the arms ---------------------
# The path does not shard across GPUs here (one GPU per box): every rank runs
# the whole workload as an independent replica; the job's time is that of its
# slowest rank and its throughput counts the units of all ranks.
def max_over_ranks(x, world, device=None):
    """Maximum of x over the ranks (float; x itself when world == 1)."""
    if world == 1:
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_throughput(world, units_per_rank, seconds):
    """Whole-job rate: the units of all ranks over the slowest rank's time."""
    return world * units_per_rank / seconds


def gather_checksums(value, world, device=None):
    """All ranks' checksums of their replica results (a list of floats)."""
    if world == 1:
        return [float(value)]
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    out = [torch.zeros_like(t) for _ in range(world)]
    dist.all_gather(out, t)
    return [float(o.item()) for o in out]


def make_problem(pdg, np, device, wl=WORKLOAD):
    n = wl["cells"]
    go = pdg.GridOperator(wl["dim"], wl["degree"], (n,) * wl["dim"], alpha=wl["alpha"],
                          device=device)
    rng = np.random.default_rng(wl["seed"])
    logK = rng.standard_normal(go.ncell)
    go.set_permeability(logK, is_log=True)
    if wl.get("convection"):
        # the convection-diffusion-reaction operator of the 48^3 Q4 leg:
        # upwind b = curl of a seeded 8-mode Fourier potential, c = 1
        go.set_reaction(np.ones(go.ncell))
        go.set_velocity_modes(pdg.fourier_velocity_modes(5))
    return go, logK


def link_bandwidth(torch, dev, xh, yh, reps=10):
    """Pinned host<->device copy rates (GB/s) for one step's vectors: each
    direction alone, and each way while both run at once on two streams."""
    dx = torch.empty(xh.numel(), dtype=xh.dtype, device=dev)
    dy = torch.empty(yh.numel(), dtype=yh.dtype, device=dev)
    s1, s2 = torch.cuda.Stream(dev), torch.cuda.Stream(dev)
    nbytes = xh.numel() * xh.element_size()

    def both():
        cur = torch.cuda.current_stream(dev)
        s1.wait_stream(cur)
        s2.wait_stream(cur)
        with torch.cuda.stream(s1):
            dx.copy_(xh, non_blocking=True)
        with torch.cuda.stream(s2):
            yh.copy_(dy, non_blocking=True)
        cur.wait_stream(s1)
        cur.wait_stream(s2)

    out = {}
    for name, fn in (("h2d", lambda: dx.copy_(xh, non_blocking=True)),
                     ("d2h", lambda: yh.copy_(dy, non_blocking=True)),
                     ("concurrent_each_way", both)):
        for _ in range(2):
            fn()
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(reps):
            fn()
        e1.record()
        torch.cuda.synchronize()
        out[name] = nbytes / (e0.elapsed_time(e1) / reps * 1e-3) / 1e9
    return out


def fma_peaks(pdg):
    import build_lib
    lib = ctypes.CDLL(build_lib.PROBE_LIB)
    lib.pdg_probe_fma_peak.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    out = {}
    for prec, name, iters in ((0, "fp64", 2000), (1, "fp32", 20000)):
        best = 0.0
        for _ in range(3):
            v = ctypes.c_double()
            if lib.pdg_probe_fma_peak(prec, iters, ctypes.byref(v)) == 0:
                best = max(best, v.value)
        out[name] = best
    # the FP64 tensor-core path (mma.sync m8n8k4 f64), for comparison only
    lib.pdg_probe_dmma_peak.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    best = 0.0
    for _ in range(3):
        v = ctypes.c_double()
        if lib.pdg_probe_dmma_peak(1000, ctypes.byref(v)) == 0:
            best = max(best, v.value)
    out["fp64_tensor_mma"] = best
    # both at once: the sum of the two rates if the tensor path were a second
    # FP64 unit, either one's rate if they share it
    lib.pdg_probe_fp64_mixed.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
    best = 0.0
    for _ in range(3):
        v = ctypes.c_double()
        if lib.pdg_probe_fp64_mixed(1000, ctypes.byref(v)) == 0:
            best = max(best, v.value)
    out["fp64_mma_plus_fma"] = best
    return out


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            return json.load(f)
    except OSError:
        return {}


def profile_traffic(key, what=None):
    """DRAM bytes per launch from the committed ncu summary, if present
    (what="captured": when and from which capture)."""
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as f:
            d = json.load(f)
    except (OSError, ValueError):
        return None
    if what == "captured":
        return d.get("_captured", {}).get(key)
    return d.get(key)


def cpu_baseline_port(np, wl=WORKLOAD, applies=2):
    import pdg_oracle as O
    n = wl["cells"]
    rng = np.random.default_rng(wl["seed"])
    P = O.Problem(wl["dim"], wl["degree"], (n,) * wl["dim"], alpha=wl["alpha"])
    P.set(K=np.exp(rng.standard_normal(P.ncell)))
    x = np.random.default_rng(1).uniform(-1, 1, P.ndof)
    y = np.zeros(P.ndof)
    t0 = time.perf_counter()
    for _ in range(applies):
        P.jacobian_apply(x, y)
    dt = time.perf_counter() - t0
    return {"value": P.ndof * applies / dt / 1e9, "unit": "GDoF/s", "cores": 1, "kind": "port",
            "sample": f"{applies} full FP64 jacobian_apply of the {n}^3 Q{wl['degree']} grid "
                      f"({P.ndof} DoF) by the oracle's reference-faithful loops, "
                      f"{dt:.1f} s on one core"}


# --------------------------------------------------------------------------
# reference arm: the oracle port on all host cores
# --------------------------------------------------------------------------
_W = {}


def _ref_worker_init(wl, shm_x, ndof):
    import numpy as np
    from multiprocessing import shared_memory
    import pdg_oracle as O
    n = wl["cells"]
    rng = np.random.default_rng(wl["seed"])
    P = O.Problem(wl["dim"], wl["degree"], (n,) * wl["dim"], alpha=wl["alpha"])
    P.set(K=np.exp(rng.standard_normal(P.ncell)))
    sx = shared_memory.SharedMemory(name=shm_x)
    _W.update(P=P, sx=sx, x=np.ndarray((ndof,), dtype=np.float64, buffer=sx.buf))


def _ref_worker_apply(args):
    import numpy as np
    from multiprocessing import shared_memory
    b, e, shm_y, ndof = args
    sy = shared_memory.SharedMemory(name=shm_y)
    y = np.ndarray((ndof,), dtype=np.float64, buffer=sy.buf)
    y[:] = 0.0
    _W["P"].jacobian_apply_range(_W["x"], y, b, e)
    del y
    sy.close()
    return 0


def run_reference(args, world, rank):
    import multiprocessing as mp
    from multiprocessing import shared_memory
    import numpy as np
    import pdg_oracle as O
    if rank != 0:
        return
    O.build()
    wl = WORKLOAD
    n = wl["cells"]
    ncell = n ** wl["dim"]
    ndof = ncell * (wl["degree"] + 1) ** wl["dim"]
    cores = os.cpu_count() or 1
    sx = shared_memory.SharedMemory(create=True, size=ndof * 8)
    x = np.ndarray((ndof,), dtype=np.float64, buffer=sx.buf)
    x[:] = np.random.default_rng(1).uniform(-1, 1, ndof)
    sys_ = [shared_memory.SharedMemory(create=True, size=ndof * 8) for _ in range(cores)]
    ys = [np.ndarray((ndof,), dtype=np.float64, buffer=s.buf) for s in sys_]
    bounds = np.linspace(0, ncell, cores + 1).astype(int)
    jobs = [(int(bounds[i]), int(bounds[i + 1]), sys_[i].name, ndof) for i in range(cores)]
    ctx = mp.get_context("spawn")
    y = np.zeros(ndof)
    with ctx.Pool(cores, initializer=_ref_worker_init, initargs=(wl, sx.name, ndof)) as pool:
        def step():
            pool.map(_ref_worker_apply, jobs, chunksize=1)
            np.sum(ys, axis=0, out=y)
        for _ in range(args.warmup):
            step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            step()
        dt = time.perf_counter() - t0
    del x, ys
    sx.close(); sx.unlink()
    for s in sys_:
        s.close(); s.unlink()
    value = ndof * args.steps / dt / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": DATA,
        "config": {"workload": f"sipg3d_q{wl['degree']}_{n}^3_f64_apply", "ndof": ndof,
                   "cells": ncell, "degree": wl["degree"], "alpha": wl["alpha"],
                   "l2": "n/a (host memory)", "parallelism": f"{cores} host processes"},
        "impl": "reference",
        "cpu_baseline": {"value": value, "unit": "GDoF/s", "cores": cores, "kind": "port",
                         "sample": f"{args.steps} full FP64 jacobian_apply of the {n}^3 grid, "
                                   f"cells split over {cores} processes, partial results "
                                   f"summed (oracle restating the reference's loops; PDELab "
                                   f"itself needs the DUNE core modules, absent here)"},
        "e2e": {"value": value, "unit": "GDoF/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


# --------------------------------------------------------------------------
# GB300 arm
# --------------------------------------------------------------------------
def run_gb300(args, world, rank, local):
    import numpy as np
    import torch
    import __graft_entry__
    if rank == 0:
        __graft_entry__.build()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
        dist.barrier()
        __graft_entry__.build()
    import pdg
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    stream = torch.cuda.Stream(device=dev)
    go, logK = make_problem(pdg, np, local)
    go.set_stream(stream)
    if args.solves_only:
        if rank == 0:
            print(json.dumps(solve_metrics(pdg, np, torch, go, stream, logK)), flush=True)
        go.close()
        return
    op = pdg.OnTheFlyOperator(go)
    ndof, ncell = go.ndof, go.ncell
    N = WORKLOAD["degree"] + 1
    f32 = args.precision == "f32"
    dt_ = torch.float32 if f32 else torch.float64
    esz = 4 if f32 else 8
    # rotating input/output pairs so that every step streams from HBM
    npairs = max(2, min(16, int(4 * 129e6 / (2 * esz * ndof)) + 1))
    gen = torch.Generator(device=dev).manual_seed(1)
    xs = [(torch.rand(ndof, dtype=torch.float64, device=dev, generator=gen) * 2 - 1).to(dt_)
          for _ in range(npairs)]
    ys = [torch.zeros(ndof, dtype=dt_, device=dev) for _ in range(npairs)]
    torch.cuda.synchronize()
    step_fn = (lambda x, y: go.jacobian_apply_f32(x, y)) if f32 else op.apply
    if args.step == "prec":
        # profiling runs: the FDM block-Jacobi apply in the step's precision
        prec = pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_FDM,
                                              precision=pdg.F32 if f32 else pdg.F64)
        prec.pre()
        step_fn = lambda x, y: prec.apply(y, x)

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            step_fn(xs[i % npairs], ys[i % npairs])
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        with ClockSampler(local) as clk:
            barrier()
            torch.cuda.synchronize()
            e0.record(stream)
            for i in range(args.steps):
                step_fn(xs[i % npairs], ys[i % npairs])
            e1.record(stream)
            torch.cuda.synchronize()
            barrier()
        ms = e0.elapsed_time(e1) / args.steps
    ms = max_over_ranks(ms, world, dev)
    value = job_throughput(world, ndof, ms * 1e-3) / 1e9
    clocks = clk.summary()
    # replicas compute the same apply: their results must agree bit for bit
    sums = gather_checksums(float(ys[0].double().sum().item()), world, dev)
    replicas_identical = all(x == sums[0] for x in sums)

    # the same applies in float-pair arithmetic (a separately labelled mode:
    # FP64 values as pairs of floats on the FP32 pipe)
    float_pair = None
    if not f32 and args.step == "apply" and WORKLOAD["dim"] == 3:
        float_pair = float_pair_metrics(pdg, torch, go, op, xs, ys, stream, args, npairs)
    # the transposed apply (the operator of the adjoint solves)
    transpose = None
    if not f32 and args.step == "apply":
        transpose = transpose_metrics(torch, go, xs, ys, stream, args, npairs)

    # end to end through the public API with host (pinned) buffers
    xh = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
    yh = torch.empty(ndof, dtype=torch.float64, pin_memory=True)
    xh.copy_(xs[0].double().cpu())
    for _ in range(max(1, args.warmup)):
        op.apply(xh, yh)
    barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        op.apply(xh, yh)       # H2D x, kernel, D2H y, synchronise
    t_e2e = time.perf_counter() - t0
    t_e2e = max_over_ranks(t_e2e, world, dev)
    e2e = {"value": job_throughput(world, ndof * args.steps, t_e2e) / 1e9, "unit": "GDoF/s",
           "h2d_bytes_per_step": ndof * 8, "d2h_bytes_per_step": ndof * 8,
           # the host link's rates for these buffers: the copies of a step
           # overlap the kernel, so e2e is bound by max(kernel, copies) + edges
           "link_gbs": link_bandwidth(torch, dev, xh, yh)}

    if rank != 0:
        go.close()
        if world > 1:
            torch.distributed.destroy_process_group()
        return

    peaks = fma_peaks(pdg) if not args.no_probe else {"fp64": None, "fp32": None}
    mp_ = measured_peaks()
    # the FP64 apply of this step runs the mass-factored kernel (non-transposed)
    fl = flops_per_cell(3, N, mass_factored=not f32) * ncell
    achieved = fl / (ms * 1e-3) / 1e12
    alg_bytes = 2 * esz * ndof + esz * ncell
    pk = peaks["fp32" if f32 else "fp64"]
    wname = (f"{'cdr' if WORKLOAD.get('convection') else 'sipg'}3d_q{WORKLOAD['degree']}_"
             f"{WORKLOAD['cells']}^3_{args.precision}_apply")
    roofline = {
        "bound": "fp32" if f32 else "fp64", "achieved": achieved, "peak": pk,
        "unit": "TFLOP/s", "frac": achieved / pk if pk else None,
        "traffic": profile_traffic(wname),
        "traffic_source": profile_traffic(wname, "captured"),
        "peak_source": "measured in this run: FMA throughput microbenchmark of the CUDA "
                       "cores (libpdg_probe.so); MEASURED_PEAKS.json has no FP64/FP32 "
                       "CUDA-core figure",
        "flops_per_launch": fl, "flops_per_dof": fl / ndof,
        "reference_algorithm_flops_per_dof": quadrature_flops_per_dof(3, N),
        "algorithmic_bytes_per_launch": alg_bytes,
        "hbm_achieved_gbs": alg_bytes / (ms * 1e-3) / 1e9,
        "hbm_peak_gbs": mp_.get("hbm_gbs"),
        "hbm_frac": (alg_bytes / (ms * 1e-3) / 1e9) / mp_["hbm_gbs"] if mp_.get("hbm_gbs") else None,
        "fp32_fma_peak_tflops": peaks["fp32"],
        "fp64_tensor_mma_peak_tflops": peaks.get("fp64_tensor_mma"),
        "fp64_mma_plus_fma_tflops": peaks.get("fp64_mma_plus_fma"),
    }

    extras = {}
    if not args.no_solves:
        extras = solve_metrics(pdg, np, torch, go, stream, logK)
    # the configurations' legs: C1 (2D Q1 solve beside the CPU solve), C3
    # (96^3 Q3 mixed vs FP64), C4 (64^3 Q2 adjoint checks) and C5 (48^3 Q4
    # convection-diffusion-reaction solves and gradients) are on the default
    # line; --legs picks a subset, --extended adds the block-preconditioner
    # and assembled-matrix legs
    if args.legs is not None:
        legs = set(args.legs.split(","))          # explicit legs run regardless
    else:
        legs = set() if args.no_solves else {"c1", "c3", "c4", "c5"}
    if args.extended:
        legs |= {"prec", "asm"}
    if legs:
        for leg, key, fn in (("c1", "solve_q1_2d_64", c1_metrics),
                             ("c3", "solve_q3_96", c3_metrics), ("c4", "adjoint_q2_64", c4_metrics),
                             ("c5", "cdr_q4_48", c5_metrics), ("prec", "block_prec_q2_64", prec_metrics),
                             ("asm", "assembled_q2_32", assembled_metrics)):
            if leg not in legs:
                continue
            if leg == "c3" and (args.c3_cells or args.c3_mixed_only):
                fn = functools.partial(fn, n=args.c3_cells or 96, mixed_only=args.c3_mixed_only)
            try:
                extras[key] = fn(pdg, np, torch, stream)
            except Exception as exc:   # report the failing leg, keep the others
                extras[key] = {"error": f"{type(exc).__name__}: {exc}"}
    cpu = cpu_baseline_port(np, WORKLOAD) if not args.no_cpu else None
    go.close()
    line = {
        "metric": METRIC, "value": value, "unit": "GDoF/s", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": args.precision,
        "data": DATA,
        "config": {"workload": wname, "ndof": ndof, "cells": ncell,
                   "degree": WORKLOAD["degree"], "alpha": 3.0,
                   "l2": f"{npairs} rotating x/y pairs ({npairs * 2 * esz * ndof / 1e6:.0f} MB "
                         f"> 129 MB L2)",
                   "parallelism": f"replicas x{world}"},
        "e2e": e2e, "gpu_launches": args.steps, "clocks": clocks, "roofline": roofline,
        "replicas_identical": replicas_identical,
        "cpu_baseline": cpu,
    }
    if float_pair:
        # the float-pair kernel's FP64 algorithm (the three-operator form, 8 N^4
        # volume MAC per cell), on the FP64 pipe's scale
        fl_fp = flops_per_cell(3, N) * ncell
        float_pair["fp64_equivalent_tflops"] = fl_fp / (float_pair["ms_per_apply"] * 1e-3) / 1e12
        if peaks["fp64"]:
            float_pair["fp64_equivalent_over_fp64_peak"] = (
                float_pair["fp64_equivalent_tflops"] / peaks["fp64"])
        float_pair["traffic"] = profile_traffic(wname.replace("_apply", "_float_pair_apply"))
        line["f64_float_pair"] = float_pair
    if transpose:
        line["transpose_apply"] = transpose
    line.update(extras)
    print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def float_pair_metrics(pdg, torch, go, op, xs, ys, stream, args, npairs):
    """The headline applies with pdg_set_f64_arithmetic(PDG_F64_FLOAT_PAIR):
    time per apply (CUDA events over the same rotating buffers and step
    count) and the max-norm difference to the native FP64 result of the same
    input, relative to its largest entry."""
    ndof = go.ndof
    ref = ys[0].clone()
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    try:
        with torch.cuda.stream(stream):
            for i in range(args.warmup):
                op.apply(xs[i % npairs], ys[i % npairs])
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for i in range(args.steps):
                op.apply(xs[i % npairs], ys[i % npairs])
            e1.record(stream)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1) / args.steps
            yfp = torch.zeros_like(ref)
            op.apply(xs[0], yfp)
            torch.cuda.synchronize()
    finally:
        go.set_f64_arithmetic(pdg.F64_NATIVE)
    return {"mode": "float pairs (hi + lo floats, 48 bits) on the FP32 pipe; not the headline",
            "ms_per_apply": ms, "gdofs": ndof / (ms * 1e-3) / 1e9,
            "rel_diff_vs_native_f64": float((yfp - ref).abs().max() / ref.abs().max())}


def transpose_metrics(torch, go, xs, ys, stream, args, npairs):
    """The transposed FP64 apply y += J^T x over the same rotating buffers and
    step count (CUDA events), and the transpose identity <J^T x, w> = <x, J w>
    at full size, relative to |J^T x| |w|."""
    ndof = go.ndof
    with torch.cuda.stream(stream):
        for i in range(args.warmup):
            go.jacobian_apply_transpose(xs[i % npairs], ys[i % npairs])
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for i in range(args.steps):
            go.jacobian_apply_transpose(xs[i % npairs], ys[i % npairs])
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1) / args.steps
        x, w = xs[0], xs[1]
        jtx = torch.zeros_like(x)
        jw = torch.zeros_like(x)
        go.jacobian_apply_transpose(x, jtx)
        go.jacobian_apply(w, jw)
        torch.cuda.synchronize()
    a, b = float(torch.dot(jtx, w)), float(torch.dot(x, jw))
    return {"form": "y += J^T x (accumulating), the adjoint solves' operator",
            "ms_per_apply": ms, "gdofs": ndof / (ms * 1e-3) / 1e9,
            "identity_rel": abs(a - b) / float(jtx.norm() * w.norm())}


def _event_ms(torch, stream, fn, reps=5):
    """Median CUDA-event time of fn() on the stream, after one warm-up call."""
    fn()
    times = []
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        fn()
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    times.sort()
    return times[len(times) // 2]


def prec_metrics(pdg, np, torch, stream):
    """64^3 Q2 (7.08M DoF), log-normal K, f = 1: each block preconditioner's
    set-up and apply time and the BiCGStab solve it gives (reduction 1e-10)."""
    n = 64
    dev = stream.device
    go = pdg.GridOperator(3, 2, (n, n, n), alpha=3.0, device=dev.index or 0)
    go.set_stream(stream)
    rng = np.random.default_rng(7)
    go.set_permeability(rng.standard_normal(go.ncell), is_log=True)
    go.set_source(fc=np.ones(go.ncell))
    out = {"workload": "sipg3d_q2_64^3 (7.08M DoF), BiCGStab, reduction 1e-10",
           "sor_hyperplane_steps": 3 * n - 2}
    # block-solver options of the reference's matrix-free test
    # (matrix_free_linear.ini: block_inverse_solver reduction 1e-14, maxiter 100)
    go.set_prec_options(block_reduction=1e-14, block_maxit=100)
    out["block_solver"] = {"reduction": 1e-14, "maxit": 100}
    d = torch.rand(go.ndof, dtype=torch.float64, device=dev)
    v = torch.zeros_like(d)
    kinds = (("bj_fdm", pdg.PREC_BJ_FDM), ("bj_dense", pdg.PREC_BJ_DENSE),
             ("bj_iterative", pdg.PREC_BJ_ITERATIVE),
             ("sor_dense", pdg.PREC_SOR | pdg.PREC_BJ_DENSE),
             ("sor_fdm", pdg.PREC_SOR | pdg.PREC_BJ_FDM),
             ("sor_iterative", pdg.PREC_SOR | pdg.PREC_BJ_ITERATIVE))
    for name, kind in kinds:
        rec = {}
        try:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pdg._check(pdg.load().pdg_prec_setup(go.handle, kind, pdg.F64))
            torch.cuda.synchronize()
            rec["setup_s"] = time.perf_counter() - t0
            rec["apply_ms"] = _event_ms(torch, stream, lambda: pdg._check(
                pdg.load().pdg_prec_apply(go.handle, d.data_ptr(), v.data_ptr())))
            if kind & 15 == pdg.PREC_BJ_ITERATIVE:
                its = go.prec_block_iterations()
                rec["block_iterations_mean"] = float(its.mean())
                rec["block_iterations_max"] = int(its.max())
            ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB, preconditioner=kind,
                                                     maxiter=20000)
            u = torch.zeros(go.ndof, dtype=torch.float64, device=dev)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
            torch.cuda.synchronize()
            r = ls.result()
            rec.update({"solve_s": time.perf_counter() - t0, "iterations": r.iterations,
                        "converged": bool(r.converged)})
        except Exception as exc:
            rec["error"] = f"{type(exc).__name__}: {exc}"
        out[name] = rec
    go.close()
    return out


def assembled_metrics(pdg, np, torch, stream):
    """32^3 Q2 (884,736 DoF): the Jacobian assembled on the device by probing,
    the BCRS block product against the matrix-free apply, and the
    matrix-based vs matrix-free CG solve (reduction 1e-10)."""
    n = 32
    dev = stream.device
    go = pdg.GridOperator(3, 2, (n, n, n), alpha=3.0, device=dev.index or 0)
    go.set_stream(stream)
    rng = np.random.default_rng(8)
    go.set_permeability(rng.standard_normal(go.ncell), is_log=True)
    go.set_source(fc=np.ones(go.ncell))
    out = {"workload": "sipg3d_q2_32^3 (884,736 DoF), CG + block Jacobi (FDM), reduction 1e-10"}
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    go.jacobian_assemble()
    torch.cuda.synchronize()
    out["assemble_s"] = time.perf_counter() - t0
    nnzb = go.jacobian_pattern()
    out["nnz_blocks"] = nnzb
    out["matrix_bytes"] = go.ncell * 7 * 27 * 27 * 8
    x = torch.rand(go.ndof, dtype=torch.float64, device=dev)
    y = torch.zeros_like(x)
    out["matrix_apply_ms"] = _event_ms(torch, stream, lambda: go.matrix_apply(x, y))
    out["matrix_apply_gbs"] = out["matrix_bytes"] / (out["matrix_apply_ms"] * 1e-3) / 1e9
    out["matrix_free_apply_ms"] = _event_ms(torch, stream, lambda: pdg._check(
        pdg.load().pdg_apply(go.handle, x.data_ptr(), y.data_ptr())))
    for assembled in (0, 1):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG)
        ls.opts.assembled = assembled
        u = torch.zeros(go.ndof, dtype=torch.float64, device=dev)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
        torch.cuda.synchronize()
        r = ls.result()
        key = "matrix_based" if assembled else "matrix_free"
        out[f"{key}_solve_s"] = time.perf_counter() - t0
        out[f"{key}_iterations"] = r.iterations
    go.close()
    return out


C1_SEED = 1


def c1_problem(pdg, np, device):
    """2D SIPG Poisson, Q1 on 64^2 cells of the unit square, K = 1, alpha = 3
    (sigma = 3 k (k+d-1) = 6), homogeneous Dirichlet, f = sin(2 pi x)
    sin(2 pi y) + eps_cell at the volume quadrature points, eps_cell i.i.d.
    normal with variance 0.01 (N(mu, sigma^2) read as sigma^2 = 0.01, so
    standard deviation 0.1), seeded.  Returns the GridOperator and f."""
    n = 64
    go = pdg.GridOperator(2, 1, (n, n), alpha=3.0, device=device)
    vp = go.volume_points()
    eps = np.random.default_rng(C1_SEED).normal(0.0, 0.1, go.ncell)
    fq = np.sin(2 * np.pi * vp[..., 0]) * np.sin(2 * np.pi * vp[..., 1]) + eps[:, None]
    go.set_source(fq=fq)
    return go, fq


def c1_metrics(pdg, np, torch, stream):
    """The 2D Q1 64^2 problem: the GPU's CG + cell-block Jacobi solve to 1e-10
    (FP64) beside the oracle's full CPU solve of the same problem on one
    core (the reference's sequential path restated)."""
    import pdg_oracle as O
    go, fq = c1_problem(pdg, np, stream.device.index or 0)
    go.set_stream(stream)
    out = {"workload": "sipg2d_q1_64^2 (16,384 DoF), K=1, f=sin(2 pi x)sin(2 pi y)+N(0,0.1^2) "
                       "per cell, CG + cell-block Jacobi (FDM), reduction 1e-10"}
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, preconditioner=pdg.PREC_BJ_FDM)
    for rep in range(2):       # the first run includes the preconditioner set-up
        u = torch.zeros(go.ndof, dtype=torch.float64, device=stream.device)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        slp.apply()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
        out["gpu_first_solve_s" if rep == 0 else "gpu_solve_s"] = dt
    r = slp.result()
    out["gpu_iterations"] = r.iterations
    out["gpu_converged"] = bool(r.converged)
    go.close()
    P = O.Problem(2, 1, (64, 64), alpha=3.0, fq=fq)
    t0 = time.perf_counter()
    uref, res, st = P.solve(solver="cg", op=0, reduction=1e-10)
    out["cpu_solve_s"] = time.perf_counter() - t0
    out["cpu_iterations"] = res.iterations
    out["cpu_cores"] = 1
    un = u.cpu().numpy()
    out["gpu_vs_cpu_rel_max"] = float(np.max(np.abs(un - uref)) / np.max(np.abs(uref)))
    out["speedup_gpu_vs_cpu"] = out["cpu_solve_s"] / out["gpu_solve_s"]
    return out


def smoothed_logK(np, n, seed=3, sigma=1.5):
    """Log-permeability of the 96^3 Q3 workload: i.i.d. N(0,1) per cell,
    3x3x3-cell box filter (zero-flux edges: the window is clipped at the
    boundary), rescaled to standard deviation sigma."""
    g = np.random.default_rng(seed).standard_normal((n, n, n))   # [z][y][x]
    pad = np.pad(g, 1, mode="edge")
    s = np.zeros_like(g)
    for dz in range(3):
        for dy in range(3):
            for dx in range(3):
                s += pad[dz:dz + n, dy:dy + n, dx:dx + n]
    s /= 27.0
    s = (s - s.mean()) / s.std() * sigma
    return np.ascontiguousarray(s.ravel())


def c3_metrics(pdg, np, torch, stream, inner_reduction=1e-4, n=96, mixed_only=False):
    """96^3 Q3 (56.6M DoF): FP64 CG + block Jacobi vs FP32-apply / FP64
    defect correction, both to 1e-10, f = 1; errors of the mixed solution
    against the FP64 one.  Profiling runs may size the grid (n) and run the
    mixed solve alone."""
    go = pdg.GridOperator(3, 3, (n, n, n), alpha=3.0, device=stream.device.index or 0)
    go.set_stream(stream)
    go.set_permeability(smoothed_logK(np, n), is_log=True)
    go.set_source(fc=np.ones(go.ncell))
    out = {"workload": "sipg3d_q3_96^3 (56.6M DoF), log-normal K box-filtered, sigma_g=1.5, "
                       "f=1, CG + cell-block Jacobi (FDM), reduction 1e-10"}
    if n != 96:
        out["workload"] = out["workload"].replace("96^3 (56.6M DoF)", f"{n}^3")
    sols = {}
    for mixed in ((True,) if mixed_only else (True, False)):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, mixed=mixed, maxiter=20000,
                                                 inner_reduction=inner_reduction)
        u = torch.zeros(go.ndof, dtype=torch.float64, device=stream.device)
        pdg.GridOperatorPreconditioner(go, precision=pdg.F32 if mixed else pdg.F64).pre()
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        slp.apply()
        dt = time.perf_counter() - t0
        r = slp.result()
        key = "mixed" if mixed else "fp64"
        sols[key] = u
        out[f"{key}_s"] = dt
        out[f"{key}_iterations"] = r.iterations
        out[f"{key}_converged"] = bool(r.converged)
        if mixed:
            out["mixed_outer_iterations"] = r.outer_iterations
    if mixed_only:
        go.close()
        return out
    e = sols["mixed"] - sols["fp64"]
    out["speedup_mixed_vs_fp64"] = out["fp64_s"] / out["mixed_s"]
    out["mixed_vs_fp64_rel_l2"] = float(torch.linalg.norm(e) / torch.linalg.norm(sols["fp64"]))
    out["mixed_vs_fp64_rel_max"] = float(e.abs().max() / sols["fp64"].abs().max())
    # the FP64 solve again with the operator applies in float-pair arithmetic
    # (a separately labelled mode; the FP64 baseline above stays native)
    go.set_f64_arithmetic(pdg.F64_FLOAT_PAIR)
    try:
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, maxiter=20000)
        u = torch.zeros(go.ndof, dtype=torch.float64, device=stream.device)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        slp.apply()
        dt = time.perf_counter() - t0
    finally:
        go.set_f64_arithmetic(pdg.F64_NATIVE)
    e = u - sols["fp64"]
    out["fp64_float_pair_s"] = dt
    out["fp64_float_pair_iterations"] = slp.result().iterations
    out["fp64_float_pair_converged"] = bool(slp.result().converged)
    out["fp64_float_pair_vs_fp64_rel_l2"] = float(torch.linalg.norm(e) /
                                                  torch.linalg.norm(sols["fp64"]))
    go.close()
    return out


def c4_metrics(pdg, np, torch, stream, ndirs=16):
    """Adjoint on 64^3 Q2: J = 1/2 |u - u_obs|^2, u_obs = u(target log K) + 1%
    noise; the autograd gradient against central differences (h = 1e-6) along
    16 seeded directions, and (on a 16^3 grid) against the oracle's gradient
    from the assembled CPU Jacobian transpose."""
    import pdg_torch
    out = {}
    for n, check in ((64, "fd"), (16, "jt")):
        rng = np.random.default_rng(40 + n)
        go = pdg.GridOperator(3, 2, (n, n, n), alpha=3.0, device=stream.device.index or 0)
        go.set_stream(stream)
        go.set_source(fc=np.ones(go.ncell))
        prob = pdg_torch.DGProblem(go, reduction=1e-11)
        logK_t = torch.tensor(rng.standard_normal(go.ncell), device=stream.device)
        u_obs = pdg_torch.solve_dg(logK_t, None, prob).detach()
        u_obs = u_obs * (1 + 0.01 * torch.tensor(rng.standard_normal(go.ndof), device=u_obs.device))
        logK = torch.tensor(rng.standard_normal(go.ncell), device=stream.device,
                            requires_grad=True)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        u = pdg_torch.solve_dg(logK, None, prob)
        torch.cuda.synchronize()
        t_fwd = time.perf_counter() - t0
        J = 0.5 * ((u - u_obs) ** 2).sum()
        t0 = time.perf_counter()
        J.backward()
        torch.cuda.synchronize()
        t_bwd = time.perf_counter() - t0
        g = logK.grad.detach()
        if check == "fd":
            h, errs = 1e-6, []
            with torch.no_grad():
                for _ in range(ndirs):
                    d = torch.tensor(rng.standard_normal(go.ncell), device=g.device)
                    Jp = 0.5 * ((pdg_torch.solve_dg(logK + h * d, None, prob) - u_obs) ** 2).sum()
                    Jm = 0.5 * ((pdg_torch.solve_dg(logK - h * d, None, prob) - u_obs) ** 2).sum()
                    fd = float((Jp - Jm) / (2 * h))
                    ad = float((g * d).sum())
                    errs.append(abs(fd - ad) / abs(ad))
            out["grid_64"] = {"forward_solve_s": t_fwd, "adjoint_solve_plus_grad_s": t_bwd,
                              "grad_over_solve": t_bwd / t_fwd,
                              "total_over_solve": (t_fwd + t_bwd) / t_fwd,
                              "fd_directions": ndirs, "fd_h": h,
                              "fd_rel_err_max": max(errs), "fd_rel_err_median": float(np.median(errs))}
        else:
            import pdg_oracle as O
            K = np.exp(logK.detach().cpu().numpy())
            P = O.Problem(3, 2, (n, n, n), alpha=3.0, K=K, fc=np.ones(go.ncell))
            A = P.assemble_jacobian()
            un = u.detach().cpu().numpy()
            lam = np.zeros(go.ndof)
            lu, piv = P.lu(P.block_diagonal())
            st, res = P.krylov("cg", lam, un - u_obs.cpu().numpy(), 1e-13, maxit=50000, op=2,
                               blocks=A, lu=lu, piv=piv)
            gref = P.grad_logK(un, lam)
            gg = g.cpu().numpy()
            out["grid_16_assembled_transpose"] = {
                "rel_err_max": float(np.max(np.abs(gg - gref)) / np.max(np.abs(gref))),
                "oracle_cg_iterations": res.iterations}
        go.close()
    return out


C5_INNER_REDUCTION = 1e-1
C5_INNER_MAXIT = 50


def c5_metrics(pdg, np, torch, stream):
    """48^3 Q4 (13.8M DoF) convection-diffusion-reaction, upwind flux, b = curl
    of a seeded 8-mode Fourier potential (|b| <= 10), c = 1, log-normal K,
    f = 1, Dirichlet 0; BiCGStab + dense cell-block Jacobi, FP32 apply in FP64
    refinement vs FP64, reduction 1e-9; gradients w.r.t. log K and f vs central
    differences along 2 seeded directions each.  The mixed solve is FP64
    flexible GMRES around FP32 BiCGStab inner solves of reduction 1e-1 (at
    most 50 iterations each)."""
    import pdg_torch
    n = 48
    dev = stream.device
    go = pdg.GridOperator(3, 4, (n, n, n), alpha=3.0, device=dev.index or 0)
    go.set_stream(stream)
    rng = np.random.default_rng(5)
    logK0 = rng.standard_normal(go.ncell)
    go.set_permeability(logK0, is_log=True)
    go.set_reaction(np.ones(go.ncell))
    go.set_velocity_modes(pdg.fourier_velocity_modes(5))
    go.set_source(fc=np.ones(go.ncell))
    # the FP32 dense block inverses of the inner solves are stored in FP16
    go.set_prec_options(dense_fp16=1)
    out = {"workload": "sipg3d_q4_48^3 (13.8M DoF), upwind convection |b|<=10, c=1, "
                       "BiCGStab + dense cell-block Jacobi (FP16-stored in the FP32 inner "
                       "solves), reduction 1e-9"}
    sols = {}
    for mixed in (True, False):
        pdg.GridOperatorPreconditioner(go, kind=pdg.PREC_BJ_DENSE,
                                       precision=pdg.F32 if mixed else pdg.F64).pre()
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.BICGSTAB,
                                                 preconditioner=pdg.PREC_BJ_DENSE,
                                                 mixed=mixed, maxiter=20000,
                                                 inner_reduction=C5_INNER_REDUCTION)
        ls.opts.inner_maxit = C5_INNER_MAXIT
        ls.opts.max_outer = 60
        u = torch.zeros(go.ndof, dtype=torch.float64, device=dev)
        slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-9)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        slp.apply()
        dt = time.perf_counter() - t0
        r = slp.result()
        key = "mixed" if mixed else "fp64"
        sols[key] = u
        out[f"{key}_s"] = dt
        out[f"{key}_iterations"] = r.iterations
        out[f"{key}_converged"] = bool(r.converged)
        if mixed:
            out["mixed_outer_iterations"] = r.outer_iterations
    e = sols["mixed"] - sols["fp64"]
    out["speedup_mixed_vs_fp64"] = out["fp64_s"] / out["mixed_s"]
    out["mixed_vs_fp64_rel_l2"] = float(torch.linalg.norm(e) / torch.linalg.norm(sols["fp64"]))
    try:
        out["adjoint"] = _c5_gradients(pdg, pdg_torch, np, torch, go, dev, rng, logK0,
                                       sols["fp64"])
    except Exception as exc:
        out["adjoint"] = {"error": f"{type(exc).__name__}: {exc}"}
    go.close()
    return out


def _c5_gradients(pdg, pdg_torch, np, torch, go, dev, rng, logK0, u_ref):
    # mixed-precision solves to the configuration's 1e-9
    prob = pdg_torch.DGProblem(go, method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                               reduction=1e-9, inner_reduction=C5_INNER_REDUCTION,
                               inner_maxit=C5_INNER_MAXIT)
    sols = {"fp64": u_ref}
    u_obs = sols["fp64"] * (1 + 0.01 * torch.tensor(rng.standard_normal(go.ndof), device=dev))
    logK = torch.tensor(logK0 + 0.3 * rng.standard_normal(go.ncell), device=dev,
                        requires_grad=True)
    fc = torch.ones(go.ncell, dtype=torch.float64, device=dev, requires_grad=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = pdg_torch.solve_dg(logK, fc, prob)
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    J = 0.5 * ((u - u_obs) ** 2).sum()
    t0 = time.perf_counter()
    J.backward()
    torch.cuda.synchronize()
    t_bwd = time.perf_counter() - t0
    errs = {}
    h = 1e-6
    # the central differences need solves well below h * |grad|: reduction 1e-11
    fdp = pdg_torch.DGProblem(go, method=pdg.BICGSTAB, preconditioner=pdg.PREC_BJ_DENSE,
                              reduction=1e-11, inner_reduction=C5_INNER_REDUCTION,
                              inner_maxit=C5_INNER_MAXIT)
    with torch.no_grad():
        for name, grad in (("logK", logK.grad), ("f", fc.grad)):
            ee = []
            for _ in range(2):
                d = torch.tensor(rng.standard_normal(go.ncell), device=dev)
                if name == "logK":
                    Jp = 0.5 * ((pdg_torch.solve_dg(logK + h * d, fc, fdp) - u_obs) ** 2).sum()
                    Jm = 0.5 * ((pdg_torch.solve_dg(logK - h * d, fc, fdp) - u_obs) ** 2).sum()
                else:
                    Jp = 0.5 * ((pdg_torch.solve_dg(logK, fc + h * d, fdp) - u_obs) ** 2).sum()
                    Jm = 0.5 * ((pdg_torch.solve_dg(logK, fc - h * d, fdp) - u_obs) ** 2).sum()
                fd = float((Jp - Jm) / (2 * h))
                ad = float((grad * d).sum())
                ee.append(abs(fd - ad) / abs(ad))
            errs[name] = max(ee)
    return {"forward_solve_s": t_fwd, "adjoint_solve_plus_grads_s": t_bwd,
            "grad_over_solve": t_bwd / t_fwd, "reduction": 1e-9, "fd_h": h,
            "fd_solve_reduction": 1e-11,
            "fd_rel_err_max_logK": errs["logK"], "fd_rel_err_max_f": errs["f"]}


def solve_metrics(pdg, np, torch, go, stream, logK):
    """Time-to-1e-10 of the FP64 and the mixed-precision solve (f = 1), and
    the adjoint gradient cost relative to one forward solve."""
    out = {}
    go.set_source(fc=np.ones(go.ncell))
    res = {}
    for mixed in (False, True):
        ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, mixed=mixed)
        for rep in range(2):      # first run includes one-time set-up (preconditioner, r0)
            u = torch.zeros(go.ndof, dtype=torch.float64, device=stream.device)
            slp = pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10)
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            slp.apply()
            dt = time.perf_counter() - t0
        r = slp.result()
        res["mixed" if mixed else "fp64"] = (dt, r, u)
    (t64, r64, u64), (tmx, rmx, umx) = res["fp64"], res["mixed"]
    err = (umx - u64)
    out["solve"] = {
        "workload": "same grid and K, f = 1, CG + cell-block Jacobi (FDM), reduction 1e-10",
        "fp64_s": t64, "fp64_iterations": r64.iterations, "fp64_converged": bool(r64.converged),
        "mixed_s": tmx, "mixed_inner_iterations": rmx.iterations,
        "mixed_outer_iterations": rmx.outer_iterations, "mixed_converged": bool(rmx.converged),
        "speedup_mixed_vs_fp64": t64 / tmx,
        "mixed_vs_fp64_rel_l2": float(torch.linalg.norm(err) / torch.linalg.norm(u64)),
        "mixed_vs_fp64_rel_max": float(err.abs().max() / u64.abs().max()),
    }
    # adjoint: J = 1/2 |u - u_obs|^2, gradient w.r.t. log K
    rng = np.random.default_rng(5)
    u_obs = u64 * (1 + 0.01 * torch.tensor(rng.standard_normal(go.ndof), device=u64.device))
    opts = pdg.default_options(mixed=1)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    u = torch.zeros_like(u64)
    ls = pdg.ISTLBackend_SEQ_MatrixFree_Base(go, method=pdg.CG, mixed=True)
    pdg.StationaryLinearProblemSolver(go, ls, u, 1e-10).apply()
    torch.cuda.synchronize()
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    lam = torch.zeros_like(u)
    go.adjoint_solve(u - u_obs, lam, opts)
    g = torch.zeros(go.ncell, dtype=torch.float64, device=u.device)
    go.grad_logK(u, lam, g)
    torch.cuda.synchronize()
    t_adj = time.perf_counter() - t0
    out["adjoint"] = {"forward_solve_s": t_fwd, "adjoint_solve_plus_grad_s": t_adj,
                      "grad_over_solve": t_adj / t_fwd,
                      "total_over_solve": (t_fwd + t_adj) / t_fwd}
    return out


def main():
    ap = argparse.ArgumentParser(description=__doc__.split("\n")[0])
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["gb300", "reference"], default="gb300")
    ap.add_argument("--no-solves", action="store_true",
                    help="skip the 64^3 Q2 solve/adjoint metrics and the default legs")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--extended", action="store_true",
                    help="also run the block-preconditioner (prec) and assembled-matrix (asm) "
                         "legs")
    ap.add_argument("--legs", default=None,
                    help="configuration legs to run (default c1,c3,c4,c5, none with "
                         "--no-solves): c1 (2D Q1 64^2 solve and its CPU solve), c3 (96^3 Q3 "
                         "mixed vs FP64), c4 (64^3 Q2 adjoint checks), c5 (48^3 Q4 "
                         "convection-diffusion-reaction); prec, asm")
    ap.add_argument("--no-probe", action="store_true",
                    help="skip the FMA peak probe (profiling runs); roofline frac is then null")
    ap.add_argument("--solves-only", action="store_true",
                    help="run only the solve/adjoint metrics (profiling runs)")
    ap.add_argument("--cells", type=int, default=None, help="override cells per direction")
    ap.add_argument("--degree", type=int, default=None, help="override polynomial degree")
    ap.add_argument("--precision", choices=["f64", "f32"], default="f64",
                    help="operator precision of the timed steps")
    ap.add_argument("--step", choices=["apply", "prec"], default="apply",
                    help="profiling runs: time the FDM block-Jacobi apply instead of the "
                         "operator (the roofline fields then describe the operator only)")
    ap.add_argument("--c3-cells", type=int, default=None,
                    help="profiling runs: the C3 leg on an N^3 grid instead of 96^3")
    ap.add_argument("--c3-mixed-only", action="store_true",
                    help="profiling runs: the C3 leg's mixed-precision solve alone")
    ap.add_argument("--convection", action="store_true",
                    help="time the convection-diffusion-reaction operator (upwind velocity "
                         "and reaction of the 48^3 Q4 leg) instead of pure diffusion")
    args = ap.parse_args()
    if args.cells:
        WORKLOAD["cells"] = args.cells
    if args.degree:
        WORKLOAD["degree"] = args.degree
    if args.convection:
        WORKLOAD["convection"] = True
    if args.warmup < 3:
        args.warmup = 3
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        run_gb300(args, world, rank, local)


if __name__ == "__main__":
    main()
