#!/usr/bin/env python
"""Benchmark of the GB300 explicit residual-and-update path.

Metric: Mcell-residuals/s (one cell-residual = one residual evaluation of one
interior cell, its update included), FEST_MIXED (FP32 stencil arithmetic,
FP64 state/metrics/norm) with the FP64 rate and the mixed-vs-FP64 wall-Cp
difference reported beside it.

Workload (default): the smooth-bump channel, 256x96x4 cells, WENO5 + SLAU,
TVD-RK3 with local time steps, CFL 0.8; one step = one TVD-RK3 iteration
(3 cell-residuals per cell).  Inputs are synthetic (analytic grid, uniform
Mach 0.5 start).  L2 is flushed (256 MiB write) before every timed step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the CPU restatement of the reference's path (the
reference itself is Fortran+MPI and cannot be built on these machines) on
all host cores for a bounded number of the same steps.
With N > 1 (torchrun), every rank advances its own replica of the block
(replicas only: one block per GPU needs no exchange); value = all ranks'
cell-residuals / max rank time.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "fest-3d_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "Mcell-residuals/s (mixed precision; FP64 and mixed-vs-FP64 wall-Cp error reported)"
# algorithmic bytes per cell-residual of a fused mixed-precision stage, each
# array once, the grid metrics at the precision the grid is stored in (FP64):
# the FP32 stencil state (20 B), the FP64 state the update starts from (40),
# one I, J and K face record {A,nx,ny,nz} (96) and the volume (8) in; the FP64
# state (40) and its FP32 copy (20) out = 224 B in stage 1; stages 2-3 of
# TVD-RK3 also read U_store (40) = 264 B.  (The sweep reads FP32 copies of
# the metrics, 52 B fewer, and the time step, 8 B more; the FP64 figures are
# the compulsory traffic of the method.)
BYTES_STAGE = (224.0, 264.0, 264.0)
# iterations of the bump configuration's mixed-vs-FP64 report (its stated count)
C2_ITERS = 10000


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="bump", choices=["bump", "bump-512x192x16"],
                    help="bump: the headline 256x96x4 block; bump-512x192x16: the same case on a "
                         "1.6M-cell block (for profiling the sweep at a size that streams HBM)")
    ap.add_argument("--converged", type=int, default=0, metavar="MAPS",
                    help="instead of the bench line: the bump's steady state in mixed precision "
                         "and FP64 by Anderson-accelerated iterations (at most MAPS maps of 50 "
                         "iterations each), with the wall Cp of the two compared")
    ap.add_argument("--plate", type=int, default=0, metavar="ITERS",
                    help="instead of the bench line: the two-block SST flat plate 192x128x2 for ITERS "
                         "iterations in mixed precision and FP64, with the skin-friction difference")
    ap.add_argument("--cavity", type=int, default=0, metavar="ITERS",
                    help="instead of the bench line: the laminar lid-driven cavity 64x64x4 for ITERS "
                         "iterations in mixed precision and FP64 (both fused sweeps)")
    ap.add_argument("--batch", action="store_true",
                    help="instead of the bench line: the 96-block batched case, one launch per "
                         "stage for all blocks against a loop over the blocks' own steps")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the 1024x384x64-cell roofline measurement")
    ap.add_argument("--adjoint-study", default="", metavar="JSON",
                    help="instead of the bench line: the wall-force sensitivity study on the "
                         "128x48x4 bump (primal to a 1e-12 drop, adjoint to 1e-10, Mach, angle and "
                         "lower-wall nodes against central differences); writes JSON")
    ap.add_argument("--study-nodes", default="1-128",
                    help="lower-wall nodes of --adjoint-study: a range a-b or a comma list")
    ap.add_argument("--study-fd-step", type=float, default=1e-6,
                    help="the central-difference step of --adjoint-study")
    ap.add_argument("--study-fd-tol", type=float, default=0.0,
                    help="the residual drop the --adjoint-study re-solves reach (default: the "
                         "primal's, 1e-12)")
    ap.add_argument("--study-params", default="mach,angle",
                    help="flow parameters of --adjoint-study (comma list, may be empty)")
    ap.add_argument("--sweep", default="", choices=["", "mixed", "fp64", "vjp"],
                    help="instead of the bench line: step the workload block --sweep-iters "
                         "iterations at this precision, or (vjp) evaluate --sweep-iters primal "
                         "residuals and residual VJPs on the adjoint workload, and exit (a short "
                         "run for profilers)")
    ap.add_argument("--sweep-iters", type=int, default=6)
    ap.add_argument("--c2-iters", type=int, default=C2_ITERS, metavar="ITERS",
                    help="iterations of the mixed-vs-FP64 bump report (wall Cp, entropy, residual "
                         "drop); 0 skips it")
    return ap.parse_args()


def bench_config(case, ws):
    """The config dict of both arms' lines: the workload and what the timed
    region does between steps."""
    ext = case["ext"]
    N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
    return {"workload": case["name"], "cells": N, "cell_residuals_per_step": 3 * N,
            "l2": "GPU arm: flushed (256 MiB write) before every timed step; CPU arm: none",
            "parallelism": "replicas" if ws > 1 else "single device"}


def max_over_ranks(x, dist, device):
    """The largest value of x over all ranks (the job's time is its slowest
    rank's); x itself when not distributed."""
    if dist is None:
        return x
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_rate(cells_per_rank_step, steps, world, seconds):
    """Whole-job Mcell-residuals/s of `world` replicas, each advancing its
    own block, timed by the slowest rank."""
    return world * cells_per_rank_step * steps / seconds / 1e6


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class Clocks:
    """nvidia-smi sampling of the SM clock and throttle reasons."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-lms", "200", "-i", str(self.gpu)],
                                      stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except Exception:
            self.p = None
        return self

    def __exit__(self, *a):
        self.out = ""
        if self.p:
            time.sleep(0.25)
            self.p.terminate()
            try:
                self.out, _ = self.p.communicate(timeout=5)
            except Exception:
                self.p.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peak():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as f:
            return float(json.load(f)["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def committed_traffic(name="k_stage_traffic.json"):
    p = os.path.join(ROOT, "profiles", name)
    try:
        with open(p) as f:
            return json.load(f)
    except Exception:
        return None


def fp64_roofline(lib, C, abi, h, it, CFL, cells, reps=30):
    """The FP64 sweep against its own roof: the FP64 unit.  Flops per
    cell-residual from the committed ncu count of the same sweep
    (profiles/k_stage_fp64_flops.json: 2 x DFMA + DADD + DMUL thread
    instructions of one launch over its cells); the launch time from an
    event pair around each sweep launch of `reps` further iterations
    (fest_profile); the peak from an event-timed FP64 FMA microkernel run
    now (fest_measure_peak).  The HBM figure beside it uses the method's
    compulsory bytes."""
    fl = committed_traffic("k_stage_fp64_flops.json") or {}
    flops = fl.get("flops_per_cell_residual")
    abi.check(lib.fest_profile(h.h, 1), "profile")
    h.step(reps, it, CFL, with_norm=False)
    nl, tot = C.c_longlong(), C.c_double()
    abi.check(lib.fest_profile_read(h.h, C.byref(nl), C.byref(tot)), "profile_read")
    abi.check(lib.fest_profile(h.h, 0), "profile off")
    launch_s = tot.value / 1e3 / max(nl.value, 1)
    t = C.c_double()
    rc = lib.fest_measure_peak(0, C.byref(t))
    peak = t.value if rc == 0 else None
    out = {"bound": "fp64", "unit": "TFLOP/s", "peak": peak,
           "peak_source": "measured now: dependent FP64 FMA chains on every SM (fest_measure_peak)",
           "kernel": "k_stage<double> (fused WENO5+SLAU sweep + update, FP64)",
           "avg_launch_us": launch_s * 1e6, "launches": int(nl.value),
           "duration": "event pair around each sweep launch (fest_profile), mean",
           "flops_per_cell_residual": flops, "flops_source": fl.get("source")}
    if flops and peak:
        out["achieved"] = flops * cells / launch_s / 1e12
        out["frac"] = out["achieved"] / peak
    hbm, _ = measured_peak()
    bytes_launch = cells * sum(BYTES_STAGE) / len(BYTES_STAGE)
    out["hbm"] = {"achieved_gbs": bytes_launch / launch_s / 1e9, "peak_gbs": hbm,
                  "frac": bytes_launch / launch_s / 1e9 / hbm}
    return out


def wall_cp(q, ext, flow):
    """Cp on the first cell row above the lower wall (j=1), all i, k=1."""
    p = q[3:ext.imx + 2, 3, 3, 4]
    qinf = 0.5 * flow.density_inf * flow.vel_mag ** 2
    return (p - flow.pressure_inf) / qinf


def cpu_rate(case, seconds=10.0, threads=None):
    """The oracle (plain C, OpenMP over all host cores) on the same block;
    returns (Mcell-residuals/s, iterations timed, threads)."""
    import oracle as O
    threads = threads or (os.cpu_count() or 1)
    O.set_threads(threads)
    ext = case["ext"]
    blk = O.Block(ext, case["flow"], case["scheme"], case["bc"])
    blk["nodes"] = case["nodes"]
    blk.setup_geometry()
    blk["qp"] = case["qp"]
    O.get_next_solution([blk], 1, case["CFL"])  # warm-up
    n, t0 = 0, time.perf_counter()
    while True:
        O.get_next_solution([blk], 2 + n, case["CFL"])
        n += 1
        if time.perf_counter() - t0 >= seconds:
            break
    dt = time.perf_counter() - t0
    N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
    return N * 3 * n / dt / 1e6, n, threads


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return
    from fest3d import cases
    case = cases.bump_case()
    import oracle as O
    O.build()
    ext = case["ext"]
    N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
    threads = os.cpu_count() or 1
    O.set_threads(threads)
    blk = O.Block(ext, case["flow"], case["scheme"], case["bc"])
    blk["nodes"] = case["nodes"]
    blk.setup_geometry()
    blk["qp"] = case["qp"]
    it = 1
    for _ in range(args.warmup):  # ~0.1 s each on the host cores
        O.get_next_solution([blk], it, case["CFL"])
        it += 1
    t0 = time.perf_counter()
    steps = 0
    budget = 90.0
    while steps < args.steps:
        O.get_next_solution([blk], it, case["CFL"])
        it += 1
        steps += 1
        if time.perf_counter() - t0 > budget:
            break
    dt = time.perf_counter() - t0
    v = N * 3 * steps / dt / 1e6
    line = {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mcell-residuals/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": args.warmup,
            "ms_per_step": dt / steps * 1e3, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": bench_config(case, ws),
            "cpu_baseline": {"value": v, "unit": "Mcell-residuals/s", "cores": threads, "kind": "port",
                             "sample": f"{steps} TVD-RK3 iterations of the full block (bounded to "
                                       f"{budget:.0f} s), C restatement of the reference path, "
                                       f"OpenMP {threads} threads"},
            "e2e": {"value": v, "unit": "Mcell-residuals/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def large_block_roofline(lib, abi, cases, Handle, peak, flush, nc=(1024, 384, 64), iters=10):
    """Event-timed stage sweeps of the mixed bump scheme on a 1024x384x64-cell
    block (25M cells): algorithmic bytes per launch / mean launch time."""
    import torch
    try:
        case = cases.bump_case(nc=nc)
        ext = case["ext"]
        h = Handle(ext, case["flow"], case["scheme"], case["bc"], lib=lib)
        h.setup_geometry(case["nodes"])
        h.upload_state(case["qp"])
        h.set_precision(abi.FEST_MIXED)
        stream = torch.cuda.current_stream()
        abi.check(lib.fest_set_stream(h.h, C.c_void_p(stream.cuda_stream)), "set_stream")
        it = 1
        for _ in range(3):
            abi.check(lib.fest_step_async(h.h, 1, it, case["CFL"]), "warmup")
            it += 1
        torch.cuda.synchronize()
        abi.check(lib.fest_profile(h.h, 1), "profile")
        for _ in range(iters):
            flush.zero_()
            abi.check(lib.fest_step_async(h.h, 1, it, case["CFL"]), "step")
            it += 1
        torch.cuda.synchronize()
        nl, tot = C.c_longlong(), C.c_double()
        abi.check(lib.fest_profile_read(h.h, C.byref(nl), C.byref(tot)), "profile_read")
        abi.check(lib.fest_last_device_error(h.h), "device error")
        N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
        avg_s = tot.value / 1e3 / max(nl.value, 1)
        bl = N * sum(BYTES_STAGE) / len(BYTES_STAGE)
        h.close()
        return {"cells": N, "block": "x".join(map(str, nc)), "launches_timed": int(nl.value),
                "avg_launch_us": avg_s * 1e6, "bytes_per_launch": bl,
                "achieved": bl / avg_s / 1e9, "peak": peak, "unit": "GB/s",
                "frac": bl / avg_s / 1e9 / peak,
                "mcell_residuals_per_s": N / avg_s / 1e6}
    except Exception as e:  # report, do not lose the main line
        return {"error": str(e)}


def adjoint_cost(lib, reps=20):
    """Adjoint/primal cost on the adjoint workload (bump 128x48x4, Euler,
    unlimited MUSCL + SLAU, FP64): the device time (CUDA events around the
    kernels of the call, fest_last_kernel_ms) of one fest_residual_vjp
    against one primal residual evaluation: the reference's
    get_total_conservative_Residue (fest_get_total_conservative_residue:
    ghosts, face states, fluxes, residue) and, beside it, one stage of the
    fused FP64 sweep (residual, time step and update in one kernel).  The
    calls' wall clock with their host transfers is reported too."""
    import numpy as np
    from fest3d import abi, adjoint as A
    try:
        case = A.adjoint_case()
        h = A.make_handle(case, lib=lib)
        q = np.array(case["qp"], order="F")
        ext = case["ext"]
        lam = np.asfortranarray(np.random.default_rng(0).standard_normal(
            (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, 5)))
        ms = C.c_double()

        def dev():
            abi.check(lib.fest_last_kernel_ms(h.h, C.byref(ms)), "fest_last_kernel_ms")
            return ms.value

        h.residual(q, 3)
        h.residual_vjp(q, 3, lam)
        tp = ta = dp = da = 0.0
        for _ in range(reps):
            t0 = time.perf_counter()
            h.residual(q, 3)
            tp += time.perf_counter() - t0
            dp += dev()
            t0 = time.perf_counter()
            h.residual_vjp(q, 3, lam)
            ta += time.perf_counter() - t0
            da += dev()
        tp, ta, dp, da = tp / reps, ta / reps, dp / reps, da / reps
        # one stage of the fused FP64 sweep on the same state
        h.upload_state(q)
        h.set_precision(abi.FEST_FP64)
        h.step(3, 1, case["CFL"], with_norm=False)
        abi.check(lib.fest_profile(h.h, 1), "profile")
        h.step(reps, 4, case["CFL"], with_norm=False)
        nl, tot = C.c_longlong(), C.c_double()
        abi.check(lib.fest_profile_read(h.h, C.byref(nl), C.byref(tot)), "profile_read")
        abi.check(lib.fest_profile(h.h, 0), "profile off")
        stage_ms = tot.value / max(nl.value, 1)
        h.close()
        return {"workload": "bump 128x48x4, Euler, MUSCL (unlimited) + SLAU, FP64",
                "vjp_device_ms": da, "primal_residual_device_ms": dp, "fused_stage_device_ms": stage_ms,
                "adjoint_over_primal": da / dp, "adjoint_over_fused_stage": da / stage_ms,
                "timing": "CUDA events around each call's kernels on the handle's stream (fest_last_kernel_ms), "
                          "mean of %d; fused stage: event pair per sweep launch" % reps,
                "wall_clock_ms": {"primal_residual": tp * 1e3, "vjp": ta * 1e3,
                                  "note": "per C-ABI call, host transfers included"}}
    except Exception as e:
        return {"error": str(e)}


def c2_report(lib, abi, cases, Handle, iters):
    """The bump configuration's own report after `iters` iterations from the
    uniform start, FP64 and mixed precision: continuity-residual drop
    (last/first iteration), relative entropy change (SmoothBump/pp/entropy.py),
    the mixed-vs-FP64 differences of wall Cp and of the entropy field, and
    each run's wall time (fest_step through the C ABI, state on the device)."""
    import numpy as np
    from fest3d import post
    try:
        case = cases.bump_case()
        ext, flow, CFL = case["ext"], case["flow"], case["CFL"]
        out = {"iters": iters, "workload": case["name"]}
        q = {}
        for prec, name in ((abi.FEST_FP64, "fp64"), (abi.FEST_MIXED, "mixed")):
            h = Handle(ext, flow, case["scheme"], case["bc"], lib=lib)
            h.setup_geometry(case["nodes"])
            h.upload_state(case["qp"])
            h.set_precision(prec)
            t0 = time.perf_counter()
            n1 = h.step(1, 1, CFL)
            nN = h.step(iters - 1, 2, CFL)
            t = time.perf_counter() - t0
            q[name] = post.interior(h.download_state(), ext)
            vol = post.interior(h.get("cells")[0], ext)
            out[name] = {"seconds": t, "l2_drop_continuity": float(nN[1] / n1[1]),
                         "resnorm_first": [float(x) for x in n1], "resnorm_last": [float(x) for x in nN],
                         "entropy_change": post.entropy_change(q[name], vol, flow.pressure_inf,
                                                               flow.density_inf)}
            h.close()
        cp = {n: (q[n][:, 0, 0, 4] - flow.pressure_inf) / (0.5 * flow.density_inf * flow.vel_mag ** 2)
              for n in q}
        ef = {n: post.entropy_field(q[n], flow.pressure_inf, flow.density_inf) for n in q}
        out["wall_cp_abs_err_mixed_vs_fp64"] = float(np.abs(cp["mixed"] - cp["fp64"]).max())
        out["entropy_field_abs_err_mixed_vs_fp64"] = float(np.abs(ef["mixed"] - ef["fp64"]).max())
        out["entropy_field_max_abs_fp64"] = float(np.abs(ef["fp64"]).max())
        out["fp64_over_mixed_time"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
        return out
    except Exception as e:  # report, do not lose the main line
        return {"error": str(e)}


def run_ours(args):
    import numpy as np
    import torch

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    # a dedicated stream, current for everything below: the events, the L2
    # flush and the library's work (fest_set_stream) share it.  (torch's
    # default stream is handle 0, which fest_set_stream reads as "the
    # handle's own stream".)
    work_stream = torch.cuda.Stream()
    torch.cuda.set_stream(work_stream)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group(backend="nccl")
    from fest3d import abi, build, cases
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    case = cases.bump_case() if args.workload == "bump" else cases.bump_case(nc=(512, 192, 16))
    ext, flow, CFL = case["ext"], case["flow"], case["CFL"]
    N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
    STAGES = 3
    stream = torch.cuda.current_stream()
    if stream.cuda_stream == 0:  # the library is bound to this stream; events must see it
        raise RuntimeError("bench needs a non-default current CUDA stream")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def barrier():
        if dist:
            dist.barrier()
        torch.cuda.synchronize()

    def make(precision):
        h = Handle(ext, flow, case["scheme"], case["bc"], lib=lib)
        h.setup_geometry(case["nodes"])
        h.upload_state(case["qp"])
        h.set_precision(precision)
        abi.check(lib.fest_set_stream(h.h, C.c_void_p(stream.cuda_stream)), "set_stream")
        return h

    def timed(h, steps, it0):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        it = it0
        barrier()
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            abi.check(lib.fest_step_async(h.h, 1, it, CFL), "fest_step_async")
            e1.record(stream)
            it += 1
        barrier()
        abi.check(lib.fest_last_device_error(h.h), "device error")
        ms = max_over_ranks(sum(a.elapsed_time(b) for a, b in evs), dist, "cuda")
        return ms, it

    results = {}
    for prec in (abi.FEST_FP64, abi.FEST_MIXED):
        h = make(prec)
        it = 1
        for _ in range(args.warmup):
            abi.check(lib.fest_step_async(h.h, 1, it, CFL), "warmup")
            it += 1
        barrier()
        abi.check(lib.fest_last_device_error(h.h), "warmup error")
        steps = args.steps if prec == abi.FEST_MIXED else max(10, args.steps // 4)
        n0 = h.launches
        with Clocks(local) as ck:
            ms, it = timed(h, steps, it)
        launches = h.launches - n0
        results[prec] = dict(h=h, ms=ms, steps=steps, it=it, launches=launches, clocks=ck.summary())
    mixed, fp64 = results[abi.FEST_MIXED], results[abi.FEST_FP64]
    rate = lambda r: replica_rate(N * STAGES, r["steps"], ws, r["ms"] / 1e3)

    # roofline of the dominant kernel: event-timed stage-sweep launches
    h = mixed["h"]
    abi.check(lib.fest_profile(h.h, 1), "profile")
    prof_steps = min(200, args.steps)
    it = mixed["it"]
    for _ in range(prof_steps):
        flush.zero_()
        abi.check(lib.fest_step_async(h.h, 1, it, CFL), "profiled step")
        it += 1
    torch.cuda.synchronize()
    nl, tot = C.c_longlong(), C.c_double()
    abi.check(lib.fest_profile_read(h.h, C.byref(nl), C.byref(tot)), "profile_read")
    abi.check(lib.fest_profile(h.h, 0), "profile off")
    iso_s = tot.value / 1e3 / max(nl.value, 1)  # event pair around each launch, no graph
    bytes_launch = N * sum(BYTES_STAGE) / len(BYTES_STAGE)
    # in-step duration: the timed region's time per step over its sweep
    # launches (graph replay; a mixed bump step after iteration 2 launches
    # the three stage sweeps and nothing else)
    per_step = mixed["launches"] / max(mixed["steps"], 1)
    step_launch_s = mixed["ms"] / mixed["steps"] / 1e3 / max(per_step, 1)
    achieved = bytes_launch / step_launch_s / 1e9
    peak, peak_kind = measured_peak()
    tr = committed_traffic()
    traffic = tr.get("bytes_per_launch") if tr else None

    # mixed vs FP64 wall Cp after the same number of iterations
    qm = mixed["h"].download_state()
    q64 = fp64["h"].download_state()
    # bring both to the same iteration count
    lag = (mixed["it"] + prof_steps) - fp64["it"]
    if lag > 0:
        fp64["h"].step(lag, fp64["it"], CFL, with_norm=False)
        q64 = fp64["h"].download_state()
    cp_err = float(np.abs(wall_cp(qm, ext, flow) - wall_cp(q64, ext, flow)).max())

    # the same sweep on a block large enough to stream HBM (the bump block's
    # 9.5 MB state fits in L2 many times over): kernel roofline at scale
    large = large_block_roofline(lib, abi, cases, Handle, peak, flush) if args.large else None

    # e2e through the host-buffer C ABI, one iteration per call: the
    # interior cells (the step's inputs and results; ghost cells are BC work
    # the step recomputes) in pinned host memory, up, one iteration, down
    he = make(abi.FEST_MIXED)
    sl = (slice(3, ext.imx + 2), slice(3, ext.jmx + 2), slice(3, ext.kmx + 2))
    ishape = (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, ext.n_var)
    ihost = torch.empty(ishape[::-1], dtype=torch.float64, pin_memory=True)
    qint = ihost.numpy().T
    qint[...] = case["qp"][sl]
    iptr = abi.ptr(qint)
    e2e_steps = max(10, args.steps // 4)
    # one untimed call: first-use setup (mirrors, k-chunk tuning)
    abi.check(lib.fest_step_host_interior(he.h, iptr, 1, 1, CFL, None), "fest_step_host_interior")
    qint[...] = case["qp"][sl]
    it = 2
    tot_e2e = 0.0
    barrier()
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        abi.check(lib.fest_step_host_interior(he.h, iptr, 1, it, CFL, None), "fest_step_host_interior")
        tot_e2e += time.perf_counter() - t0
        it += 1
    ibytes = int(qint.nbytes)
    kms = C.c_double()
    abi.check(lib.fest_last_kernel_ms(he.h, C.byref(kms)), "fest_last_kernel_ms")
    e2e_step_device_us = kms.value * 1e3  # the last call's device work between its copies
    # the padded state (ghost layers included: 2.4x the interior for this
    # block), one synchronisation per call
    host = torch.empty(abi.shapes(ext)["qp"][::-1], dtype=torch.float64, pin_memory=True)
    qhost = host.numpy().T  # Fortran-ordered view of pinned memory
    abi.check(lib.fest_download_state(he.h, abi.ptr(qhost)), "download")
    ptr = abi.ptr(qhost)
    totp = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        abi.check(lib.fest_step_host(he.h, ptr, 1, it, CFL, None), "fest_step_host")
        totp += time.perf_counter() - t0
        it += 1
    # the same through three synchronous calls (upload, step, download)
    tot3 = 0.0
    for _ in range(e2e_steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        abi.check(lib.fest_upload_state(he.h, ptr), "upload")
        abi.check(lib.fest_step(he.h, 1, it, CFL, None), "fest_step")
        abi.check(lib.fest_download_state(he.h, ptr), "download")
        tot3 += time.perf_counter() - t0
        it += 1
    tot_e2e = max_over_ranks(tot_e2e, dist, "cuda")
    e2e_rate = replica_rate(N * STAGES, e2e_steps, ws, tot_e2e)
    nbytes = int(qhost.nbytes)
    # the host link alone: upload and download of the state, each synchronous
    tu = td = 0.0
    for _ in range(10):
        t0 = time.perf_counter()
        abi.check(lib.fest_upload_state(he.h, ptr), "upload")
        tu += time.perf_counter() - t0
        t0 = time.perf_counter()
        abi.check(lib.fest_download_state(he.h, ptr), "download")
        td += time.perf_counter() - t0
    link = {"h2d_gbs": 10 * nbytes / tu / 1e9, "d2h_gbs": 10 * nbytes / td / 1e9,
            "upload_us": tu / 10 * 1e6, "download_us": td / 10 * 1e6}

    fp64_roof = fp64_roofline(lib, C, abi, fp64["h"], fp64["it"], CFL, N)
    fp64["it"] += 30
    adj = adjoint_cost(lib) if rank == 0 else None
    c2 = c2_report(lib, abi, cases, Handle, args.c2_iters) if rank == 0 and args.c2_iters > 1 else None

    cpu = None
    if rank == 0 and ws == 1:
        v1, n1, _ = cpu_rate(case, seconds=3.0, threads=1)
        v, n_it, threads = cpu_rate(case, seconds=10.0)
        cpu = {"value": v, "unit": "Mcell-residuals/s", "cores": threads, "kind": "port",
               "sample": f"{n_it} TVD-RK3 iterations of the full 256x96x4 block (~10 s), "
                         f"C restatement of the reference path, OpenMP {threads} threads",
               "single_thread": {"value": v1, "sample": f"{n1} iterations (~3 s), 1 thread"}}

    if rank == 0:
        line = {
            "metric": METRIC, "value": rate(mixed), "unit": "Mcell-residuals/s", "n_gpus": ws,
            "steps": mixed["steps"], "warmup": args.warmup,
            "ms_per_step": mixed["ms"] / mixed["steps"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32 stencil / f64 state",
            "data": "synthetic (analytic bump grid, uniform Mach 0.5 start)",
            "config": bench_config(case, ws),
            "fp64": {"value": rate(fp64), "unit": "Mcell-residuals/s", "steps": fp64["steps"],
                     "ms_per_step": fp64["ms"] / fp64["steps"],
                     "roofline": fp64_roof, "clocks": fp64["clocks"]},
            "mixed_over_fp64": rate(mixed) / rate(fp64),
            "wall_cp_abs_err_mixed_vs_fp64": cp_err,
            "wall_cp_compare": {"iterations": int(mixed["it"] + prof_steps - 1),
                                "note": "mixed and FP64 after the same number of iterations from the "
                                        "uniform start, mid-transient; the converged comparison is "
                                        "bench.py --converged"},
            "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                         "frac": achieved / peak, "traffic": traffic,
                         "kernel": "k_stage<float> (fused WENO5+SLAU sweep + update)",
                         "peak_source": peak_kind, "launches_per_step": per_step,
                         "avg_launch_us": step_launch_s * 1e6,
                         "duration": "timed region's ms_per_step / sweep launches per step (graph "
                                     "replay, inter-launch gaps included)",
                         "isolated_launch_us": iso_s * 1e6, "isolated_launches": int(nl.value),
                         "bytes_per_cell_residual": list(BYTES_STAGE),
                         "bytes_per_launch": bytes_launch},
            "roofline_large_block": large,
            "bump_report": c2,
            "adjoint": adj,
            "clocks": mixed["clocks"],
            "e2e": {"value": e2e_rate, "unit": "Mcell-residuals/s", "h2d_bytes_per_step": ibytes,
                    "d2h_bytes_per_step": ibytes,
                    "path": "fest_step_host_interior (interior cells up, one iteration, interior "
                            "cells down; one synchronisation), pinned host buffer",
                    "over_device_rate": e2e_rate / rate(mixed),
                    "call_us": tot_e2e / e2e_steps * 1e6, "call_device_work_us": e2e_step_device_us,
                    "padded_state": {"value": replica_rate(N * STAGES, e2e_steps, ws, totp),
                                     "bytes_each_way": nbytes,
                                     "path": "fest_step_host (the padded qp with ghost layers)"},
                    "three_calls": {"value": replica_rate(N * STAGES, e2e_steps, ws, tot3),
                                    "path": "fest_upload_state + fest_step + fest_download_state "
                                            "(padded qp)"},
                    "host_link": link},
            "gpu_launches": int(mixed["launches"]),
            "cpu_baseline": cpu,
        }
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def run_adjoint_study(args):
    """fest3d.adjoint.wall_force_study through the C ABI; the result as JSON
    to args.adjoint_study and a one-line summary on stdout."""
    from fest3d import abi, build, adjoint as A
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    spec = args.study_nodes
    if "-" in spec:
        a, b = (int(x) for x in spec.split("-"))
        nodes = tuple(range(a, b + 1))
    else:
        nodes = tuple(int(x) for x in spec.split(",") if x)
    t0 = time.perf_counter()

    def save(o):
        with open(args.adjoint_study, "w") as f:
            json.dump(o, f, indent=1)

    params = tuple(x for x in args.study_params.split(",") if x)
    out = A.wall_force_study(lib, wall_nodes=nodes, params=params, fd_step=args.study_fd_step,
                             fd_tol=args.study_fd_tol or None,
                             log=lambda *a: print(*a, file=sys.stderr, flush=True), progress=save)
    out["seconds"] = time.perf_counter() - t0
    with open(args.adjoint_study, "w") as f:
        json.dump(out, f, indent=1)
    print(json.dumps({k: out[k] for k in ("primal", "adjoint", "max_rel_diff", "seconds")
                      if k in out}), flush=True)


def run_sweep(args):
    """The workload block stepped --sweep-iters iterations at one precision
    through fest_step, nothing else: the command profilers capture."""
    from fest3d import abi, build, cases
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    if args.sweep == "vjp":
        import numpy as np
        from fest3d import adjoint as A
        case = A.adjoint_case()
        ext = case["ext"]
        h = A.make_handle(case, lib=lib)
        q = np.array(case["qp"], order="F")
        lam = np.asfortranarray(np.random.default_rng(0).standard_normal(
            (ext.imx - 1, ext.jmx - 1, ext.kmx - 1, 5)))
        for _ in range(args.sweep_iters):
            h.residual(q, 3)
            h.residual_vjp(q, 3, lam)
        print(json.dumps({"sweep": "vjp", "calls": args.sweep_iters, "launches": h.launches}), flush=True)
        h.close()
        return
    case = cases.bump_case() if args.workload == "bump" else cases.bump_case(nc=(512, 192, 16))
    h = Handle(case["ext"], case["flow"], case["scheme"], case["bc"], lib=lib)
    h.setup_geometry(case["nodes"])
    h.upload_state(case["qp"])
    h.set_precision(abi.FEST_FP64 if args.sweep == "fp64" else abi.FEST_MIXED)
    h.step(args.sweep_iters, 1, case["CFL"], with_norm=False)
    print(json.dumps({"sweep": args.sweep, "workload": case["name"], "iters": args.sweep_iters,
                      "launches": h.launches}), flush=True)
    h.close()


def run_converged(args):
    """The bump's steady state in mixed precision (from the free stream) and
    in FP64 (from the mixed one), by Anderson-accelerated iterations of each
    precision's own sweep (fest3d.adjoint.converge_accelerated, 50
    iterations per map, at most args.converged maps): the mass-residual drop
    each reaches against the first iteration's, its wall time, and the
    wall Cp of the two steady states against each other.  Mixed precision
    levels off at its rounding floor; FP64 stops at a 1e-12 drop."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    from fest3d import abi, build, cases, adjoint as A
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    case = cases.bump_case()
    ext, flow, CFL = case["ext"], case["flow"], case["CFL"]

    def make(prec):
        h = Handle(ext, flow, case["scheme"], case["bc"], lib=lib)
        h.setup_geometry(case["nodes"])
        h.upload_state(case["qp"])
        h.set_precision(prec)
        return h

    out = {"mode": "converged wall Cp", "workload": case["name"], "maps_cap": args.converged}
    res = {}
    ref, start = None, None
    for prec, name, tol in ((abi.FEST_MIXED, "mixed", 1e-12), (abi.FEST_FP64, "fp64", 1e-12)):
        h = make(prec)
        n1 = float(h.step(1, 1, CFL)[1])
        ref = ref or n1
        if start is not None:
            h.upload_state(start)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        q, it, drop, _, maps, iters = A.converge_accelerated(h, h.download_state(), CFL, first_iter=2, tol=tol,
                                                             ref=ref, max_maps=args.converged)
        start = q
        sec = time.perf_counter() - t0
        res[name] = {"q": q, "drop": drop, "maps": maps, "iterations": iters + 1, "seconds": sec}
        h.close()
    cp = {k: wall_cp(v["q"], ext, flow) for k, v in res.items()}
    for k, v in res.items():
        out[k] = {x: v[x] for x in ("drop", "maps", "iterations", "seconds")}
    out["wall_cp_abs_err_mixed_vs_fp64"] = float(np.abs(cp["mixed"] - cp["fp64"]).max())
    out["wall_cp_max_abs"] = float(np.abs(cp["fp64"]).max())
    print(json.dumps(out), flush=True)


def run_batch(args):
    """96 seeded blocks (cell dims uniform in [16,160]x[16,96]x[2,16]),
    laminar (Sutherland) MUSCL + AUSM+, TVD-RK3, mixed precision: Mcell-residuals/s of
    the batched step (one ghost and one sweep launch per stage for all
    blocks) against stepping each block through its own handle."""
    import ctypes as C
    import torch
    torch.cuda.set_device(0)
    stream = torch.cuda.Stream()
    torch.cuda.set_stream(stream)
    from fest3d import abi, build, cases
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    blocks = cases.batch_blocks()
    cells = sum(c["cells"] for c in blocks)
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")

    def handles():
        hs = []
        for c in blocks:
            h = Handle(c["ext"], c["flow"], c["scheme"], c["bc"], lib=lib)
            h.setup_geometry(c["nodes"])
            h.upload_state(c["qp"])
            h.set_precision(abi.FEST_MIXED)
            abi.check(lib.fest_set_stream(h.h, C.c_void_p(stream.cuda_stream)), "set_stream")
            hs.append(h)
        return hs

    def timed(step, steps, it0):
        evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
               for _ in range(steps)]
        torch.cuda.synchronize()
        it = it0
        for e0, e1 in evs:
            flush.zero_()
            e0.record(stream)
            step(it)
            e1.record(stream)
            it += 1
        torch.cuda.synchronize()
        return sum(a.elapsed_time(b) for a, b in evs) / 1e3

    steps, warm = args.steps if args.steps != 2000 else 200, max(args.warmup, 3)
    out = {"mode": "batched multiblock", "blocks": len(blocks), "cells": cells,
           "workload": "96 blocks, dims uniform in [16,160]x[16,96]x[2,16] (seed 0), laminar "
                       "(Sutherland) MUSCL+AUSM+, TVD-RK3, CFL 0.5, periodic/extrapolated faces",
           "steps": steps, "warmup": warm, "dtype": "f32 stencil / f64 state"}
    hs = handles()
    arr = (C.c_void_p * len(hs))(*[h.h.value for h in hs])
    b = C.c_void_p()
    abi.check(lib.fest_batch_create(arr, len(hs), C.byref(b)), "batch_create")
    for it in range(1, warm + 1):
        abi.check(lib.fest_batch_step_async(b, 1, it, 0.5), "batch warmup")
    torch.cuda.synchronize()
    n0 = hs[0].launches
    tb = timed(lambda it: abi.check(lib.fest_batch_step_async(b, 1, it, 0.5), "batch step"),
               steps, warm + 1)
    nb_launch = (hs[0].launches - n0) / steps
    for h in hs:
        abi.check(lib.fest_last_device_error(h.h), "device error")
    out["batched"] = {"mcell_residuals_per_s": 3 * cells * steps / tb / 1e6, "ms_per_step": tb / steps * 1e3,
                      "launches_per_step": nb_launch}
    lib.fest_batch_destroy(b)
    for h in hs:
        h.close()
    hs = handles()
    for it in range(1, warm + 1):
        for h in hs:
            abi.check(lib.fest_step_async(h.h, 1, it, 0.5), "loop warmup")
    torch.cuda.synchronize()
    n1 = sum(h.launches for h in hs)

    def loop(it):
        for h in hs:
            abi.check(lib.fest_step_async(h.h, 1, it, 0.5), "loop step")

    tl = timed(loop, steps, warm + 1)
    out["per_block_loop"] = {"mcell_residuals_per_s": 3 * cells * steps / tl / 1e6,
                             "ms_per_step": tl / steps * 1e3,
                             "launches_per_step": (sum(h.launches for h in hs) - n1) / steps}
    out["batched_over_loop"] = tl / tb
    for h in hs:
        h.close()
    print(json.dumps(out), flush=True)


def run_cavity(args):
    """Laminar lid-driven cavity (64x64x4 cells, MUSCL + AUSM, forward Euler,
    local dt, CFL 0.5, constant mu for Re 100): ITERS iterations in mixed
    precision and in FP64 (the fused sweeps with their viscous terms), wall
    times and the u-velocity difference along the vertical centre line,
    relative to the lid speed."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    from fest3d import abi, build, cases
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    case = cases.ldc_case()
    ext = case["ext"]
    out = {"mode": "lid-driven cavity", "workload": case["name"], "iters": args.cavity}
    prof = {}
    for prec, name in ((abi.FEST_MIXED, "mixed"), (abi.FEST_FP64, "fp64")):
        h = Handle(ext, case["flow"], case["scheme"], case["bc"], lib=lib)
        h.setup_geometry(case["nodes"])
        h.upload_state(case["qp"])
        h.set_precision(prec)
        h.step(2, 1, case["CFL"], with_norm=False)  # first-use setup, fix() iterations
        torch.cuda.synchronize()
        n = args.cavity - 2
        t0 = time.perf_counter()
        norm = h.step(n, 3, case["CFL"])
        t = time.perf_counter() - t0
        q = h.download_state()
        prof[name] = q[3 + (ext.imx - 1) // 2, 3:ext.jmx + 2, 3, 1] / 34.7
        N = (ext.imx - 1) * (ext.jmx - 1) * (ext.kmx - 1)
        # find_resnorm scales by the free-stream speed, zero in the cavity
        # (resnorm.f90:128-169): the norm itself is not finite here
        out[name] = {"seconds": t, "mcell_residuals_per_s": N * n / t / 1e6}
        h.close()
    out["centreline_u_max_abs_diff_over_lid_speed"] = float(np.abs(prof["mixed"] - prof["fp64"]).max())
    out["mixed_over_fp64_time"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    print(json.dumps(out), flush=True)


def run_plate(args):
    """Turbulent flat plate with k-omega SST, 192x128x2 cells as the
    reference's two-block layout (0.33 m symmetry run-in + 2 m plate joined
    by an interface; MUSCL + AUSM-UP, RK4, local dt, CFL 1.0, M 0.2, Re 5e6
    per metre): ITERS iterations of both blocks in one batch, in mixed
    precision and in FP64; wall times, rates, residual norms and the skin
    friction along the plate.  Cf = tau_w / (1/2 rho_inf U_inf^2) with tau_w
    = mu(T_1) u_1 / d_1 from the first cell row (u_1 its x-velocity, d_1 its
    wall distance, mu by Sutherland's law at its temperature)."""
    import numpy as np
    import torch
    torch.cuda.set_device(0)
    from fest3d import abi, build, cases
    from fest3d.handle import Handle
    if not os.path.exists(abi.LIB_PATH):
        build.build()
    lib = abi.load()
    case = cases.plate_case()
    flow = case["flow"]
    out = {"mode": "SST flat plate", "workload": case["name"], "iters": args.plate}
    cf = {}
    N = sum((b["ext"].imx - 1) * (b["ext"].jmx - 1) * (b["ext"].kmx - 1) for b in case["blocks"])
    U, rho_inf = flow.x_speed_inf, flow.density_inf
    for prec, name in ((abi.FEST_MIXED, "mixed"), (abi.FEST_FP64, "fp64")):
        hs = []
        for blk in case["blocks"]:
            h = Handle(blk["ext"], blk["flow"], blk["scheme"], blk["bc"], lib=lib)
            h.setup_geometry(blk["nodes"])
            h.find_wall_dist(case["wall"])
            h.upload_state(blk["qp"])
            h.set_precision(prec)
            hs.append(h)
        arr = (C.c_void_p * len(hs))(*[h.h.value for h in hs])
        b = C.c_void_p()
        abi.check(lib.fest_batch_create(arr, len(hs), C.byref(b)), "fest_batch_create")
        abi.check(lib.fest_batch_step(b, 2, 1, case["CFL"]), "batch step")  # first-use setup, fix() iterations
        torch.cuda.synchronize()
        n = args.plate - 2
        t0 = time.perf_counter()
        abi.check(lib.fest_batch_step(b, n, 3, case["CFL"]), "batch step")
        t = time.perf_counter() - t0
        lib.fest_batch_destroy(b)
        plate = hs[1]
        ext = plate.ext
        q = plate.download_state()
        dist = plate.get("dist")
        norm = [list(h.resnorm()) for h in hs]
        rho1, u1, p1 = q[3:ext.imx + 2, 3, 3, 0], q[3:ext.imx + 2, 3, 3, 1], q[3:ext.imx + 2, 3, 3, 4]
        T1 = p1 / (rho1 * flow.R_gas)
        mu = flow.mu_ref * (T1 / flow.T_ref) ** 1.5 * (flow.T_ref + flow.Sutherland_temp) / (T1 + flow.Sutherland_temp)
        d1 = dist[3:ext.imx + 2, 3, 3]
        cf[name] = mu * u1 / d1 / (0.5 * rho_inf * U * U)
        out[name] = {"seconds": t, "mcell_residuals_per_s": 4 * N * n / t / 1e6,
                     "finite": bool(np.all(np.isfinite(q))),
                     "resnorm_per_block": [[float(x) for x in r] for r in norm]}
        for h in hs:
            h.close()
    out["cf_max_abs_diff"] = float(np.abs(cf["mixed"] - cf["fp64"]).max())
    out["cf_max_abs"] = float(np.abs(cf["fp64"]).max())
    out["cf_fp64_sample"] = [float(x) for x in cf["fp64"][:: max(1, len(cf["fp64"]) // 8)]]
    out["mixed_over_fp64_time"] = out["fp64"]["seconds"] / out["mixed"]["seconds"]
    print(json.dumps(out), flush=True)


def main():
    args = parse()
    if args.plate:
        run_plate(args)
        return
    if args.cavity:
        run_cavity(args)
        return
    if args.batch:
        run_batch(args)
        return
    if args.converged:
        run_converged(args)
        return
    if args.sweep:
        run_sweep(args)
        return
    if args.adjoint_study:
        run_adjoint_study(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
