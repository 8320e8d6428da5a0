"""Throughput of the residual + RK step on the 128^3 periodic workload.

One "step" is one full SSP-RK3 time step of the solver (CFL time-step
reduction + 3 stages of reconstruction, HLLC fluxes, residual and RK update)
over every cell of the 128^3 = 2,097,152-cell periodic ideal-gas case
(seeded synthetic state: sinusoidal density, 8-mode Fourier velocities,
noisy pressure).  The metric is Mcell-updates/s = cells x steps / s.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl fvgpu|reference]

--impl fvgpu (default) times libfvgpu on the GPU: `value` is the headline
precision (FP32-mixed when the library supports the case, else FP64) with
the state resident in HBM; `fp64` holds the FP64 path; `e2e` repeats the
measurement through the C ABI with the state copied from / to pinned host
memory every step (three contexts on three host threads by default).
--impl reference times the CPU implementation of the same step (the
oracle's C restatement of the reference, all host threads).  Under torchrun
each rank runs an independent replica of the whole workload (the timed path
exchanges nothing between ranks); value = all ranks' cells / max time.
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

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

METRIC = "Mcell-updates/s FP32-mixed vs FP64 plain at ≤1e-6 rel err; adjoint/fwd cost"
UNIT = "Mcell-updates/s"
L2_BYTES = 129 * 1024 * 1024


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def peaks():
    path = os.path.join(REPO, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index: int):
        self.dev = device_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "20"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "power_w_median": statistics.median(power) if power else None, "samples": len(sm),
                "reasons": sorted(reasons)}


def build_case(level: int):
    from fv_140823_gb300 import cases
    return cases.periodic(level=level)


def algorithmic_bytes_per_cell_step(neq: int = 5, n_nb: int = 6) -> int:
    """Compulsory HBM bytes of one SSP-RK3 step per cell with FP64 state:
    stage 1 reads U and writes U1, stages 2 and 3 read U_k and U and write
    (8 state passes of neq doubles), plus per stage the n_nb int32 neighbour
    ids and the 8-byte volume.  neq=5, n_nb=6: 320 + 96 = 416 B."""
    return 8 * neq * (2 + 3 + 3) + 3 * (4 * n_nb + 8)


def traffic_per_launch(kernel: str, ncells: int):
    """DRAM bytes per launch of `kernel` from the committed ncu summary
    (profiles/traffic.json: bytes per cell of a captured launch), or None."""
    path = os.path.join(REPO, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            t = json.load(fh)
        return float(t[kernel]["bytes_per_cell"]) * ncells
    except Exception:
        return None


def fp64_ops_per_cell(key: str):
    """Counted FP64 operations per cell of a kernel (profiles/traffic.json)."""
    try:
        with open(os.path.join(REPO, "profiles", "traffic.json")) as fh:
            return float(json.load(fh)["fp64_ops"][key])
    except Exception:
        return None


def measured_fp64_gops(device: int):
    import ctypes as C
    from fv_140823_gb300._native import load_gpu_lib
    out = C.c_double()
    return out.value if load_gpu_lib().fvgpu_measure_fp64(int(device), C.byref(out)) == 0 else None


def e2e_pipelined(case, cfg, nctx: int, steps: int, warmup: int, cfl: float, n: int) -> float:
    """End-to-end throughput through the public C ABI with `nctx` contexts,
    each driven by its own host thread (one context per thread, as the ABI
    prescribes).  Every step of every context does the full host round trip:
    upload of the step's input from pinned host memory, one SSP-RK3 step,
    download of the new state; the contexts' transfers in both directions
    overlap one another and the other contexts' compute.  Wall clock over all
    `steps` steps."""
    import ctypes as C
    import threading

    import torch

    from fv_140823_gb300 import abi
    from fv_140823_gb300.solver import Solver
    solvers = [Solver(case.tables, cfg) for _ in range(nctx)]
    hostU = [torch.from_numpy(np.ascontiguousarray(case.U)).pin_memory() for _ in range(nctx)]
    hostO = [torch.empty_like(h).pin_memory() for h in hostU]
    errors = []

    def worker(i, k):
        sv = solvers[i]
        lib = sv.lib
        for _ in range(k):
            rc = lib.fvgpu_upload_state(sv._ctx, C.c_void_p(hostU[i].data_ptr()), C.c_int64(n))
            rc |= lib.fvgpu_step(sv._ctx, abi.SCHEME_SSPRK3, 0.0, cfl, 1)
            rc |= lib.fvgpu_download_state(sv._ctx, C.c_void_p(hostO[i].data_ptr()), C.c_int64(n))
            if rc:
                errors.append(rc)
                return

    def run(counts):
        th = [threading.Thread(target=worker, args=(i, k)) for i, k in enumerate(counts)]
        for t in th:
            t.start()
        for t in th:
            t.join()

    try:
        run([max(warmup, 1)] * nctx)
        torch.cuda.synchronize()
        counts = [steps // nctx + (1 if i < steps % nctx else 0) for i in range(nctx)]
        t0 = time.perf_counter()
        run(counts)
        for sv in solvers:
            sv.synchronize()
        wall = time.perf_counter() - t0
    finally:
        for sv in solvers:
            sv.close()
    if errors:
        raise RuntimeError(f"pipelined e2e step failed rc={errors[0]}")
    return n * steps / wall / 1e6


def time_steps(torch, s, stream, flush, steps: int, cfl: float, scheme="ssprk3", dt: float = 0.0):
    """Per-step device times (ms), each step bracketed by events on the
    library's stream, with an L2 flush before each step outside the events
    (CFL steps, or fixed-dt steps when dt > 0)."""
    times = []
    with torch.cuda.stream(stream):
        for _ in range(steps):
            flush.fill_(1)
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            s.step(scheme, dt=dt, cfl=0.0 if dt > 0 else cfl, nsteps=1)
            e1.record(stream)
            times.append((e0, e1))
    torch.cuda.synchronize()
    s.synchronize()
    return [a.elapsed_time(b) for a, b in times]


def run_gpu(args):
    import torch

    from fv_140823_gb300 import abi
    from fv_140823_gb300.solver import FvGpuError, Solver

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    dist = None
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    case = build_case(args.level)
    t = case.tables
    n = t.ncells
    cfl = case.cfl

    results = {}
    hbm_peak, peak_kind = peaks()
    flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
    precisions = [abi.MIXED, abi.FP64] if args.precision == "auto" else (
        [abi.MIXED] if args.precision == "mixed" else [abi.FP64])
    states = {}
    for prec in precisions:
        cfg = case.cfg
        cfg.precision = prec
        cfg.device = local
        try:
            s = Solver(t, cfg)
        except FvGpuError as e:
            if e.code == abi.ERR_UNSUPPORTED:
                results[prec] = {"unsupported": str(e)}
                continue
            raise
        stream = torch.cuda.ExternalStream(s.stream_handle())
        s.set_state(case.U)
        s.step("ssprk3", cfl=cfl, nsteps=args.warmup)
        s.synchronize()
        if dist:
            dist.barrier()
        torch.cuda.synchronize()
        clocks = ClockSampler(local)
        clocks.start()
        nsteps = args.steps if prec == abi.MIXED or args.precision == "fp64" else min(args.steps, args.fp64_steps)
        ms = time_steps(torch, s, stream, flush, nsteps, cfl)
        clk = clocks.stop()
        total_ms = float(sum(ms))
        if dist:
            tt = torch.tensor([total_ms], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            total_ms = float(tt.item())
        value = ws * n * nsteps / (total_ms * 1e-3) / 1e6
        # live per-kernel timing (eager, events between launches on the library stream)
        s.set_state(case.U)
        kms, klaunch = s.profile_step("ssprk3", cfl=cfl, nsteps=max(3, min(args.steps, 10)))
        dom = int(np.argmax(kms))
        launches_per_step = int(sum(klaunch)) / max(3, min(args.steps, 10))
        avg_ms = kms[dom] / max(klaunch[dom], 1)
        # algorithmic bytes of one stage launch: one third of the step's compulsory bytes
        alg_bytes = algorithmic_bytes_per_cell_step(case.cfg.neq) / 3.0 * n
        achieved = alg_bytes / (avg_ms * 1e-3) / 1e9
        kname = abi.KIND_NAMES[dom]
        traffic = traffic_per_launch(f"{'mixed' if prec == abi.MIXED else 'fp64'}_{kname}", n)
        # end to end through the C ABI with pinned host buffers
        hostU = torch.from_numpy(np.ascontiguousarray(case.U)).pin_memory()
        hostOut = torch.empty_like(hostU).pin_memory()
        import ctypes as C
        e2e_ms = []
        lib = s.lib
        for it in range(args.warmup + nsteps):
            torch.cuda.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            rc = lib.fvgpu_upload_state(s._ctx, C.c_void_p(hostU.data_ptr()), C.c_int64(n))
            rc |= lib.fvgpu_step(s._ctx, abi.SCHEME_SSPRK3, 0.0, cfl, 1)
            rc |= lib.fvgpu_download_state(s._ctx, C.c_void_p(hostOut.data_ptr()), C.c_int64(n))
            e1.record(stream)
            e1.synchronize()
            if rc:
                raise RuntimeError(f"e2e step failed rc={rc}")
            if it >= args.warmup:
                e2e_ms.append(e0.elapsed_time(e1))
        e2e_total = float(sum(e2e_ms))
        if dist:
            tt = torch.tensor([e2e_total], device="cuda")
            dist.all_reduce(tt, op=dist.ReduceOp.MAX)
            e2e_total = float(tt.item())
        e2e_value = ws * n * nsteps / (e2e_total * 1e-3) / 1e6
        e2e_pipe = None
        if args.e2e_contexts > 1:
            e2e_pipe = e2e_pipelined(case, cfg, args.e2e_contexts, nsteps, args.warmup, cfl, n)
            if dist:
                tt = torch.tensor([n * nsteps / (e2e_pipe * 1e6)], device="cuda")
                dist.all_reduce(tt, op=dist.ReduceOp.MAX)
                e2e_pipe = ws * n * nsteps / float(tt.item()) / 1e6
        # state after a fixed number of steps at a fixed dt, for the error check
        s.set_state(case.U)
        dt0 = s.compute_dt(cfl)
        s.step("ssprk3", dt=dt0, nsteps=args.err_steps)
        states[prec] = (s.state(), dt0)
        results[prec] = {
            "value": value, "ms_per_step": total_ms / nsteps, "steps": nsteps, "clocks": clk,
            "kernel_ms": {abi.KIND_NAMES[k]: float(kms[k]) for k in range(len(kms)) if klaunch[k]},
            "kernel_launches": {abi.KIND_NAMES[k]: int(klaunch[k]) for k in range(len(kms)) if klaunch[k]},
            "launches_per_step": launches_per_step,
            "roofline": {"bound": "hbm", "kernel": kname, "achieved": achieved, "peak": hbm_peak,
                         "unit": "GB/s", "frac": achieved / hbm_peak, "traffic": traffic,
                         "peak_source": peak_kind, "algorithmic_bytes_per_launch": alg_bytes,
                         "avg_launch_ms": avg_ms},
            "e2e": {"value": e2e_pipe if e2e_pipe else e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": int(hostU.numel() * 8), "d2h_bytes_per_step": int(hostOut.numel() * 8),
                    "contexts": args.e2e_contexts if e2e_pipe else 1,
                    "timing": ("wall clock over all steps of all contexts (each step: upload from pinned host "
                               "memory, one SSP-RK3 step, download of the new state)") if e2e_pipe else
                              "CUDA events around upload + step + download, one context",
                    "single_context": e2e_value},
        }
        if prec == abi.MIXED:
            # FP32 reverse passes of the residual (a mixed context's VJP) on
            # device arrays, against one mixed stage launch
            w = torch.ones(case.cfg.neq, n, dtype=torch.float64, device="cuda")
            o = torch.empty_like(w)
            torch.cuda.synchronize()
            s.set_state(case.U)
            for _ in range(2):
                s.residual_vjp_device(w.data_ptr(), o.data_ptr())
            s.synchronize()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            for _ in range(5):
                s.residual_vjp_device(w.data_ptr(), o.data_ptr())
            e1.record(stream)
            e1.synchronize()
            ms_vjp = e0.elapsed_time(e1) / 5
            results[prec]["adjoint"] = {"ms_vjp_fp32": ms_vjp, "ms_stage": avg_ms, "vjp_over_stage": ms_vjp / avg_ms}
        if prec == abi.FP64:
            # FP64-pipe roofline of the residual kernel: counted FP64 operations
            # per launch over its live launch time, against the measured rate
            ops = fp64_ops_per_cell("residual_per_cell")
            gops = measured_fp64_gops(local)
            if ops is not None and gops and "residual" in results[prec]["kernel_ms"]:
                kl = results[prec]["kernel_launches"]["residual"]
                res_ms = results[prec]["kernel_ms"]["residual"] / max(kl, 1)
                ach = ops * n / (res_ms * 1e-3) / 1e9
                results[prec]["roofline_fp64"] = {
                    "bound": "fp64", "kernel": "residual", "achieved": ach, "peak": gops, "unit": "GFLOP/s",
                    "frac": ach / gops, "ops_per_cell": ops, "avg_launch_ms": res_ms,
                    "peak_source": "measured (fvgpu_measure_fp64: separate FP64 adds and multiplies)",
                    "note": "FP64 divisions and square roots count one operation each"}
            # hand-written adjoint of the FP64 residual against one residual evaluation
            s.set_state(case.U)
            ms_res, ms_vjp = s.profile_adjoint(reps=5)
            results[prec]["adjoint"] = {"ms_residual": ms_res, "ms_vjp": ms_vjp, "vjp_over_residual": ms_vjp / ms_res}
        s.close()
    results["workloads"] = None if args.no_workloads else amr_workloads(args, torch, flush, hbm_peak)
    err = None
    if abi.MIXED in states and abi.FP64 in states:
        a, b = states[abi.MIXED][0], states[abi.FP64][0]
        names = ["rho", "rho_u", "rho_v", "rho_w", "E"]
        err = {names[v]: float(np.linalg.norm(a[v] - b[v]) / np.linalg.norm(b[v])) for v in range(a.shape[0])}
    return results, err, case, ws, rank, dist


WORKLOADS = {
    "C2": ("two-phase bubble (model 3 mixture EOS), 16^3 base + 3 levels by the density criterion, "
           "MUSCL/minmod + HLLC, SSP-RK3", lambda: __import__("fv_140823_gb300.cases", fromlist=["x"]).bubble(4, 3)),
    "C5": ("viscous Taylor-Green vortex Re 1600 Mach 0.1, 32^3 base + 2 levels by the vorticity criterion, "
           "MUSCL/minmod + HLLC + viscous fluxes, SSP-RK3", lambda: __import__("fv_140823_gb300.cases",
                                                                             fromlist=["x"]).tgv(5, 2)),
}


def amr_workloads(args, torch, flush, hbm_peak):
    """The AMR workloads (1:4 faces, two-phase mixture, viscous) on the mixed
    and FP64 paths: graph-launched SSP-RK3 steps at a fixed dt (the FP64 CFL
    step of the initial state), each bracketed by events on the library
    stream with an L2 flush before it; relative L2 error of the mixed state
    against the FP64 state after `err_steps` steps (momentum components
    against the norm of the whole momentum)."""
    from fv_140823_gb300 import abi
    from fv_140823_gb300.abi import SolverConfig
    from fv_140823_gb300.solver import Solver
    out = {}
    for key, (desc, make) in WORKLOADS.items():
        case = make()
        n, nhang = case.tables.ncells, case.tables.nhang
        # compulsory bytes per step: 416 B per cell plus the 1:4 records read per stage
        alg = algorithmic_bytes_per_cell_step(case.cfg.neq) * n + 3 * 16 * nhang
        res = {"workload": desc, "cells": n, "hanging_faces": nhang, "algorithmic_bytes_per_step": alg}
        states = {}
        with Solver(case.tables, SolverConfig(**{**case.cfg.__dict__, "precision": abi.FP64})) as s:
            s.set_state(case.U)
            dt = s.compute_dt(case.cfl)
        res["dt"] = dt
        for prec, name, k in ((abi.MIXED, "mixed", args.workload_steps), (abi.FP64, "fp64", args.workload_fp64_steps)):
            with Solver(case.tables, SolverConfig(**{**case.cfg.__dict__, "precision": prec})) as s:
                stream = torch.cuda.ExternalStream(s.stream_handle())
                s.set_state(case.U)
                s.step("ssprk3", dt=dt, nsteps=args.warmup)
                s.synchronize()
                ms = time_steps(torch, s, stream, flush, k, 0.0, dt=dt)
                tot = float(sum(ms))
                res[name] = {"value": n * k / (tot * 1e-3) / 1e6, "unit": UNIT, "ms_per_step": tot / k, "steps": k,
                             "hbm_frac": alg / (tot / k * 1e-3) / 1e9 / hbm_peak}
                s.set_state(case.U)
                s.step("ssprk3", dt=dt, nsteps=args.err_steps_amr)
                states[prec] = s.state()
        a, b = states[abi.MIXED], states[abi.FP64]
        names = ["rho", "rho_u", "rho_v", "rho_w", "E" if case.cfg.model == 1 else "rho_Y"]
        mom = max(float(np.linalg.norm(b[1:4])), 1e-300)
        err = {}
        for v in range(a.shape[0]):
            den = mom if v in (1, 2, 3) else max(float(np.linalg.norm(b[v])), 1e-300)
            err[names[v]] = float(np.linalg.norm(a[v] - b[v])) / den
        res["mixed_over_fp64"] = res["mixed"]["value"] / res["fp64"]["value"]
        res["rel_l2_mixed_vs_fp64"] = {"steps": args.err_steps_amr, "momentum_against": "|rho u| norm", **err}
        if key in ADAPTIVE:
            res["adaptive"] = adaptive_run(make, ADAPTIVE[key], torch)
        out[key] = res
    return out


# C2 as configured: 200 steps with an adaptation every 10 (|grad rho| h > 50
# kg/m^3 asks for the finest level; levels 4..7)
ADAPTIVE = {"C2": dict(steps=200, every=10, threshold=50.0, min_level=4, max_level=7)}


def adaptive_run(make, cfg, torch):
    """The whole configured run on each path: CFL SSP-RK3 steps, the device
    criterion, host adaptation with state transfer and re-upload every
    `every` steps.  Host wall clock over the run (adaptations included);
    cell-updates counted on the mesh each segment ran on."""
    from fv_140823_gb300 import abi
    from fv_140823_gb300.abi import SolverConfig
    from fv_140823_gb300.adaptive import AdaptConfig, run_adaptive_gpu
    from fv_140823_gb300.solver import Solver
    ac = AdaptConfig(every=cfg["every"], kind=abi.CRIT_GRAD_RHO_H, threshold=cfg["threshold"],
                     min_level=cfg["min_level"], max_level=cfg["max_level"])
    out = {"steps": cfg["steps"], "every": cfg["every"], "criterion": "|grad rho| h > %g" % cfg["threshold"],
           "levels": [cfg["min_level"], cfg["max_level"]], "timing": "host wall clock over the whole run, "
           "adaptations (criterion, host refine/merge, transfer, re-upload) included"}
    for prec, name in ((abi.MIXED, "mixed"), (abi.FP64, "fp64")):
        case = make()
        n0 = case.tables.ncells
        with Solver(case.tables, SolverConfig(**{**case.cfg.__dict__, "precision": prec})) as s:
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            run = run_adaptive_gpu(s, case.mesh, case.U, cfg["steps"], ac, "ssprk3", case.cfl)
            s.synchronize()
            wall = time.perf_counter() - t0
        seg = [n0] + list(run.cells)
        updates = sum(c * min(cfg["every"], cfg["steps"] - i * cfg["every"]) for i, c in enumerate(seg))
        out[name] = {"value": updates / wall / 1e6, "unit": UNIT, "seconds": wall, "adaptations": len(run.cells),
                     "cells_first_last": [n0, run.cells[-1] if run.cells else n0]}
    out["mixed_over_fp64"] = out["mixed"]["value"] / out["fp64"]["value"]
    return out


def cpu_baseline(case, steps: int = 1):
    """The oracle's C restatement on the host cores (all threads), a bounded
    sample: `steps` SSP-RK3 steps of the full mesh."""
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from pyoracle import Oracle, ref_available
    threads = os.cpu_count() or 1
    Oracle.set_threads(threads)
    orc = Oracle(case.tables, case.cfg)
    dt = orc.cfl_dt(case.U, case.cfl)
    t0 = time.perf_counter()
    S = case.U
    for _ in range(steps):
        S = orc.step(S, dt, "ssprk3", 1)
    el = time.perf_counter() - t0
    return {"value": case.tables.ncells * steps / el / 1e6, "unit": UNIT, "cores": Oracle.threads(),
            "kind": "port",
            "sample": f"{steps} SSP-RK3 step(s) of the full {case.tables.ncells}-cell mesh, "
                      f"CFL dt, C restatement of the reference path with {Oracle.threads()} OpenMP threads"
                      + ("" if not ref_available() else "; oracle/_ref present but serial")}


def run_reference(args):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    full = build_case(args.level)
    sys.path.insert(0, os.path.join(REPO, "oracle"))
    from pyoracle import Oracle
    threads = os.cpu_count() or 1
    Oracle.set_threads(threads)
    # bounded sample: the largest periodic mesh of the same generator whose
    # K + W steps fit about two minutes on these cores (~0.3 Mcell-updates/s
    # per core for the C restatement)
    budget_cells = 120.0 * 0.3e6 * threads / max(args.steps + args.warmup, 1)
    level = args.level
    while level > 4 and 8 ** level > budget_cells:
        level -= 1
    case = full if level == args.level else build_case(level)
    orc = Oracle(case.tables, case.cfg)
    S = case.U
    for _ in range(args.warmup):
        S = orc.step(S, orc.cfl_dt(S, case.cfl), "ssprk3", 1)
    per = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        dt = orc.cfl_dt(S, case.cfl)
        S = orc.step(S, dt, "ssprk3", 1)
        per.append(time.perf_counter() - t0)
    total = sum(per)
    value = case.tables.ncells * args.steps / total / 1e6
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic", "config": config_of(full, args, gpu=False),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": Oracle.threads(), "kind": "port",
                         "sample": f"every step is one full SSP-RK3 step (CFL dt) of the "
                                   f"{case.tables.ncells}-cell periodic mesh of the same generator"
                                   f"{'' if case is full else ' (the workload at level ' + str(level) + ')'}"
                                   f" on {Oracle.threads()} threads"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def config_of(case, args, gpu: bool = True):
    cfg = {"workload": f"periodic ideal gas {2 ** args.level}^3 uniform octree (level {args.level}), "
                       f"{case.tables.ncells} cells, SSP-RK3, CFL 0.5, MUSCL/minmod + HLLC, seed 1234",
           "cells": case.tables.ncells, "scheme": "ssprk3", "cfl": 0.5, "parallelism": "replicas"}
    if gpu:
        cfg["l2"] = "flushed before every timed step (256 MiB write on the library stream)"
    return cfg


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=300)
    ap.add_argument("--e2e-contexts", type=int, default=3,
                    help="contexts (one host thread each) of the end-to-end measurement; 1 = sequential")
    ap.add_argument("--fp64-steps", type=int, default=20,
                    help="timed steps of the FP64 comparison arm (default 20: it runs ~37 ms per step)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="fvgpu", choices=["fvgpu", "reference"])
    ap.add_argument("--precision", default="auto", choices=["auto", "mixed", "fp64"])
    ap.add_argument("--level", type=int, default=7)
    ap.add_argument("--err-steps", type=int, default=50)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-workloads", action="store_true", help="skip the AMR workloads (C2, C5) of the line")
    ap.add_argument("--workloads-only", action="store_true",
                    help="print only the AMR workloads' JSON (no 128^3 arms)")
    ap.add_argument("--workload-steps", type=int, default=30)
    ap.add_argument("--workload-fp64-steps", type=int, default=5)
    ap.add_argument("--err-steps-amr", type=int, default=10)
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    if args.impl == "reference":
        return run_reference(args)
    from fv_140823_gb300 import abi
    if args.workloads_only:
        import torch
        torch.cuda.set_device(dist_env()[2])
        flush = torch.empty(2 * L2_BYTES // 4, dtype=torch.float32, device="cuda")
        print(json.dumps(amr_workloads(args, torch, flush, peaks()[0])))
        return 0
    results, err, case, ws, rank, dist = run_gpu(args)
    if rank == 0:
        head = abi.MIXED if "value" in results.get(abi.MIXED, {}) else abi.FP64
        r = results[head]
        line = {
            "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": r["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+f64" if head == abi.MIXED else "f64", "data": "synthetic",
            "config": config_of(case, args), "precision": "mixed" if head == abi.MIXED else "fp64",
            "e2e": r["e2e"], "roofline": r["roofline"], "clocks": r["clocks"],
            "gpu_launches": int(round(r["launches_per_step"] * args.steps)),
            "kernel_ms": r["kernel_ms"], "kernel_launches": r["kernel_launches"],
        }
        if abi.FP64 in results and head != abi.FP64 and "value" in results[abi.FP64]:
            f = results[abi.FP64]
            line["fp64"] = {"value": f["value"], "ms_per_step": f["ms_per_step"], "roofline": f["roofline"],
                            "roofline_fp64": f.get("roofline_fp64"), "e2e": f["e2e"], "kernel_ms": f["kernel_ms"]}
            line["mixed_over_fp64"] = r["value"] / f["value"]
        elif abi.MIXED in results and "unsupported" in results[abi.MIXED]:
            line["mixed"] = results[abi.MIXED]
        if "adjoint" in results.get(abi.FP64, {}):
            line["adjoint"] = dict(results[abi.FP64]["adjoint"])
            if "adjoint" in results.get(abi.MIXED, {}):
                line["adjoint"]["mixed"] = results[abi.MIXED]["adjoint"]
        if err is not None:
            line["rel_l2_mixed_vs_fp64"] = {"steps": args.err_steps, **err}
        if results.get("workloads"):
            line["workloads"] = results["workloads"]
        if not args.no_cpu_baseline:
            line["cpu_baseline"] = cpu_baseline(case)
        print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
