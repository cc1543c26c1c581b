#!/usr/bin/env python3
"""Benchmark of the semi-Lagrangian stream + collide step on GB300.

Workload (one "step" = one fused stream + collide time step over the whole
field): 3-D Taylor-Green vortex, D3Q19, BGK, semi-Lagrangian streaming on a
periodic cube [0, 2 pi)^3 with 16^3 hexahedra and FE_DGQ order 4 (125
nodes / cell, 512,000 nodes x 19), Ma = 0.1, Re = 1600, CFL = 0.4;
synthetic analytic initial state, equilibrium-initialised.

value:   node updates/s of the plain FP64 path (the reference's own
         arithmetic) with f resident in HBM (device time from CUDA events
         around each step; L2 flushed by a 256 MiB write between timed steps,
         outside the events).
e2e:     the same metric through the C ABI with host buffers: each step
         uploads f (FP64, pinned host memory), runs the step and reads rho
         and u back.  Pipelined: step k's upload runs on the handle's copy
         stream while step k-1 is stepped and read back (asynchronous
         read-back tickets); the blocking one-step-at-a-time loop is
         reported beside it (e2e.serial), with the measured host link.
roofline: the FP64 kernel is bound by the FP64 pipe, not by HBM: achieved =
         executed FP64 flops per launch (one ncu capture) over the live launch
         time, against the FP64 peak measured in the same run (cuBLAS DGEMM);
         the HBM fraction (algorithmic bytes 2 Q s_f per node) beside it.
fp32dev: the mixed-precision form (f - w_i stored in FP32) on the same
         workload: device rate, speed-up over FP64, HBM roofline, its own e2e
         and its error against the FP64 path after 1000 steps.
cpu_baseline: the CPU oracle (FP64 restatement of the reference algorithm:
         copy + per-direction CSR SpMV + collide sweep, OpenMP) on a bounded
         sample of the same workload.

--impl reference: the reference's CPU path cannot be built (deal.II,
Trilinos, p4est, Boost, MPI absent); its algorithm restated in the oracle
is timed on all host threads on the same workload instead.

Multi-GPU (torchrun): replicas only -- every rank runs the same solve on its
own GPU, value = total node updates / max rank time.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = dict(
    name="tgv3d_d3q19_bgk_sl_dg_p4_16x16x16",
    stencil="D3Q19", cells=(16, 16, 16), order=4, topology="dg", collision="BGK_STANDARD",
    Ma=0.1, Re=1600.0, cfl=0.4, L=2 * math.pi,
)
METRIC = "node updates/s (semi-Lagrangian stream + collide)"
UNIT = "node_updates/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def spec_for(precision: str, topology: str = None):
    import natrium_gb300 as N
    w = WORKLOAD
    scaling = math.sqrt(3) / w["Ma"]
    nu = 1.0 / w["Re"]  # U = 1, characteristic length 1 (TaylorGreenVortex3D.cpp:21)
    return N.SolverSpec(stencil=w["stencil"], order=w["order"], cells=w["cells"], length=(w["L"],) * 3,
                        scaling=scaling, viscosity=nu, cfl=w["cfl"], collision=w["collision"],
                        precision=precision, topology=topology or w["topology"])


def bench_feq(torch, stream, flush, steps: int = 50, warmup: int = 5):
    """The same workload on the reference's own node topology, FE_Q p = 4
    (16^3 cells: 64^3 = 262,144 device nodes, the periodic duplicates folded;
    274,625 in the reference layout), FP64 and FP32 deviation, each with the
    autotuner's kernel, device-timed like the headline (L2 flushed between
    steps)."""
    import natrium_gb300 as N
    out = {"workload": WORKLOAD["name"].replace("_dg_", "_feq_"), "unit": UNIT}
    for prec in ("fp64", "fp32dev"):
        spec = spec_for(prec, "feq")
        with N.Solver(spec) as sol:
            sol.set_stream(stream.cuda_stream)
            f0 = initial_state(spec)
            sol.upload_f(f0)
            sol.autotune(5)
            sol.upload_f(f0)
            per, launches = time_device(sol, torch, stream, flush, steps, warmup)
            ms = sum(per) / steps
            out[prec] = {"ms_per_step": ms, "value": sol.n_dev / (ms * 1e-3), "nodes": sol.n_dev,
                         "kernel": sol.kernel_info(), "gpu_launches": launches}
    return out


def initial_state(spec):
    from natrium_gb300 import problems as P
    X = P.node_coords(spec.cells, spec.order, spec.length, spec.topology)
    rho, u = P.taylor_green_3d(X, WORKLOAD["Ma"])
    return P.equilibrium(spec.stencil, spec.scaling, rho, u * 1.0)


class ClockSampler:
    """nvidia-smi clock / throttle sampling while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "50"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = float(parts[2])
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


def time_device(sol, torch, stream, flush, steps: int, warmup: int, nvtx: str = None):
    """Per-step CUDA-event timing on the solver's stream, L2 flushed between
    steps outside the events.  Returns (per-step ms list, launches).  With
    nvtx, the timed steps are enclosed in an NVTX range of that name."""
    for _ in range(warmup):
        sol.step_async(1, write_macro=False)
        with torch.cuda.stream(stream):
            flush.add_(1.0)
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(steps)]
    if nvtx:
        torch.cuda.nvtx.range_push(nvtx)
    l0 = sol.launches
    for k in range(steps):
        ev[k][0].record(stream)
        sol.step_async(1, write_macro=False)
        ev[k][1].record(stream)
        with torch.cuda.stream(stream):
            flush.add_(1.0)
    launches = sol.launches - l0
    if nvtx:
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize()
    sol.status()
    return [a.elapsed_time(b) for a, b in ev], launches


def time_e2e(sol, torch, f_host, rho_h, u_h, steps: int):
    """C-ABI calls with host buffers, one step at a time: upload f, one step,
    blocking read of rho/u, status check.  Returns s per step."""
    sol.upload_f(f_host)
    sol.step(1)
    sol.download_macro(rho_h, u_h)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(steps):
        sol.upload_f(f_host)
        sol.step_async(1, True)              # enqueue; the download below synchronises
        r, u = sol.download_macro(rho_h, u_h)
        sol.status()                         # the step's density check, every step
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps


def measure_link(torch, nbytes: int, reps: int = 5):
    """Host link bandwidth (GB/s) of copies of nbytes between page-locked host
    memory and the device, each direction alone (CUDA events)."""
    h = torch.empty(nbytes, dtype=torch.uint8).pin_memory()
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    out = {}
    for name, dst, src in (("h2d_gbs", d, h), ("d2h_gbs", h, d)):
        dst.copy_(src, non_blocking=True)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            dst.copy_(src, non_blocking=True)
        b.record()
        torch.cuda.synchronize()
        out[name] = nbytes * reps / (a.elapsed_time(b) * 1e-3) / 1e9
    return out


def time_e2e_pipelined(sol, torch, f_host, rho_bufs, u_bufs, steps: int):
    """The same calls pipelined: every step still uploads its whole f from
    page-locked host memory and reads its rho/u back, but the read-back is
    asynchronous (a ticket) and the host waits for the results of step
    k - depth + 1 only after enqueueing step k (depth = the number of host
    result buffers, 3), so the uploads (their own copy stream) run back to
    back while earlier steps are stepped and read back; with two steps in
    flight the host's wait put each read-back in the chain before the upload
    two steps later.  Each wait checks the status of its step.  Returns s per
    step."""
    depth = len(rho_bufs)

    def run(n):
        pending = []
        for k in range(n):
            sol.upload_f(f_host)
            sol.step_async(1, True)
            pending.append(sol.download_macro_async(rho_bufs[k % depth], u_bufs[k % depth]))
            if len(pending) == depth:
                sol.wait(pending.pop(0))     # step k - depth + 1's rho/u are on the host
        for t in pending:
            sol.wait(t)

    run(3)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    run(steps)
    torch.cuda.synchronize()
    return (time.perf_counter() - t0) / steps


def traffic_from_profile():
    try:
        with open(os.path.join(ROOT, "profiles", "traffic.json")) as fh:
            d = json.load(fh)
        return d
    except Exception:
        return None


def cpu_baseline(sample_cells=(8, 8, 8), steps=5):
    """Oracle (FP64 restatement of the reference algorithm) on a bounded
    sample of the workload: same stencil / order / topology, fewer cells."""
    import oracle as O
    w = WORKLOAD
    st = O.stencil(w["stencil"], math.sqrt(3) / w["Ma"])
    mesh = O.Mesh(3, sample_cells, w["order"], w["topology"] == "dg", (w["L"],) * 3)
    dt = O.time_step(mesh.h_min(), w["order"], st.max_speed, w["cfl"])
    tau = (1.0 / w["Re"]) / (dt * st.cs2) + 0.5
    rho, u = O.tgv3d_init(mesh.coords(), w["Ma"])
    f = O.equilibrium(st, rho, np.ascontiguousarray(u))
    S = O.SLOperator(mesh, st, dt)
    threads = O.max_threads()
    S.step_bgk(f, tau, 1, threads)
    t0 = time.perf_counter()
    S.step_bgk(f, tau, steps, threads)
    el = (time.perf_counter() - t0) / steps
    # the same sample on one thread (one timed step)
    t0 = time.perf_counter()
    S.step_bgk(f, tau, 1, 1)
    el1 = time.perf_counter() - t0
    return {"value": mesh.n_nodes / el, "unit": UNIT, "cores": threads, "kind": "port",
            "value_1_thread": mesh.n_nodes / el1,
            "sample": f"{w['stencil']} BGK FE_DGQ p={w['order']}, {sample_cells[0]}^3 cells "
                      f"({mesh.n_nodes} nodes), {steps} timed steps of copy + CSR SpMV + collide, FP64, "
                      f"{threads} OpenMP threads (value_1_thread: one step on one thread)"}


COMPRESSIBLE = dict(
    name="riemann2d_d2q25h_quartic_sl_dg_p2_128x128",
    cells=(128, 128), order=2, topology="dg", scaling=1.0, viscosity=1e-3, cfl=0.4, velocity_unit=1.58,
    t_end=0.3,
)


def compressible_spec(precision: str = "fp64"):
    import natrium_gb300 as N
    c = COMPRESSIBLE
    return N.SolverSpec(stencil="D2Q25H", order=c["order"], cells=c["cells"], length=(1.0, 1.0),
                        scaling=c["scaling"], viscosity=c["viscosity"], cfl=c["cfl"], collision="BGK_COMPRESSIBLE",
                        precision=precision, topology=c["topology"], periodic=(False, False, True))


def open_boundaries(sol):
    """The configuration's extrapolation boundaries: do-nothing on all four
    faces (the reference's DoNothingBoundary, boundaries/DoNothingBoundary.h)."""
    for face in range(4):
        sol.set_boundary(face, "DO_NOTHING")


# the FP32 two-population kernel's forms by kernel variant (nat_select_candidate index)
TH_FORMS = {5: 0, 9: 1, 10: 2, 14: 3}


def _compressible_leg(torch, stream, flush, precision, steps, warmup, full_run, variant=0):
    import natrium_gb300 as N
    from natrium_gb300 import problems as P
    c = COMPRESSIBLE
    spec = compressible_spec(precision)
    X = P.node_coords(spec.cells, spec.order, spec.length, spec.topology)
    rho, u, T = P.riemann_2d(X, c["velocity_unit"], spec.scaling)
    sol = N.Solver(spec)
    open_boundaries(sol)
    sol.set_stream(stream.cuda_stream)
    sol.init_thermal(rho, u, T)
    if precision != "fp64":
        if variant:  # a pinned form (a launch list of the form the autotuner picks outside ncu)
            sol.select_candidate(TH_FORMS[variant])
        else:
            sol.autotune(10)  # FP32: register, shared-memory or staged-row form of the fused kernel
    per, launches = time_device(sol, torch, stream, flush, steps, warmup)
    ms = sum(per) / steps
    n = sol.n_dev
    es = 8 if precision == "fp64" else 4
    out = {"precision": precision, "ms_per_step": ms, "value": n / (ms * 1e-3), "gpu_launches": launches,
           "algorithmic_bytes_per_launch": 2 * 2 * sol.Q * es * n,
           "achieved_gbs": 2 * 2 * sol.Q * es * n / (ms * 1e-3) / 1e9,
           "kernel": f"k_thermal_step<{'double' if es == 8 else 'float'},true>", "kernel_variant": sol.kernel_variant,
           "autotune": sol.autotune_report()}
    fields = None
    if full_run:
        sol.init_thermal(rho, u, T)
        sol.step(1)
        m0, _ = sol.mass_energy()
        dt = sol.dt
        nsteps = int(round(c["t_end"] * c["velocity_unit"] / dt))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        sol.step(nsteps - 1)
        wall = time.perf_counter() - t0
        m1, _ = sol.mass_energy()
        r, uu = sol.download_macro()
        Tn, _ = sol.download_thermal()
        fields = (r, uu, Tn)
        out["full_run"] = {"steps": nsteps, "t_end_lattice": nsteps * dt, "wall_s": wall,
                           "mass_rel_change": abs(m1 - m0) / abs(m0),
                           "rho_range": [float(r.min()), float(r.max())],
                           "T_range": [float(Tn.min()), float(Tn.max())],
                           "finite": bool(np.isfinite(r).all() and np.isfinite(Tn).all())}
    sol.close()
    return out, n, fields


def bench_compressible(torch, stream, flush, steps: int = 200, warmup: int = 5, full_run: bool = True,
                       variant: int = 0):
    """The compressible two-population path (D2Q25H, quartic BGK with g) on
    the four-quadrant Riemann problem: 128^2 cells, FE_DGQ p = 2 (147,456
    nodes x 25 x 2 populations), do-nothing (extrapolation) boundaries.  FP32
    deviation storage (the configuration's storage) and plain FP64, each
    device-timed; with full_run
    both also run to t = 0.3 and the FP32 fields are compared with the FP64
    ones (the FP64 path matches the oracle to 1e-12 per step).  variant
    (5, 9, 10, 14) pins the FP32 kernel form instead of autotuning it."""
    c = COMPRESSIBLE
    o32, n, F32 = _compressible_leg(torch, stream, flush, "fp32dev", steps, warmup, full_run, variant)
    o64, _, F64 = _compressible_leg(torch, stream, flush, "fp64", max(20, steps // 4), warmup, full_run)
    out = {"workload": c["name"], "nodes": n, "dtype": "f32", "unit": UNIT, "value": o32["value"],
           "ms_per_step": o32["ms_per_step"], "fp32dev": o32, "fp64": o64,
           "speedup_fp32dev_vs_fp64": o64["ms_per_step"] / o32["ms_per_step"],
           "boundaries": "do-nothing (extrapolation) on all four faces",
           "state": "lattice units: u / 1.58, T = 3 (p / rho) / 1.58^2, nu = 1e-3, scaling 1, CFL 0.4"}
    if full_run:
        rl2 = lambda a, b: float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))
        out["fp32dev_vs_fp64_at_t_end"] = {"rel_l2_rho": rl2(F32[0], F64[0]), "rel_l2_u": rl2(F32[1], F64[1]),
                                           "rel_l2_T": rl2(F32[2], F64[2])}
    return out


MIXED = {"name": "tgv3d_d3q27_kbc_sl_dg_p3_32x32x32", "stencil": "D3Q27", "collision": "KBC_STANDARD",
         "order": 3, "cells": (32, 32, 32), "Ma": 0.1, "Re": 1600.0, "cfl": 0.4, "steps": 2000, "every": 100}


def bench_mixed(torch, stream, flush, steps: int = None, profile: bool = False, candidate: int = -1,
                variant: int = 0):
    """The mixed-precision accuracy configuration: 3-D Taylor-Green, D3Q27
    KBC, 32^3 hexahedra, FE_DGQ p = 3 (2,097,152 nodes x 27), Ma 0.1,
    Re 1600, 2000 steps.  The FP32 deviation path and the FP64 path run side
    by side from the same initial f; every 100 steps the relative L2
    difference of u and rho is recorded (the FP64 path is the oracle-pinned
    one), and each path's device time per step is reported.

    profile: the FP32 path alone, 3 warm-up and `steps` timed steps, with
    the autotuner's choice (its report is returned, with the chosen index) or,
    with candidate >= 0, that candidate of its list without timing (then the
    3 warm-up steps are the only launches of the kernel before the timed
    ones, for a one-launch capture); with variant > 0 the autotuner chooses
    among that kernel variant's shapes only (12: the tensor-core corners).

    A third solver runs the FP32 path with kernel variant 12 (the 8 corner
    directions as tf32x3 tensor-core tiles) beside the autotuned one: its
    time and its error against FP64 decide whether that form is kept."""
    import natrium_gb300 as N
    from natrium_gb300 import problems as P
    c = MIXED
    steps = steps or c["steps"]
    scaling = math.sqrt(3) / c["Ma"]
    if profile:
        spec = N.SolverSpec(stencil=c["stencil"], order=c["order"], cells=c["cells"], length=(2 * math.pi,) * 3,
                            scaling=scaling, viscosity=1.0 / c["Re"], cfl=c["cfl"], collision=c["collision"],
                            precision="fp32dev", topology="dg")
        with N.Solver(spec) as sol:
            sol.set_stream(stream.cuda_stream)
            X = P.node_coords(c["cells"], c["order"], spec.length, "dg")
            rho, u = P.taylor_green_3d(X, c["Ma"])
            sol.upload_f(P.equilibrium(c["stencil"], scaling, rho, u))
            rep, chosen = [], candidate
            if variant:
                sol.set_kernel_variant(variant)
            if candidate >= 0:
                sol.select_candidate(candidate)
            else:
                _, chosen = sol.autotune(3)
                rep = sol.autotune_report()
            sol.step_async(3, False)
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            torch.cuda.nvtx.range_push("timed")  # ncu --nvtx-include timed/
            e0.record(stream)
            sol.step_async(steps, False)
            e1.record(stream)
            torch.cuda.nvtx.range_pop()
            sol.status()
            ms = e0.elapsed_time(e1) / steps
            return {"workload": c["name"], "nodes": sol.n_dev, "ms_per_step": ms, "kernel": sol.kernel_info(),
                    "candidate": chosen, "autotune": rep}
    sols, reports = {}, {}
    for name, prec, var in (("fp64", "fp64", 0), ("fp32dev", "fp32dev", 0), ("fp32dev_tc", "fp32dev", 12)):
        spec = N.SolverSpec(stencil=c["stencil"], order=c["order"], cells=c["cells"], length=(2 * math.pi,) * 3,
                            scaling=scaling, viscosity=1.0 / c["Re"], cfl=c["cfl"], collision=c["collision"],
                            precision=prec, topology="dg")
        sol = N.Solver(spec)
        sol.set_stream(stream.cuda_stream)
        X = P.node_coords(c["cells"], c["order"], spec.length, "dg")
        rho, u = P.taylor_green_3d(X, c["Ma"])
        sol.upload_f(P.equilibrium(c["stencil"], scaling, rho, u))
        if var:
            sol.set_kernel_variant(var)
        sol.autotune(3)
        reports[name] = sol.autotune_report()
        sols[name] = sol
    rl2 = lambda a, b: float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))
    curve, ms = [], {name: 0.0 for name in sols}
    done = 0
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    while done < steps:
        k = min(c["every"], steps - done)
        out = {}
        for prec, sol in sols.items():
            torch.cuda.synchronize()
            e0.record(stream)
            sol.step_async(k, True)
            e1.record(stream)
            sol.status()
            ms[prec] += e0.elapsed_time(e1)
            out[prec] = sol.download_macro()
        done += k
        curve.append({"step": done, "rel_l2_u": rl2(out["fp32dev"][1], out["fp64"][1]),
                      "rel_l2_rho": rl2(out["fp32dev"][0], out["fp64"][0]),
                      "tc_rel_l2_u": rl2(out["fp32dev_tc"][1], out["fp64"][1]),
                      "tc_rel_l2_rho": rl2(out["fp32dev_tc"][0], out["fp64"][0])})
    n = sols["fp64"].n_dev
    res = {"workload": c["name"], "nodes": n, "steps": steps, "unit": UNIT,
           "fp32dev": {"ms_per_step": ms["fp32dev"] / steps, "value": n * steps / (ms["fp32dev"] * 1e-3),
                       "kernel": sols["fp32dev"].kernel_info(), "autotune": reports["fp32dev"]},
           "fp64": {"ms_per_step": ms["fp64"] / steps, "value": n * steps / (ms["fp64"] * 1e-3),
                    "kernel": sols["fp64"].kernel_info(), "autotune": reports["fp64"]},
           "fp32dev_tensor_core_corners": {
               "ms_per_step": ms["fp32dev_tc"] / steps, "value": n * steps / (ms["fp32dev_tc"] * 1e-3),
               "kernel": sols["fp32dev_tc"].kernel_info(),
               "vs_autotuned_fp32dev": ms["fp32dev"] / ms["fp32dev_tc"],
               "max_rel_l2_u": max(r["tc_rel_l2_u"] for r in curve),
               "max_rel_l2_rho": max(r["tc_rel_l2_rho"] for r in curve),
               "form": "kernel variant 12: the 8 corner directions as mma.sync m16n8k8 tf32 tiles, operands split "
                       "into two TF32 halves (3 products), FP32 accumulation; the other 18 directions "
                       "sum-factorised as in variant 11"},
           "speedup_fp32dev_vs_fp64": ms["fp64"] / ms["fp32dev"],
           "max_rel_l2_u": max(r["rel_l2_u"] for r in curve), "max_rel_l2_rho": max(r["rel_l2_rho"] for r in curve),
           "every_100_steps": curve,
           "storage": "FP32 f - w_i with FP32 arithmetic and FP64 departure weights (no BF16/FP16 operands: "
                      "the 1e-6 velocity target rules them out)",
           "timing": "device events around each 100-step block, L2 not flushed (2.1 M nodes x 27 x 4 B = "
                     "226 MB per f buffer exceeds the L2)"}
    for sol in sols.values():
        sol.close()
    return res


MAPPED = {"name": "lubrication_sine_d2q9_bgk_sl_dg_p4_256x64", "refinement": 6, "order": 4, "Ma": 0.1,
          "viscosity": 1e-3, "cfl": 0.4, "bottom_velocity": 0.05}


def bench_mapped(torch, stream, flush, steps: int = 100, warmup: int = 5):
    """MappingQ1 cells: the LubricationSine channel (the reference's
    non-Cartesian benchmark) refined to 256 x 64 cells, D2Q9 BGK, FE_DGQ
    p = 4 (409,600 nodes), moving bottom wall; the departure-point kernel in
    FP32 deviation storage and in FP64, each device-timed."""
    import natrium_gb300 as N
    from natrium_gb300 import problems as P
    c = MAPPED
    V = P.lubrication_sine_grid(refinement=c["refinement"])
    cells = tuple(s - 1 for s in V.shape[:2])
    scaling = math.sqrt(3) / c["Ma"]
    U = c["bottom_velocity"] * scaling
    out = {"workload": c["name"], "unit": UNIT}
    for precision in ("fp32dev", "fp64"):
        spec = N.SolverSpec(stencil="D2Q9", order=c["order"], cells=cells, length=(1.0, 0.25), scaling=scaling,
                            viscosity=c["viscosity"], cfl=c["cfl"], collision="BGK_STANDARD", precision=precision,
                            topology="dg", periodic=(True, False, True), vertices=V)
        t0 = time.perf_counter()
        sol = N.Solver(spec)
        t_create = time.perf_counter() - t0
        sol.set_boundary(2, "VELOCITY_BOUNCE_BACK", np.array([U, 0.0, 0.0]))
        sol.set_stream(stream.cuda_stream)
        X = P.mapped_node_coords(V, c["order"], "dg")
        u = P.lubrication_sine_velocity(X, U, 0.25, 0.05)
        sol.upload_f(P.equilibrium("D2Q9", scaling, np.ones(sol.n_ref), u))
        n_steps = steps if precision == "fp32dev" else max(20, steps // 4)
        per, launches = time_device(sol, torch, stream, flush, n_steps, warmup)
        ms = sum(per) / n_steps
        n = sol.n_dev
        es = 8 if precision == "fp64" else 4
        # f read and written once, plus the rows per (node, direction): base,
        # D unit coordinates (FP32) or D (p + 1) Lagrange values (FP64),
        # constant, flags
        per_row = 2 * es if es == 4 else 2 * (c["order"] + 1) * es
        row_bytes = (sol.Q - 1) * (4 + per_row + es + 1)
        alg = n * (2 * sol.Q * es + row_bytes)
        out[precision] = {"ms_per_step": ms, "value": n / (ms * 1e-3), "gpu_launches": launches,
                          "algorithmic_bytes_per_launch": alg, "achieved_gbs": alg / (ms * 1e-3) / 1e9,
                          "create_s": t_create, "kernel": f"k_mapped<D2Q9,{'double' if es == 8 else 'float'},BGK,4>",
                          "kernel_variant": sol.kernel_variant}
        out["nodes"] = n
        sol.close()
    out["value"] = out["fp32dev"]["value"]
    out["cells"] = list(cells)
    out["departure_search"] = bench_departure_search()
    return out


def bench_departure_search(cells=(32, 32, 32), order=2):
    """Setup of a mapped mesh: the departure-point search with the MappingQ1
    Newton inverse (SemiLagrangian.cpp:525-757, SemiLagrangianTools.cpp:15-64)
    for every (node, direction) of D3Q19, FE_DGQ p = 2 on a deformed periodic
    grid of 32^3 cells (884,736 nodes x 18 rows): nat_create (which searches
    on the device), then the search alone on the device and on all host
    threads (the same tracker code, rows equal bit for bit)."""
    import natrium_gb300 as N
    from natrium_gb300 import problems as P
    L = (1.0, 1.0, 1.0)
    V = P.wavy_grid(cells, L, 0.05)
    scaling = math.sqrt(3) / 0.1
    spec = N.SolverSpec(stencil="D3Q19", order=order, cells=cells, length=L, scaling=scaling, viscosity=1e-3,
                        cfl=0.4, collision="BGK_STANDARD", precision="fp32dev", topology="dg", vertices=V)
    t0 = time.perf_counter()
    sol = N.Solver(spec)
    t_create = time.perf_counter() - t0
    sol.mapped_rows("device", copy=False)  # warm (module and allocations)
    t0 = time.perf_counter()
    sol.mapped_rows("device", copy=False)
    t_dev = time.perf_counter() - t0
    t0 = time.perf_counter()
    sol.mapped_rows("host", copy=False)
    t_host = time.perf_counter() - t0
    out = {"mesh": f"D3Q19 FE_DGQ p={order}, {cells[0]}^3 deformed cells", "nodes": sol.n_dev,
           "rows": (sol.Q - 1) * sol.n_dev, "create_s": t_create, "search_device_s": t_dev,
           "search_host_s": t_host, "host_threads": os.cpu_count(), "speedup_device_vs_host": t_host / t_dev}
    sol.close()
    return out


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def aggregate_ranks(torch, ws: int, total_ms: float, nodes: int, steps: int, device="cuda"):
    """Replicas: every rank timed `steps` steps of its own `nodes`-node solve.
    Returns the slowest rank's total (all ranks must call this; a MAX
    all-reduce, no data-path collective) and the whole-job throughput
    ws * nodes * steps / that time."""
    if ws > 1:
        t = torch.tensor([total_ms], device=device, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
    return total_ms, ws * nodes * steps / (total_ms * 1e-3)


def bench_config(nodes: int, ws: int) -> dict:
    """The workload as both arms name it (identical keys and values)."""
    w = WORKLOAD
    return {"workload": w["name"], "nodes": nodes, "stencil": w["stencil"], "collision": w["collision"],
            "order": w["order"], "topology": w["topology"], "cells": list(w["cells"]), "Ma": w["Ma"], "Re": w["Re"],
            "cfl": w["cfl"], "storage": "fp64 (plain)", "parallelism": f"replicas x{ws}",
            "l2": "GPU arm: L2 flushed between timed steps (256 MiB write outside the timed events); "
                  "CPU arm: no flush (host caches)"}


def run_reference(args):
    ws, rank, local = dist_env()
    if rank != 0:
        return 0
    import oracle as O
    w = WORKLOAD
    st = O.stencil(w["stencil"], math.sqrt(3) / w["Ma"])
    mesh = O.Mesh(3, w["cells"], w["order"], w["topology"] == "dg", (w["L"],) * 3)
    dt = O.time_step(mesh.h_min(), w["order"], st.max_speed, w["cfl"])
    tau = (1.0 / w["Re"]) / (dt * st.cs2) + 0.5
    rho, u = O.tgv3d_init(mesh.coords(), w["Ma"])
    f = O.equilibrium(st, rho, np.ascontiguousarray(u))
    S = O.SLOperator(mesh, st, dt)
    threads = O.max_threads()
    S.step_bgk(f, tau, max(args.warmup, 1), threads)
    t0 = time.perf_counter()
    S.step_bgk(f, tau, args.steps, threads)
    el = (time.perf_counter() - t0) / args.steps
    v = mesh.n_nodes / el
    line = {
        "impl": "reference", "metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": el * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (analytic TGV3D state)",
        "config": bench_config(mesh.n_nodes, args.gpus),
        "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"full workload, {args.steps} steps; the reference (deal.II/Trilinos) cannot "
                                   "be built, its algorithm is restated in oracle/natoracle.c"},
        "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def fp64_peak_tflops(torch, n: int = 4096, reps: int = 3) -> float:
    """Measured FP64 peak of this GPU: cuBLAS DGEMM (torch float64 matmul) of
    n^3, 2 n^3 flops, best of reps, CUDA events."""
    a = torch.randn(n, n, dtype=torch.float64, device="cuda")
    b = torch.randn(n, n, dtype=torch.float64, device="cuda")
    c = a @ b
    torch.cuda.synchronize()
    best = float("inf")
    for _ in range(reps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b, out=c)
        e1.record()
        torch.cuda.synchronize()
        best = min(best, e0.elapsed_time(e1) * 1e-3)
    del a, b, c
    return 2.0 * n ** 3 / best / 1e12


def fp64_profile():
    """Executed FP64 flops and DRAM traffic per launch of the FP64 kernel, from
    one ncu capture (profiles/fp64_flops.json)."""
    try:
        with open(os.path.join(ROOT, "profiles", "fp64_flops.json")) as fh:
            return json.load(fh)
    except Exception:
        return None


def time_e2e_legs(sol, torch, ws, f0, nodes, e2e_steps):
    """The e2e legs of one solver: link bandwidth, the serial loop and the
    pipelined loop (the reported value), and the check that a pipelined
    read-back equals the blocking one."""
    f_host = torch.from_numpy(f0).pin_memory().numpy()
    rho_h = torch.empty(sol.n_ref, dtype=torch.float64).pin_memory().numpy()
    u_h = torch.empty((sol.D, sol.n_ref), dtype=torch.float64).pin_memory().numpy()
    link = measure_link(torch, f0.nbytes)
    serial_s = time_e2e(sol, torch, f_host, rho_h, u_h, e2e_steps)
    serial_ms, _ = aggregate_ranks(torch, ws, serial_s * 1e3, nodes, 1)
    rho_b = [rho_h] + [torch.empty(sol.n_ref, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    u_b = [u_h] + [torch.empty((sol.D, sol.n_ref), dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    torch.cuda.nvtx.range_push("e2e")
    e2e_s = time_e2e_pipelined(sol, torch, f_host, rho_b, u_b, 4 * e2e_steps)
    torch.cuda.nvtx.range_pop()
    e2e_ms, _ = aggregate_ranks(torch, ws, e2e_s * 1e3, nodes, 1)
    sol.upload_f(f0)
    sol.step(1)
    r_ref, u_ref = sol.download_macro()
    sol.upload_f(f0)
    sol.step_async(1, True)
    sol.wait(sol.download_macro_async(rho_b[1], u_b[1]))
    pipeline_ok = bool(np.array_equal(rho_b[1], r_ref) and np.array_equal(u_b[1], u_ref))
    h2d = f0.nbytes
    d2h = 8 * (1 + sol.D) * sol.n_ref
    return {"value": ws * nodes / (e2e_ms * 1e-3), "unit": UNIT, "h2d_bytes_per_step": h2d,
            "d2h_bytes_per_step": d2h, "ms_per_step": e2e_ms,
            "mode": "pipelined, three steps in flight: uploads back to back on their own copy stream while "
                    "earlier steps are stepped and their rho/u read back on the read-back stream; every step "
                    "uploads its f (FP64, reference layout, page-locked) and reads its rho/u, status checked "
                    "per step",
            "link": link, "link_floor_ms": h2d / (link["h2d_gbs"] * 1e6),
            "serial": {"value": ws * nodes / (serial_ms * 1e-3), "ms_per_step": serial_ms,
                       "mode": "upload, step, blocking read-back, one step at a time"},
            "pipeline_matches_blocking": pipeline_ok}


KERNEL_NAMES = {1: "k_sl_step", 2: "k_sl_step_v2", 3: "k_sl_row", 6: "k_sl_rowt", 7: "k_sl_rowg", 11: "k_sl_cell", 12: "k_sl_cell[tensor-core corners]", 13: "k_sl_cell[z sharing]"}


def run_ours(args):
    import torch
    import natrium_gb300 as N

    ws, rank, local = dist_env()
    torch.cuda.set_device(local)
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    stream = torch.cuda.Stream()
    flush = torch.zeros(64 * 1024 * 1024, dtype=torch.float32, device="cuda")  # 256 MiB > L2
    if args.mapped_only:
        print(json.dumps(bench_mapped(torch, stream, flush, steps=args.steps, warmup=args.warmup)))
        return 0
    if args.mixed_only:
        print(json.dumps(bench_mixed(torch, stream, flush, steps=args.steps if args.profile else None,
                                     profile=args.profile, candidate=args.candidate, variant=args.variant)))
        return 0
    if args.compressible_only:
        print(json.dumps(bench_compressible(torch, stream, flush, steps=args.steps, warmup=args.warmup,
                                            full_run=not args.profile, variant=args.variant)))
        return 0

    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    try:
        smi_index = int(vis.split(",")[local]) if vis else local
    except (ValueError, IndexError):
        smi_index = local

    if args.profile:
        spec = spec_for(args.profile_precision)
        f0 = initial_state(spec)
        with N.Solver(spec) as sol:
            sol.set_stream(stream.cuda_stream)
            sol.upload_f(f0)
            if args.candidate >= 0:
                sol.select_candidate(args.candidate)
            else:
                if args.variant:  # the autotuner then chooses among that variant's shapes
                    sol.set_kernel_variant(args.variant)
                sol.autotune(10)
            # the timed steps sit in an NVTX range "timed" (ncu --nvtx-include timed/)
            per, launches = time_device(sol, torch, stream, flush, args.steps, args.warmup, nvtx="timed")
            print(json.dumps({"profile_run": True, "precision": args.profile_precision,
                              "ms_per_step": sum(per) / args.steps, "launches": launches,
                              "kernel": sol.kernel_info(), "autotune": sol.autotune_report()}))
        return 0

    dgemm = fp64_peak_tflops(torch)

    # --- headline: the plain FP64 path (the reference's own arithmetic) --------
    spec = spec_for("fp64")
    f0 = initial_state(spec)
    sol = N.Solver(spec)
    sol.set_stream(stream.cuda_stream)
    sol.upload_f(f0)
    at64 = []
    if args.variant:
        sol.set_kernel_variant(args.variant)
        ncand, chosen = 1, 0
    else:
        ncand, chosen = sol.autotune(5)
        at64 = sol.autotune_report()
    kinfo = sol.kernel_info()
    sol.upload_f(f0)
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    with ClockSampler(smi_index) as clk:
        per, launches = time_device(sol, torch, stream, flush, args.steps, args.warmup, nvtx="headline")
    torch.cuda.synchronize()
    if ws > 1:
        torch.distributed.barrier()
    nodes = sol.n_dev
    Q = sol.Q
    total_ms, value = aggregate_ranks(torch, ws, sum(per), nodes, args.steps)
    ms = total_ms / args.steps
    e2e = time_e2e_legs(sol, torch, ws, f0, nodes, max(5, min(50, args.steps // 4)))
    rho, u = sol.download_macro()
    ok = bool(np.all(np.isfinite(rho)) and abs(float(np.mean(rho)) - 1.0) < 1e-2)
    sol.close()

    # --- FP32 deviation storage (the mixed-precision form) -------------------------
    spec32 = spec_for("fp32dev")
    sol32 = N.Solver(spec32)
    sol32.set_stream(stream.cuda_stream)
    sol32.upload_f(f0)
    if args.variant:
        sol32.set_kernel_variant(args.variant)
        ncand32, chosen32 = 1, 0
    else:
        ncand32, chosen32 = sol32.autotune(10)
    kinfo32 = sol32.kernel_info()
    sol32.upload_f(f0)
    steps32 = max(args.steps, 20)
    per32, launches32 = time_device(sol32, torch, stream, flush, steps32, args.warmup, nvtx="fp32dev")
    total32, value32 = aggregate_ranks(torch, ws, sum(per32), nodes, steps32)
    ms32 = total32 / steps32
    e2e32 = time_e2e_legs(sol32, torch, ws, f0, nodes, max(5, min(50, args.steps // 4)))
    # accuracy against the FP64 path (the path pinned to the oracle), same start
    acc_steps = 1000
    sol32.upload_f(f0)
    sol32.step(acc_steps)
    r32, u32 = sol32.download_macro()
    sol32.close()
    with N.Solver(spec) as s64:
        s64.set_stream(stream.cuda_stream)
        s64.upload_f(f0)
        s64.step(acc_steps)
        r64, u64 = s64.download_macro()
    rl2 = lambda a, b: float(np.sqrt(np.sum((a - b) ** 2) / np.sum(b ** 2)))

    hbm, peak_kind = peaks()
    alg64 = 2 * Q * 8 * nodes
    alg32 = 2 * Q * 4 * nodes
    prof = fp64_profile()
    traffic64 = flops64 = busy64 = None
    if prof and prof.get("workload") == WORKLOAD["name"] and prof.get("kernel_variant") == kinfo["variant"] \
            and prof.get("tile_nodes") == kinfo["tile_nodes"]:
        traffic64 = prof.get("dram_bytes_per_launch")
        flops64 = prof.get("fp64_flops_per_launch")
        busy64 = prof.get("fp64_pipe_busy")
    tr = traffic_from_profile()
    traffic32 = None
    if tr and tr.get("workload") == WORKLOAD["name"] and tr.get("kernel_variant", 3) == kinfo32["variant"]:
        traffic32 = tr.get("dram_bytes_per_launch")
    ach64_gbs = alg64 / (ms * 1e-3) / 1e9
    fp64_tflops = flops64 / (ms * 1e-3) / 1e12 if flops64 else None

    if rank != 0:
        if ws > 1:
            torch.distributed.destroy_process_group()
        return 0
    cpu = cpu_baseline() if ws == 1 else None
    compressible = None if args.no_compressible else bench_compressible(torch, stream, flush)
    mapped = None if args.no_mapped else bench_mapped(torch, stream, flush)
    mixed = None if args.no_mixed else bench_mixed(torch, stream, flush)
    feq = None if args.no_mixed else bench_feq(torch, stream, flush)
    serving = None
    if not args.no_serving:
        from natrium_gb300 import serving as SV
        arr, reqs = SV.workload(512, seed=0, rate=200.0)
        serving = SV.run_workload(arr, reqs)
        seq = SV.run_sequential(reqs[:args.fp64_sample], "fp64")
        cap = SV.run_workload(np.zeros(len(reqs)), reqs)
        serving["capacity"] = {"solves_per_s": cap["solves_per_s"], "wall_s": cap["wall_s"],
                               "latency_p50_s": cap["latency_p50_s"], "latency_p99_s": cap["latency_p99_s"],
                               "node_updates_per_s": cap["node_updates_per_s"],
                               "server_steps": cap["server_steps"], "graph_builds": cap["graph_builds"],
                               "graph_updates": cap["graph_updates"], "host_rebuild_s": cap["host_rebuild_s"],
                               "note": "all 512 requests submitted at t = 0 (saturated server)"}
        serving.update({"workload": "512 D2Q9 solves (TGV / shear layer, BGK / KBC, N in {4..64}, p 2-6, "
                                    "Ma 0.02-0.1, Re 100-5000, 50-2000 steps), Poisson 200 req/s, seed 0, "
                                    "FP32 deviation storage",
                        "fp64_one_at_a_time": {**seq, "sample": f"first {args.fp64_sample} requests of the same "
                                                                "stream"}})
    kname = KERNEL_NAMES.get(kinfo["variant"], str(kinfo["variant"]))
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (analytic Taylor-Green initial state, equilibrium-initialised)",
        "config": bench_config(nodes, ws),
        "l2": "flushed between timed steps (256 MiB write, outside the timed events)",
        "roofline": {"bound": "fp64", "achieved": fp64_tflops, "peak": dgemm, "unit": "TFLOP/s",
                     "frac": fp64_tflops / dgemm if fp64_tflops else None, "traffic": traffic64,
                     "peak_kind": "measured in this run: cuBLAS DGEMM 4096^3 (torch float64 matmul), best of 3",
                     "achieved_from": "executed FP64 flops per launch (2 DFMA + DADD + DMUL, one ncu capture, "
                                      "profiles/fp64_flops.json) / the live mean launch time",
                     "fp64_pipe_busy_ncu": busy64,
                     "hbm": {"achieved": ach64_gbs, "peak": hbm, "unit": "GB/s", "frac": ach64_gbs / hbm,
                             "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg64},
                     "kernel": kname + "<D3Q19,double,BGK>", "tile_nodes": kinfo["tile_nodes"],
                     "threads": kinfo["threads"], "autotune": {"candidates": ncand, "chosen": chosen,
                                                               "report": at64}},
        "cpu_baseline": cpu,
        "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "fp32dev": {"value": value32, "ms_per_step": ms32, "steps": steps32, "gpu_launches": launches32,
                    "storage": "fp32 deviation f - w_i, FP32 arithmetic, FP64 departure weights",
                    "speedup_vs_fp64_plain": ms / ms32,
                    "roofline": {"bound": "hbm", "achieved": alg32 / (ms32 * 1e-3) / 1e9, "peak": hbm,
                                 "unit": "GB/s", "frac": alg32 / (ms32 * 1e-3) / 1e9 / hbm, "traffic": traffic32,
                                 "peak_kind": peak_kind, "algorithmic_bytes_per_launch": alg32,
                                 "kernel": KERNEL_NAMES.get(kinfo32["variant"], str(kinfo32["variant"]))
                                           + "<D3Q19,float,BGK>",
                                 "tile_nodes": kinfo32["tile_nodes"], "threads": kinfo32["threads"],
                                 "autotune": {"candidates": ncand32, "chosen": chosen32}},
                    "e2e": e2e32,
                    "error_vs_fp64": {"steps": acc_steps, "rel_l2_u": rl2(u32, u64), "rel_l2_rho": rl2(r32, r64)}},
        "serving": serving,
        "compressible": compressible,
        "mapped": mapped,
        "mixed_d3q27": mixed,
        "feq_topology": feq,
        "state_ok": ok,
    }
    print(json.dumps(line))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--variant", type=int, default=0,
                    help="fused kernel: 0 autotuned, 1 generic, 3 tile, 4 row-segment, 6 bulk-copy row-segment, "
                         "7 row-group, 11 cell-row, 12 cell-row with tensor-core corners (D3Q27 FP32); with "
                         "--compressible-only the FP32 two-population form: 5 registers, 9 / 10 shared memory, "
                         "14 staged rows")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving workload")
    ap.add_argument("--candidate", type=int, default=-1,
                    help="with --profile: use this autotuner candidate without timing")
    ap.add_argument("--profile-precision", default="fp64", choices=["fp32dev", "fp64"],
                    help="with --profile: the path to time (the headline plain FP64 path or FP32 deviation)")
    ap.add_argument("--profile", action="store_true",
                    help="lean run for ncu: device timing of one path only (no e2e, other legs, CPU baseline "
                         "or clocks)")
    ap.add_argument("--fp64-sample", type=int, default=512,
                    help="serving: requests of the stream timed one at a time on the plain FP64 path")
    ap.add_argument("--no-compressible", action="store_true", help="skip the compressible D2Q25H leg")
    ap.add_argument("--no-mapped", action="store_true", help="skip the mapped-mesh (LubricationSine) leg")
    ap.add_argument("--no-mixed", action="store_true", help="skip the D3Q27 KBC FP32-vs-FP64 accuracy leg")
    ap.add_argument("--mixed-only", action="store_true",
                    help="run only the D3Q27 KBC FP32-vs-FP64 accuracy leg (prints its JSON object)")
    ap.add_argument("--mapped-only", action="store_true",
                    help="time only the mapped-mesh leg (prints its JSON object)")
    ap.add_argument("--compressible-only", action="store_true",
                    help="time only the compressible D2Q25H leg (prints its JSON object)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return run_reference(args)
    return run_ours(args)


if __name__ == "__main__":
    sys.exit(main())
