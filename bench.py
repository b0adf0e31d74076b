#!/usr/bin/env python
"""Throughput of the HERMESHD DG step on GB300: DOF-updates/s per RK stage.

Headline workload (one GPU): the 2-D isentropic vortex, 128x128x1 cells,
5-moment Euler, quadratic Legendre basis (nbasis 10, iquad 3), HLLC, SSP-RK3,
FP64 (the "plain" path).  A step is one SSP-RK3 time step (CFL reduction +
three stages) of the whole grid; DOF = nx*ny*nz*nQ*nbasis with nQ = 11.
Variants on the same JSON line: the same workload in FP32, and the FP32
batched fluctuating-hydro ensemble (256 periodic boxes of sizes drawn from
{16,24,32,48}^3, 10-moment + stochastic stress, nb 4) against the plain FP64
path on one such box.  Inputs are synthetic (seeded initial conditions);
between timed steps a 256 MiB buffer is written to flush L2 (129 MB).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

--impl reference times the reference algorithm's CPU implementation (the
FP64 C restatement in oracle/, all host threads) on the same workload.
N > 1 (torchrun): replicas, one independent copy of the workload per GPU.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "DOF-updates/s per RK stage, FP64 plain vs FP32 batched at stated L2 error"
UNIT = "DOF-updates/s"
WORKLOAD = ("2D isentropic vortex {n}x{n}x1 periodic, 5-moment Euler, quadratic Legendre basis "
            "(nbasis 10, iquad 3), HLLC, SSP-RK3, FP64")
# FP64 arithmetic instructions the kernels execute per cell and stage on this
# workload, from one ncu launch of each kernel at 256x256 (2 * dfma + dadd +
# dmul thread instructions / cells, profiles/fp64_ops_vortex256_f64.txt); the
# reference algorithm's count (perfmodel) is larger: the kernels use the
# mirror symmetries of the tables
EXECUTED_FLOPS_VORTEX = {"cell": 8428.0, "update": 4818.0, "face_x": 1902.4, "face_y": 1899.4, "face_z": 2078.0,
                         "trace": 2442.0}
FALLBACK_HBM_GBS = 6800.0


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=("ours", "reference"))
    ap.add_argument("--n", type=int, default=128, help="vortex grid size (default 128)")
    ap.add_argument("--no-variants", action="store_true")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline (profiling runs)")
    ap.add_argument("--ensemble-accuracy", type=int, default=0, metavar="STEPS",
                    help="only the FP32-vs-FP64 ensemble-mean accuracy of the timed 256-box draw (Roe) over "
                         "STEPS steps of the ensemble configuration's 500, with the density S(k) accumulated "
                         "every 10 steps in both precisions, printed as one JSON line")
    return ap.parse_args()


# ---------------------------------------------------------------------------
def dist_init():
    import torch
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    elif torch.cuda.is_available():
        torch.cuda.set_device(0)
    return rank, ws


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws):
    """The largest of every rank's x (the slowest replica's time): the only
    collective of a replica run, outside the timed region."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_throughput(units_per_rank, elapsed_local, ws):
    """Whole-job throughput of ws independent replicas: every rank processes
    units_per_rank units; the job takes as long as its slowest rank."""
    elapsed = max_over_ranks(elapsed_local, ws)
    return ws * units_per_rank / elapsed, elapsed


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.p:
            self.p.terminate()
            self.p.wait(timeout=10)

    def summary(self):
        self.f.flush()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        try:
            os.unlink(self.f.name)
        except OSError:
            pass
        sm, mx, reasons = [], None, set()
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = float(r[2])
                for n, v in zip(names, r[5:9]):
                    if v.strip().lower() == "active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def hbm_share(dof_per_s, precision, iorder):
    """Algorithmic HBM throughput of a DOF-update rate (2s bytes per DOF for a
    plain stage, 3s for one that folds in Q^n) and its fraction of the
    measured HBM copy rate."""
    from hermeshd_gb300 import perfmodel
    gbs = dof_per_s * perfmodel.bytes_per_dof_stage(precision, iorder) / 1e9
    return {"algorithmic_gbs": gbs, "frac_hbm": gbs / peaks()["hbm_gbs"], "peak_source": peaks()["source"]}


def peaks():
    p = {"hbm_gbs": FALLBACK_HBM_GBS, "source": "fallback"}
    f = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(f):
        d = json.load(open(f))
        if d.get("hbm_gbs"):
            p = {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return p


def alu_peaks():
    """FP64 and FP32 (non-tensor) GEMM throughput measured here with torch
    (cuBLAS); MEASURED_PEAKS.json carries only HBM and bf16."""
    import torch
    out = {}
    torch.backends.cuda.matmul.allow_tf32 = False
    for name, dt, n, reps in (("fp64_tflops", torch.float64, 4096, 3), ("fp32_tflops", torch.float32, 8192, 5)):
        a = torch.randn(n, n, device="cuda", dtype=dt)
        b = torch.randn(n, n, device="cuda", dtype=dt)
        torch.matmul(a, b)
        torch.cuda.synchronize()
        best = 1e9
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            torch.matmul(a, b)
            e1.record()
            torch.cuda.synchronize()
            best = min(best, e0.elapsed_time(e1) * 1e-3)
        out[name] = 2 * n ** 3 / best / 1e12
        del a, b
    torch.cuda.empty_cache()
    return out


def bench_config(cfg, ws):
    """The workload description both arms (--impl ours and --impl reference)
    print, key for key."""
    return {"workload": WORKLOAD.format(n=cfg.nx), "nx": cfg.nx, "ny": cfg.ny, "nz": cfg.nz, "nQ": 11,
            "nbasis": cfg.nbasis, "dof": cfg.dof, "rk_stages": cfg.stages,
            "l2": "GPU arm: 256 MiB written to flush L2 before every timed step",
            "parallelism": "replicas" if ws > 1 else "single GPU"}


# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# the one-kernel cell update from an ncu capture: the configuration it was
# captured on and the bytes (profiles/k_cell_vortex256_f64.txt)
CELL_CAPTURE = {"nbasis": 10, "precision": "fp64", "cells": 256 * 256, "bytes": 380e6}


def cell_traffic(cfg):
    """DRAM bytes per launch of the cell update: the ncu capture scaled by
    cells, plus the split update's volume-term round trip (nQ x nbasis values
    per cell written and read once, counted).  None for a configuration the
    capture does not describe."""
    c = CELL_CAPTURE
    if cfg.nbasis != c["nbasis"] or cfg.precision != c["precision"]:
        return None, None
    es = 8 if cfg.precision == "fp64" else 4
    vol = 2.0 * 11 * cfg.nbasis * es
    t = c["bytes"] * cfg.ncells / c["cells"] + vol * cfg.ncells
    return t, (f"ncu dram__bytes_read.sum + dram__bytes_write.sum of one one-kernel cell update "
               f"({c['bytes'] / 1e6:.0f} MB at {c['cells']} cells, nbasis {c['nbasis']}, {c['precision']}), "
               f"scaled by cells, plus the split update's volume-term buffer "
               f"(2 x 11 x {cfg.nbasis} x {es} B per cell, counted)")


# ---------------------------------------------------------------------------
def time_steps(solver, q, q1, steps, flush):
    """Per-step device time (s) with CUDA events on the kernels' own stream,
    an L2 flush on that stream before every step."""
    import torch
    st = torch.cuda.ExternalStream(solver.cuda_stream)
    evs = []
    with torch.cuda.stream(st):
        for _ in range(steps):
            flush.fill_(1)
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            solver.enqueue_steps(q, q1, 1)
            e1.record(st)
            evs.append((e0, e1))
    torch.cuda.synchronize()
    return [a.elapsed_time(b) * 1e-3 for a, b in evs]


def run_ours(args, rank, ws):
    import numpy as np
    import torch

    from hermeshd_gb300 import autotune, config, ic, perfmodel
    from hermeshd_gb300.solver import Ensemble, Solver

    dev = torch.device("cuda", torch.cuda.current_device())
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=dev)
    K, W = args.steps, args.warmup
    cfg = config.isentropic_vortex_2d(n=args.n)
    Q0 = ic.isentropic_vortex(cfg)
    s = Solver(cfg)
    q, q1 = s.from_numpy(Q0), s.new_state()
    s.advance(q, q1, W)
    tune = autotune.autotune(s, q, steps=3, repeats=2, use_cache=False)
    barrier(ws)
    with ClockSampler(torch.cuda.current_device()) as clk:
        times = time_steps(s, q, q1, K, flush)
    clocks = clk.summary()
    qg64 = q.clone()          # FP64 state after W + K steps, the reference for the FP32 error
    dof_stage = cfg.dof * cfg.stages
    value, elapsed = replica_throughput(dof_stage * K, sum(times), ws)
    ms_per_step = 1e3 * elapsed / K
    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": ws, "steps": K, "warmup": W,
           "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": "f64", "data": "synthetic",
           "config": bench_config(cfg, ws), "timing": "CUDA events per step on the kernels' stream",
           "clocks": clocks,
           "autotune": {"launch": tune["launch"], "tuned_ms_per_step": tune["ms_per_step"],
                        "default_ms_per_step": tune["default_ms_per_step"], "trials": len(tune["trials"])}}

    # ---- end to end through the C ABI with host buffers -----------------
    qh = torch.empty(cfg.shape_c, dtype=torch.float64, pin_memory=True)
    qh.copy_(torch.from_numpy(np.ascontiguousarray(Q0.T)))
    qhn = qh.numpy()
    s.advance_host(qhn, 1)
    Ke = max(3, K // 2)
    t0 = time.perf_counter()
    for _ in range(Ke):
        s.advance_host(qhn, 1)
    e2e_s = max_over_ranks(time.perf_counter() - t0, ws)
    qbytes = int(np.prod(cfg.shape_c)) * 8
    out["e2e"] = {"value": ws * dof_stage * Ke / e2e_s, "unit": UNIT, "h2d_bytes_per_step": qbytes,
                  "d2h_bytes_per_step": qbytes, "steps": Ke,
                  "path": "hermes_advance_host (pinned host array -> H2D, one step whose last stage stores the new "
                          "state into the pinned array over the host link, synchronise)"}

    # ---- per-kernel device times (event pairs around every launch) ------
    s.profile(True)
    torch.cuda.synchronize()
    st = torch.cuda.ExternalStream(s.cuda_stream)
    with torch.cuda.stream(st):
        for _ in range(K):
            flush.fill_(1)
            s.enqueue_steps(q, q1, 1)
    prof = s.profile_read()
    s.profile(False)
    # the repository's kernels launched per step: the profiled kinds (the
    # split cell update is two launches under one kind) and k_dt_finalize
    lk = s.get_launch()
    per_step = (sum(n for _, n in prof.values()) + (prof["cell"][1] if lk["split_update"] else 0)) / K + 1
    out["gpu_launches"] = int(round(per_step * K))
    out["gpu_launches_per_step"] = per_step
    total = sum(v[0] for v in prof.values())
    kern = {k: {"launches": n, "ms_total": ms, "ms_avg": ms / max(n, 1), "share": ms / total}
            for k, (ms, n) in prof.items()}
    top = max(kern, key=lambda k: kern[k]["ms_total"])
    pk = peaks()
    sbytes = perfmodel.bytes_per_dof_stage(cfg.precision, cfg.iorder)
    # algorithmic bytes per launch: the cell kernel is the stage (reads the
    # stage input and Q^n, writes the output); a face kernel reads the state
    per_launch = {"cell": cfg.dof * sbytes, "face_x": cfg.dof * 8.0, "face_y": cfg.dof * 8.0,
                  "face_z": cfg.dof * 8.0, "limiter": cfg.dof * 8.0 * 5 / 11, "cfl_dt": cfg.ncells * 5 * 8.0}
    ach = per_launch[top] / (kern[top]["ms_avg"] * 1e-3) / 1e9
    traffic, traffic_source = cell_traffic(cfg) if top == "cell" else (None, None)
    out["roofline"] = {"bound": "hbm", "kernel": top, "achieved": ach, "peak": pk["hbm_gbs"], "unit": "GB/s",
                       "frac": ach / pk["hbm_gbs"], "peak_source": pk["source"], "traffic": traffic,
                       "traffic_source": traffic_source,
                       "algorithmic_bytes_per_launch": per_launch[top], "kernels": kern}
    fl = perfmodel.flops_per_cell_stage(cfg)
    try:
        ap = alu_peaks()
    except Exception as e:  # pragma: no cover
        ap = {"error": str(e)}
    step_flops = fl["total"] * cfg.ncells * cfg.stages
    out["alu"] = {"bound_by": "fp64 pipe", "flops_per_cell_stage": fl, "achieved_tflops": step_flops / (ms_per_step * 1e-3) / 1e12,
                  "peak": ap, "frac_fp64": (step_flops / (ms_per_step * 1e-3) / 1e12) / ap["fp64_tflops"] if "fp64_tflops" in ap else None,
                  "flop_model": "reference algorithm: nonzero table products (FMA = 2), division/sqrt = 1"}
    ex_flops = sum(EXECUTED_FLOPS_VORTEX.values()) * cfg.ncells * cfg.stages
    ex_tf = ex_flops / (ms_per_step * 1e-3) / 1e12
    out["alu"]["executed"] = {
        "flops_per_cell_stage": EXECUTED_FLOPS_VORTEX, "achieved_tflops": ex_tf,
        "frac_fp64": ex_tf / ap["fp64_tflops"] if "fp64_tflops" in ap else None,
        "source": "ncu smsp__sass_thread_inst_executed_op_{dfma,dadd,dmul}_pred_on.sum, one launch per kernel "
                  "at 256x256, per cell (profiles/fp64_ops_vortex256_f64.txt)"}
    s.close()

    # ---- variants -------------------------------------------------------
    if not args.no_variants:
        out["variants"] = variants(args, cfg, Q0, qg64, flush, dev, ws, value)

    # ---- CPU baseline: the oracle on this host's cores ------------------
    if rank == 0 and not args.no_cpu:
        out["cpu_baseline"] = cpu_baseline(cfg, Q0, steps=6)
    return out


def variants(args, cfg64, Q0, qg64, flush, dev, ws, value64):
    import numpy as np
    import torch

    from hermeshd_gb300 import autotune, config, ic
    from hermeshd_gb300.solver import Ensemble, Solver

    K, W = args.steps, args.warmup
    res = {}
    # FP32 vortex, error vs the FP64 GPU state after the same number of steps
    c32 = cfg64.replace(precision="fp32")
    s = Solver(c32)
    q, q1 = s.from_numpy(Q0), s.new_state()
    s.advance(q, q1, W)
    times = time_steps(s, q, q1, K, flush)
    el = max_over_ranks(sum(times), ws)
    v32 = ws * c32.dof * c32.stages * K / el
    e = (q.double() - qg64).norm() / qg64.norm()
    res["fp32"] = {"value": v32, "unit": UNIT, "ms_per_step": 1e3 * el / K, "dtype": "f32",
                   "rel_l2_vs_fp64": float(e), "speedup_vs_fp64": v32 / value64,
                   "hbm": hbm_share(v32, "fp32", c32.iorder)}
    s.close()

    # FP32 batched ensemble against the FP64 batched ensemble of the same 256
    # boxes (and the plain FP64 path on one 48^3 box), with and without the
    # stochastic stress; its accuracy on the same draw, Roe and HLLC
    res.update(ensembles(args, flush, ws))
    res["vortex_one_period"] = vortex_one_period(cfg64)
    res["adjoint_poiseuille"] = adjoint_poiseuille()
    res["tgv64"] = tgv64()
    res["sod256"] = sod256()
    res["derived_fields"] = derived_fields(cfg64, Q0, flush)
    res["checkpoint_io"] = checkpoint_io(cfg64, Q0)
    return res


def vortex_one_period(cfg, T=10.0):
    """The headline vortex advected for one period (t >= 10, the mean flow
    (1, 1) crosses the 10 x 10 box once), FP64 and FP32: the relative L2 and
    largest error of the cell-average density against the exactly advected
    solution averaged over each cell (5 x 5 Gauss points,
    initialcon.f90:158-177), beside the same error of the initial state (the
    reference's initial condition samples the cell centres, so its own
    deviation from the exact averages is the floor)."""
    import numpy as np

    from hermeshd_gb300 import ic
    from hermeshd_gb300.solver import Solver

    Q0 = ic.isentropic_vortex(cfg)
    ex0 = ic.isentropic_vortex_exact(cfg, 0.0, quad=5)
    r0 = Q0[:, :, 0, 0, 0]
    out = {"t_target": T, "initial_state": {"rel_l2": float(np.linalg.norm(r0 - ex0) / np.linalg.norm(ex0)),
                                            "max_abs": float(np.abs(r0 - ex0).max())}}
    for prec in ("fp64", "fp32"):
        c = cfg.replace(precision=prec)
        s = Solver(c)
        q, q1 = s.from_numpy(Q0), s.new_state()
        t, n = 0.0, 0
        while t < T:
            k = 100 if t < T - 0.5 else 1
            t, _ = s.advance(q, q1, k, t=t)
            n += k
        rho = s.to_numpy(q)[:, :, 0, 0, 0]
        s.close()
        ex = ic.isentropic_vortex_exact(cfg, t, quad=5)
        out[prec] = {"steps": n, "t_end": t, "rel_l2": float(np.linalg.norm(rho - ex) / np.linalg.norm(ex)),
                     "max_abs": float(np.abs(rho - ex).max())}
    out["definition"] = ("cell-average density (coefficient 1 of rho) against the exact solution at t_end "
                         "averaged over each cell; relative L2 over the grid")
    return out


def adjoint_poiseuille(nsteps=200, every=20):
    """The 64x128 channel (ivis 1, Roe, body force 1e-3, mu = 0.05, velocity
    perturbation 1e-3 seed 0): gradient of the outflow kinetic energy after
    200 steps with respect to mu and the perturbation field by the
    checkpointed adjoint, its wall time, and its agreement with central
    differences of the same forward map (mu: h = 1e-4 mu; perturbation: one
    random direction, h = 1e-4)."""
    import time

    import torch

    from hermeshd_gb300 import config
    from hermeshd_gb300.adjoint import (Rollout, channel_perturbation, channel_state, outflow_kinetic_energy,
                                        rollout)

    cfg = config.poiseuille_2d()
    mu0, p = 0.05, 1.0
    roll = Rollout(cfg, checkpoint_every=every)
    pert = channel_perturbation(cfg, 1e-3, 0).requires_grad_(True)
    mu = torch.tensor(mu0, dtype=torch.float64, device=pert.device, requires_grad=True)
    # warm-up outside the timed region: context creation and the first launch
    # of every kernel involved (lazy module loading)
    pw = pert.detach().clone().requires_grad_(True)
    cw = torch.tensor(p / mu0, dtype=torch.float64, device=pw.device)
    outflow_kinetic_energy(rollout(channel_state(cfg, pw), cw, roll, 2), cfg).backward()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    qf = rollout(channel_state(cfg, pert), p / mu, roll, nsteps)
    L = outflow_kinetic_energy(qf, cfg)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    L.backward()
    torch.cuda.synchronize()
    t2 = time.perf_counter()

    def loss(pt, m):
        q, _, _ = roll.forward(channel_state(cfg, pt), p / m, nsteps)
        return float(outflow_kinetic_energy(q, cfg))

    hm = 1e-4 * mu0
    fd_mu = (loss(pert.detach(), mu0 + hm) - loss(pert.detach(), mu0 - hm)) / (2 * hm)
    g = torch.Generator(device=pert.device).manual_seed(7)
    D = torch.randn(pert.shape, generator=g, dtype=pert.dtype, device=pert.device) * 1e-3
    hp = 1e-4
    fd_p = (loss(pert.detach() + hp * D, mu0) - loss(pert.detach() - hp * D, mu0)) / (2 * hp)
    adj_mu, adj_p = float(mu.grad), float((D * pert.grad).sum())
    return {"config": {"grid": "64x128x1", "nbasis": 4, "ivis": 1, "riemann": "Roe (ihllc 2)", "rk": "SSP-RK2",
                       "steps": nsteps, "checkpoint_every": every, "mu": mu0, "body_force": 1e-3,
                       "perturbation": "Gaussian cell-average velocity, amplitude 1e-3, seed 0",
                       "observable": "kinetic energy of the cell column at x = lx (cell averages x dx dy)"},
            "L": float(L.detach()), "dL_dmu": adj_mu, "dL_dpert_norm": float(pert.grad.norm()),
            "forward_s": t1 - t0, "backward_s": t2 - t1, "backward_over_forward": (t2 - t1) / (t1 - t0),
            "fd_dL_dmu": fd_mu, "rel_err_mu_vs_fd": abs(adj_mu - fd_mu) / abs(adj_mu),
            "fd_dL_dpert_dir": fd_p, "rel_err_pert_vs_fd": abs(adj_p - fd_p) / abs(adj_p),
            "limiter_events": roll.limiter_events}


def tgv64(nsteps=200, oracle_steps=20):
    """The 3-D Taylor-Green vortex, 10-moment ivis 1, 64^3, nb 4, RK3, Mach
    0.1, Re 400 (symmetry broken by 1e-3, seed 1): 200 steps in FP64 and in
    FP32 (FP64 CFL, limiter fixes and conservation sums), device time of the
    200 steps by CUDA events, FP32 relative L2 from the FP64 state, and the
    FP64 conservation sums' drift."""
    import numpy as np
    import torch

    from hermeshd_gb300 import config, ic
    from hermeshd_gb300.solver import Solver

    out, states = {}, {}
    for prec in ("fp64", "fp32"):
        cfg = config.taylor_green_3d(n=64, precision=prec)
        s = Solver(cfg)
        q0 = s.from_numpy(ic.taylor_green(cfg, perturb=1e-3, seed=1))
        q, q1 = q0.clone(), s.new_state()
        s.enqueue_steps(q, q1, 1)                 # graph capture outside the timed region
        q.copy_(q0)
        s.set_time(0.0)
        c0 = s.conserved(q)
        st = torch.cuda.ExternalStream(s.cuda_stream)
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(st)
        s.enqueue_steps(q, q1, nsteps)
        b.record(st)
        b.synchronize()
        ms = a.elapsed_time(b)
        c1 = s.conserved(q)
        drift = np.abs(c1[0] - c0[0]) / np.maximum(np.abs(c0[0]), 1e-300)
        val = cfg.dof * cfg.stages * nsteps / (ms * 1e-3)
        out[prec] = {"value": val, "unit": UNIT, "ms_per_step": ms / nsteps, "hbm": hbm_share(val, prec, cfg.iorder),
                     "conservation_rel_drift": {"mass": float(drift[0]), "energy": float(drift[4])}}
        states[prec] = q.double()
        s.close()
    out["fp32"]["rel_l2_vs_fp64"] = float((states["fp32"] - states["fp64"]).norm() / states["fp64"].norm())
    out["fp32"]["speedup_vs_fp64"] = out["fp32"]["value"] / out["fp64"]["value"]
    out["config"] = {"grid": "64^3", "nbasis": 4, "ivis": 1, "riemann": "HLLC", "rk": "SSP-RK3", "steps": nsteps}
    out["vs_fp64_oracle"] = tgv_vs_oracle(oracle_steps)
    return out


def tgv_vs_oracle(steps):
    """FP64 and FP32 Taylor-Green 64^3 states after `steps` steps against the
    FP64 oracle's (all host cores) from the same initial state."""
    import numpy as np

    from hermeshd_gb300 import config, ic
    from hermeshd_gb300.solver import Solver

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = config.taylor_green_3d(n=64, precision="fp64")
    Q0 = ic.taylor_green(cfg, perturb=1e-3, seed=1)
    O.set_num_threads(os.cpu_count() or 1)
    Qo = Q0.copy(order="F")
    t0 = time.perf_counter()
    to, _ = O.Oracle(cfg).advance(Qo, steps)
    oracle_s = time.perf_counter() - t0
    res = {"steps": steps, "oracle_wall_s": oracle_s}
    for prec in ("fp64", "fp32"):
        s = Solver(cfg.replace(precision=prec))
        q, q1 = s.from_numpy(Q0), s.new_state()
        t, _ = s.advance(q, q1, steps)
        g = s.to_numpy(q)
        s.close()
        res[prec] = {"rel_l2": float(np.linalg.norm(g - Qo) / np.linalg.norm(Qo)), "t_rel_diff": abs(t - to) / to}
    res["note"] = (f"the oracle's {steps} steps of 64^3 take about {oracle_s:.0f} s on the host cores; its 200 "
                   "are left to the FP64 GPU state, which holds the oracle to rounding")
    return res


def sod256():
    """The 1-D Sod shock tube of the CPU-runnable configuration (256 cells,
    nb 4, HLLC, RK2, CFL 0.3) to t = 0.2: wall time through hermes_advance on
    the GPU (one launch of steps per CUDA graph, read-back every 50 steps)
    and the oracle on the host cores."""
    import time

    import torch

    from hermeshd_gb300 import config, ic
    from hermeshd_gb300.solver import Solver

    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O

    cfg = config.sod_1d(nx=256)
    s = Solver(cfg)

    def run_gpu():
        q, q1 = s.from_numpy(ic.sod(cfg)), s.new_state()
        t, n = 0.0, 0
        while t < cfg.tf:
            t, dt = s.advance(q, q1, 50, t=t)
            n += 50
        return n, t

    run_gpu()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    n, t = run_gpu()
    gpu_s = time.perf_counter() - t0
    o = O.Oracle(cfg)
    Q = ic.sod(cfg)
    t0 = time.perf_counter()
    tt, steps = 0.0, 0
    while tt < cfg.tf:
        tt, _ = o.advance(Q, 50, t=tt)
        steps += 50
    cpu_s = time.perf_counter() - t0
    s.close()
    dofs = cfg.dof * cfg.stages * n / gpu_s
    return {"steps": n, "t_end": t, "gpu_wall_s": gpu_s, "oracle_wall_s": cpu_s, "oracle_threads": O.num_threads(),
            "value": dofs, "unit": UNIT, "hbm": hbm_share(dofs, "fp64", cfg.iorder),
            "note": "256 cells fill 2 of 152 SMs: launch-latency bound on the GPU"}


def derived_fields(cfg, Q0, flush, reps=20):
    """The VTK derived fields (all 14 variables, float32) of the 128x128 vortex
    state (nvtk 1 and 2) and of a 512x512 vortex (230 MB, above L2) on the
    device: time per launch by CUDA events on the kernels' stream, L2 flushed
    before each launch, and HBM throughput from the algorithmic bytes (8 of
    the 11 variables' coefficients read, FP64; 14 float32 values written per
    sub-cell)."""
    import torch

    from hermeshd_gb300.output import VARIABLES, derived
    from hermeshd_gb300.solver import Solver

    from hermeshd_gb300 import config as _config

    res = {}
    for n, nvtk in ((cfg.nx, 1), (cfg.nx, 2), (512, 1)):
        c = cfg if n == cfg.nx else _config.isentropic_vortex_2d(n=n)
        s = Solver(c)
        if n == cfg.nx:
            q = s.from_numpy(Q0)
        else:
            q = s.init_state(s.new_state(), 2)
        st = torch.cuda.ExternalStream(s.cuda_stream)
        out, _ = derived(s, q, VARIABLES, nvtk)
        ms = []
        for _ in range(reps):
            flush.fill_(1)
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record(st)
            derived(s, q, VARIABLES, nvtk, out=out)
            b.record(st)
            b.synchronize()
            ms.append(a.elapsed_time(b))
        ms_avg = sum(ms) / len(ms)
        nbytes = c.ncells * 8 * c.nbasis * 8 + c.ncells * nvtk ** 3 * len(VARIABLES) * 4
        gbs = nbytes / (ms_avg * 1e-3) / 1e9
        res[f"vortex{n}_nvtk{nvtk}"] = {"ms_per_launch": ms_avg, "algorithmic_bytes": nbytes, "achieved_gbs": gbs,
                                        "frac_hbm": gbs / peaks()["hbm_gbs"], "peak_source": peaks()["source"]}
        s.close()
        del q, out
    return res


def checkpoint_io(cfg, Q0, reps=3):
    """writeQ/readQ text checkpoints of the vortex state (FP64, 1.8 M values)
    through the library: device -> pinned host copy + multi-threaded format
    + write, and read + parse; MB of FP64 state per second."""
    import tempfile
    import time

    import numpy as np
    import torch

    from hermeshd_gb300 import checkpoint
    from hermeshd_gb300.solver import Solver

    s = Solver(cfg)
    q = s.from_numpy(Q0)
    mb = Q0.size * 8 / 1e6
    with tempfile.TemporaryDirectory() as d:
        path = os.path.join(d, checkpoint.checkpoint_name())
        tw, tr = [], []
        for _ in range(reps):
            torch.cuda.synchronize()
            t0 = time.perf_counter()
            checkpoint.write(path, q, 1.0, 0.01, 2)
            tw.append(time.perf_counter() - t0)
            t0 = time.perf_counter()
            R, *_ = checkpoint.read(path, cfg)
            tr.append(time.perf_counter() - t0)
        size = os.path.getsize(path)
        exact = bool(np.array_equal(R, s.to_numpy(q)))
    s.close()
    return {"state_mb": mb, "file_mb": size / 1e6, "write_mb_s": mb / min(tw), "read_mb_s": mb / min(tr),
            "round_trip_bit_exact": exact, "host_threads": os.cpu_count()}


ENS_BOXES, ENS_SIZES = 256, (16, 24, 32, 48)


def ensemble_draw(nbox=ENS_BOXES, seed=0):
    """Box extents of the fluctuating-hydro ensemble: nbox cubes with edges
    drawn uniformly from {16, 24, 32, 48} (numpy default_rng(seed)), all with
    the 48^3 box's cell size; Philox key = realisation id."""
    import numpy as np
    sizes = np.random.default_rng(seed).choice(ENS_SIZES, size=nbox)
    return [(int(n),) * 3 for n in sizes]


def make_ensemble(base, dims):
    from hermeshd_gb300.solver import Ensemble
    dx = base.lx / 48
    ens = Ensemble(base, dims, [(d[0] * dx, d[1] * dx, d[2] * dx) for d in dims], seeds=list(range(len(dims))))
    q, q1 = ens.new_state(), ens.new_state()
    equilibrate(ens, q)
    return ens, q, q1


def equilibrate(ens, q):
    """rho = 1, T = 1 (p = 1), v = 0 in every box; time and noise counter 0."""
    for i in range(ens.nbox):
        v = ens.box_view(q, i)
        v.zero_()
        v[0, 0].fill_(1.0)
        v[0, 4].fill_(1.0 / (ens.cfg.aindex - 1.0))
    ens.set_time(0.0)
    ens.set_noise_step(0)


def time_ensemble(base, dims, K, flush, ws, tune=True):
    """Device time of K steps of the batched ensemble (after 2 warm-up steps
    and, with tune, the autotuner), CUDA events per step, L2 flushed."""
    from hermeshd_gb300 import autotune
    ens, q, q1 = make_ensemble(base, dims)
    ens.advance(q, q1, 2)
    tune_res = autotune.autotune(ens, q, steps=1, repeats=2, use_cache=False) if tune else None
    times = time_steps(ens, q, q1, K, flush)
    v, el = replica_throughput(ens.dof * base.stages * K, sum(times), ws)
    out = {"value": v, "unit": UNIT, "ms_per_step": 1e3 * el / K, "steps": K,
           "dtype": "f32" if base.precision == "fp32" else "f64",
           "hbm": hbm_share(v, base.precision, base.iorder)}
    if tune_res:
        out["autotune"] = {"launch": tune_res["launch"], "tuned_ms_per_step": tune_res["ms_per_step"],
                           "default_ms_per_step": tune_res["default_ms_per_step"]}
    cells, dof = ens.ncells, ens.dof
    ens.close()
    return out, cells, dof


def ensemble_accuracy(base, dims, steps, sk_every=0):
    """Relative L2 error of the ensemble-averaged density field of the FP32
    batched run against the same ensemble in FP64 (same draw, seeds and
    steps from the same equilibrium), per box size; and the density S(k) of
    the FP64 run.  sk_every > 0: the static structure factor of the density
    accumulated every sk_every steps over the run, for both precisions, with
    each run's wall time (steps and accumulation)."""
    import torch
    from hermeshd_gb300.analysis import StructureFactor
    states, acc, wall = {}, {}, {}
    for prec in ("fp32", "fp64"):
        ens, q, q1 = make_ensemble(base.replace(precision=prec), dims)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        if sk_every > 0:
            sfa = StructureFactor(kmax=8)
            done = 0
            while done < steps:
                k = min(sk_every, steps - done)
                ens.advance(q, q1, k)
                done += k
                sfa.add_state(q, base.nbasis, dims, ens.offsets)
            acc[prec] = sfa
        else:
            ens.advance(q, q1, steps)
        torch.cuda.synchronize()
        wall[prec] = time.perf_counter() - t0
        states[prec] = (ens, q)
    err = {}
    sizes = [d[0] for d in dims]
    e32, q32 = states["fp32"]
    e64, q64 = states["fp64"]
    for n in sorted(set(sizes)):
        idx = [i for i, s in enumerate(sizes) if s == n]
        a32 = torch.stack([e32.box_view(q32, i)[0, 0].double() for i in idx]).mean(0)
        a64 = torch.stack([e64.box_view(q64, i)[0, 0] for i in idx]).mean(0)
        err[int(n)] = float((a32 - a64).norm() / a64.norm())
    sf = StructureFactor(kmax=8)
    sf.add_state(q64, base.nbasis, dims, e64.offsets)
    e32.close()
    e64.close()
    del states, q32, q64
    torch.cuda.empty_cache()
    out = {"boxes": len(dims), "steps": steps, "rel_l2_ensemble_mean_density_vs_fp64": err,
           "max_rel_l2": max(err.values()), "density_S_k_fp64": {int(k): v for k, v in sf.result().items()}}
    if sk_every > 0:
        r32, r64 = acc["fp32"].result(), acc["fp64"].result()
        out["S_k_accumulated"] = {
            "every_steps": sk_every, "samples_per_box": acc["fp32"].samples // len(dims),
            "fp32": {int(k): v for k, v in r32.items()}, "fp64": {int(k): v for k, v in r64.items()},
            "max_rel_diff_fp32_vs_fp64": max(abs(r32[k] - r64[k]) / abs(r64[k]) for k in r64),
            "wall_s": wall}
    return out


def ensembles(args, flush, ws, acc_steps=40, acc_steps_hllc=20):
    """The batched fluctuating-hydro ensemble (256 periodic boxes, 10-moment
    ivis 1 + stochastic stress, nb 4, SSP-RK2, Roe): FP32 batched against the
    FP64 batched ensemble of the same draw and against the plain FP64 path on
    one 48^3 box, with and without the stochastic stress; then the accuracy
    of the FP32 ensemble means against FP64 on the same 256-box draw over
    acc_steps of the configuration's 500 steps, with Roe and with the
    reference's HLLC (the FP64 ensemble's steps dominate the bench's
    wall time, so the accuracy runs cover the first acc_steps steps)."""
    import torch
    from hermeshd_gb300 import config, ic
    from hermeshd_gb300.solver import Solver
    K = max(2, args.steps // 5)
    dims = ensemble_draw()
    out = {}
    for llns, tag in ((True, ""), (False, "_no_noise")):
        b32 = config.fh_box(48, precision="fp32", seed=0, llns=llns)
        r32, cells, dof = time_ensemble(b32, dims, K, flush, ws)
        r64, _, _ = time_ensemble(b32.replace(precision="fp64"), dims, K, flush, ws, tune=False)
        # plain FP64 on one 48^3 box of the same physics
        c64 = config.fh_box(48, precision="fp64", seed=0, llns=llns)
        s = Solver(c64)
        q = s.from_numpy(ic.equilibrium(c64))
        q1 = s.new_state()
        s.advance(q, q1, 2)
        times = time_steps(s, q, q1, K, flush)
        v1, el = replica_throughput(c64.dof * c64.stages * K, sum(times), ws)
        s.close()
        r32["config"] = {"boxes": len(dims), "sizes": "uniform from {16,24,32,48}^3, seed 0", "cells": cells,
                         "dof": dof, "nbasis": 4, "ivis": 1, "stochastic_stress": llns, "rk": "SSP-RK2",
                         "riemann": "Roe (ihllc 2)", "noise": "kT/(rho dV) = 1e-3, eta = 1, Philox key = realisation id"}
        r32["fp64_batched"] = r64
        r32["speedup_vs_fp64_batched"] = r32["value"] / r64["value"]
        r32["fp64_plain_box48"] = {"value": v1, "unit": UNIT, "ms_per_step": 1e3 * el / K,
                                   "hbm": hbm_share(v1, "fp64", c64.iorder)}
        r32["speedup_vs_fp64_plain_box48"] = r32["value"] / v1
        out["fp32_batched_ensemble" + tag] = r32
        torch.cuda.empty_cache()
    base = config.fh_box(48, precision="fp32", seed=0)
    out["fp32_batched_ensemble"]["accuracy"] = {
        "roe": ensemble_accuracy(base, dims, acc_steps),
        "hllc": ensemble_accuracy(base.replace(ihllc=1), dims, acc_steps_hllc),
        "note": "the reference's HLLC with the stress-augmented point flux is discontinuous at S_M = 0, where an "
                "equilibrium fluctuating state sits at every face, so FP32 and FP64 runs pick its branches by "
                "rounding; the Roe solver is continuous there"}
    return out


def _time_oracle(cfg, Q0, steps, warmup, timing):
    import oracle as O
    O.set_num_threads(os.cpu_count() or 1)
    o = O.Oracle(cfg, timing=timing)
    Q = Q0.copy(order="F")
    o.advance(Q, warmup)
    t0 = time.perf_counter()
    o.advance(Q, steps)
    return time.perf_counter() - t0


def cpu_baseline(cfg, Q0, steps):
    """The oracle (the reference's step restated in C, OpenMP over its (k, j)
    loops) on all host cores: the timing build (host-tuned, FMA contraction),
    with the parity build's figure beside it."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    el = _time_oracle(cfg, Q0, steps, 1, timing=True)
    el_parity = _time_oracle(cfg, Q0, steps, 1, timing=False)
    v = cfg.dof * cfg.stages * steps / el
    return {"value": v, "unit": UNIT, "cores": O.num_threads(), "kind": "port",
            "sample": f"{steps} SSP-RK3 steps of the same 128x128 vortex, FP64, OpenMP over the oracle's (k,j) loops",
            "build": "gcc " + O.timing_flags(),
            "parity_build": {"value": cfg.dof * cfg.stages * steps / el_parity,
                             "flags": "gcc -O3 -fopenmp -ffp-contract=off (the checker's build)"}}


def run_reference(args, rank, ws):
    """The reference algorithm's CPU implementation (the C restatement of the
    Fortran step; the Fortran itself needs ifort/gfortran, MPI and MKL, none of
    which exist here or on the GPU host) on all host threads, same workload
    and metric, timing build (host-tuned, FMA contraction)."""
    from hermeshd_gb300 import config, ic
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    cfg = config.isentropic_vortex_2d(n=args.n)
    nthreads = os.cpu_count() or 1
    el = _time_oracle(cfg, ic.isentropic_vortex(cfg), args.steps, args.warmup, timing=True)
    v = cfg.dof * cfg.stages * args.steps / el
    return {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1e3 * el / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": bench_config(cfg, ws), "timing": "wall clock around the oracle's advance on the host",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                             "sample": f"{args.steps} full SSP-RK3 steps after {args.warmup} warm-up steps",
                             "build": "gcc " + O.timing_flags()},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    args = parse()
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        ws = int(os.environ.get("WORLD_SIZE", "1"))
        if rank != 0:
            return 0
        print(json.dumps(run_reference(args, rank, ws)))
        return 0
    rank, ws = dist_init()
    from hermeshd_gb300 import build
    build.build()
    if args.ensemble_accuracy > 0:
        if rank == 0:
            from hermeshd_gb300 import config
            t0 = time.perf_counter()
            acc = ensemble_accuracy(config.fh_box(48, precision="fp32", seed=0), ensemble_draw(),
                                    args.ensemble_accuracy, sk_every=10)
            acc["wall_s"] = time.perf_counter() - t0
            print(json.dumps({"ensemble_accuracy": acc}))
        return 0
    out = run_ours(args, rank, ws)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
