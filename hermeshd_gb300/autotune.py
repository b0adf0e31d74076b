"""Launch-shape autotuner of a Solver or Ensemble.

The knobs are the run-time launch parameters of the step (hermes_launch in
include/hermes_gb300.h):

* ``face_tpb``         faces per block of the three face kernels (32/64/128):
                       smaller blocks spread a small grid over more SMs,
                       larger ones amortise scheduling on a large one;
* ``dt_tpb``           cells per block of the CFL reduction (64/128/256);
* ``steps_per_graph``  whole steps per CUDA graph launch (1/2/4/8): fewer
                       launches for grids so small that a step is launch-bound;
* ``noise_inline``     where the stochastic stress is drawn: its own
                       kernels staging it in device memory (0) or inside the
                       face and cell kernels (1);
* ``face_traces``      face traces evaluated once per stage by their own
                       kernel and read by the face kernels (1) or evaluated
                       by the face kernels (0); tuned where the trace kernel
                       exists (FP64, nbasis 8/10, no stochastic stress);
* ``split_update``     the cell update as the volume kernel plus a surface and
                       update kernel of one thread per (cell, variable) (1) or
                       one kernel (0); tuned where it exists (ivis 0/1);
* ``pdl``              programmatic dependent launch of the step's kernels (1)
                       or plain launches (0);
* ``faces_merged``     the face kernels: the three directions in one launch
                       (1), one launch each with a thread per face point (0),
                       or one launch each with a thread per face looping
                       over its points (2); the context's default first;
* ``tile_stage``       each stage as one fused kernel over tiles of cells (1)
                       or the separate kernels (0); tried where the context
                       has it (nbasis 4, ivis 0/1).  With it on, only
                       steps_per_graph still applies;
* ``update_tpb``       threads per block of the split update (64/128/256),
                       tuned where the split update is on;
* ``cell_concurrent``  the split update's volume kernel on a second stream
                       beside the trace and face kernels (1) or after them (0).

The cell kernel keeps 32 cells per block: its hydro and stress thread groups
must each fill whole warps (with 16 cells both groups would share one warp and
run their two code paths one after the other), and its register cap is fixed
at compile time.

Tuning is a coordinate search: each knob in turn, the others at their best so
far, each candidate timed with CUDA events over ``steps`` steps (best of
``repeats``) on a copy of the state.  It advances the context's time and
stochastic-stress step counter, so it belongs before a run; both are reset
afterwards to ``t0`` and ``step0``.  Results are cached per device and problem
signature in a JSON file ($HERMES_AUTOTUNE_CACHE, default
~/.cache/hermeshd_gb300/autotune.json).
"""
from __future__ import annotations

import json
import os
from typing import Dict, Optional, Sequence

KNOBS = {
    "face_tpb": (128, 64, 32),
    "dt_tpb": (256, 128, 64),
    "steps_per_graph": (1, 2, 4, 8),
    "noise_inline": (0, 1),          # tuned only with the stochastic stress on
    "face_traces": (1, 0),           # tuned only where the context has the trace buffer
    "split_update": (1, 0),          # tuned only where the context has the split-update buffer
    "pdl": (0, 1),
    "faces_merged": (1, 0),          # the context's default is tried first
    "tile_stage": (0, 1),            # tuned only where the context has the fused stage
    "update_tpb": (128, 64, 256),    # tuned only with the split update
    "cell_concurrent": (0, 1),       # tuned only with the split update (the context's default first)
}


def _torch():
    import torch
    return torch


def cache_path() -> str:
    return os.environ.get("HERMES_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "hermeshd_gb300", "autotune.json"))


def signature(solver) -> str:
    """Device name and the problem properties the launch shape depends on."""
    torch = _torch()
    c = solver.cfg
    dims = getattr(solver, "_dims", None)
    cells = int(sum(int(a) * int(b) * int(d) for a, b, d in dims)) if dims is not None else c.nx * c.ny * c.nz
    nbox = getattr(solver, "nbox", 1)
    return "|".join(str(x) for x in (torch.cuda.get_device_name(solver.device), c.precision, c.nbasis, c.iquad,
                                     c.ivis, c.ihllc, int(c.llns), c.iorder, nbox, cells))


def _load() -> Dict[str, dict]:
    try:
        with open(cache_path()) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _store(key: str, value: dict) -> None:
    d = _load()
    d[key] = value
    p = cache_path()
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(d, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass


def _can_tile(solver, cur) -> bool:
    """Whether the context has the fused stage (it is off by default)."""
    from ._lib import HermesError
    try:
        solver.set_launch(**dict(cur, tile_stage=1))
    except HermesError:
        return False
    solver.set_launch(**cur)
    return True


def time_steps(solver, q, q1, steps: int, repeats: int) -> float:
    """Best-of-repeats milliseconds per step, CUDA events on the kernels' stream."""
    torch = _torch()
    st = torch.cuda.ExternalStream(solver.cuda_stream)
    solver.enqueue_steps(q, q1, steps)   # first use of a launch shape captures its graphs
    best = float("inf")
    for _ in range(repeats):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        a.record(st)
        solver.enqueue_steps(q, q1, steps)
        b.record(st)
        b.synchronize()
        best = min(best, a.elapsed_time(b) / steps)
    return best


def autotune(solver, q, steps: int = 4, repeats: int = 3, use_cache: bool = True, t0: float = 0.0,
             step0: int = 0, knobs: Optional[Dict[str, Sequence[int]]] = None) -> dict:
    """Pick and apply the fastest launch shape for stepping `q` with `solver`.

    Returns {"launch": chosen, "ms_per_step": tuned, "default_ms_per_step":
    with the compiled defaults, "trials": [...], "cached": bool}."""
    key = signature(solver)
    if use_cache:
        hit = _load().get(key)
        if hit:
            solver.set_launch(**hit["launch"])
            return dict(hit, cached=True)
    knobs = dict(knobs or KNOBS)
    if not solver.cfg.llns:
        knobs.pop("noise_inline", None)
    cur = solver.get_launch()
    for k in ("face_traces", "split_update"):
        if cur[k] == 0:
            knobs.pop(k, None)
    if cur["split_update"] == 0:
        knobs.pop("update_tpb", None)
        knobs.pop("cell_concurrent", None)
    else:   # the context's current choices first
        if "cell_concurrent" in knobs:
            knobs["cell_concurrent"] = (cur["cell_concurrent"], 1 - cur["cell_concurrent"])
        if "update_tpb" in knobs:
            knobs["update_tpb"] = (cur["update_tpb"],) + tuple(u for u in (64, 128, 256) if u != cur["update_tpb"])
    if cur["tile_stage"] == 0 and not _can_tile(solver, cur):
        knobs.pop("tile_stage", None)
    if "faces_merged" in knobs:
        knobs["faces_merged"] = (cur["faces_merged"],) + tuple(m for m in (0, 1, 2) if m != cur["faces_merged"])
    qt, q1t = q.clone(), q.clone()
    best = {k: v[0] for k, v in knobs.items()}
    solver.set_launch(**best)
    default_ms = time_steps(solver, qt, q1t, steps, repeats)
    best_ms = default_ms
    trials = [dict(best, ms_per_step=default_ms)]
    for name, values in knobs.items():
        for v in values:
            if v == best[name]:
                continue
            cand = dict(best, **{name: v})
            solver.set_launch(**cand)
            ms = time_steps(solver, qt, q1t, steps, repeats)
            trials.append(dict(cand, ms_per_step=ms))
            if ms < best_ms:
                best_ms, best = ms, cand
    solver.set_launch(**best)
    solver.set_time(t0)
    solver.set_noise_step(step0)
    _torch().cuda.synchronize()
    res = {"launch": solver.get_launch(), "ms_per_step": best_ms, "default_ms_per_step": default_ms,
           "trials": trials}
    if use_cache:
        _store(key, res)
    return dict(res, cached=False)
