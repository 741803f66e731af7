"""Autotuner of the neighbour-search settings (``ndsph_tuning``).

None of the settings changes which pairs are summed; they trade the cost of
rebuilding the search structures against the cost of carrying extra
candidates in every sweep:

* ``nl_skin`` -- the neighbour rows hold every pair within
  2 max(h_i, h_j) * skin.  A thicker skin lengthens every row (each sweep
  screens more candidates) but lets the rows be kept for more steps.
* ``nl_reuse`` -- whether a step may keep the previous link (FP32 form).
* ``stencil`` -- 5: search 5^ndim stencils of half-size cells (FP32 form of
  one simulation), fewer candidates per row build; 3: 3^ndim stencils.
* ``graph_cell_margin`` -- batched captured steps size their cells
  2 hmax * margin; a step whose h outgrows the margin leaves the graph and is
  redone on the eager path, a larger margin puts more candidates in each
  cell.

The reference rebuilds its cell link list on every call of derivs
(derivs.f90:82-92, linkND.f90:45-161) and has nothing to tune; this module
is new.  ``tune_device`` and ``tune_batched`` time each candidate on a short
run of the caller's own workload (fresh contexts on copies of the state, so
the caller's simulation does not advance) and return the fastest, and cache
it per workload signature (GPU name, dimension, options that change the
sweeps, particle count rounded to a power of two) in a JSON file:
``$NDSPH_TUNE_CACHE`` or ``~/.cache/ndspmhd_gb300/tuning.json``.
"""
from __future__ import annotations

import json
import math
import os

DEVICE_CANDIDATES = [
    {"nl_reuse": 0, "nl_skin": 1.1, "stencil": 5},
    {"nl_reuse": 1, "nl_skin": 1.1, "stencil": 3},
    {"nl_reuse": 1, "nl_skin": 1.05, "stencil": 5},
    {"nl_reuse": 1, "nl_skin": 1.1, "stencil": 5},
    {"nl_reuse": 1, "nl_skin": 1.15, "stencil": 5},
    {"nl_reuse": 1, "nl_skin": 1.2, "stencil": 5},
    {"nl_reuse": 1, "nl_skin": 1.3, "stencil": 5},
]
BATCHED_CANDIDATES = [
    {"graph_cell_margin": m, "nl_skin": s} for m in (1.02, 1.05, 1.1) for s in (1.05, 1.1, 1.2)
]


def _cache_path() -> str:
    p = os.environ.get("NDSPH_TUNE_CACHE")
    if p:
        return p
    return os.path.join(os.path.expanduser("~"), ".cache", "ndspmhd_gb300", "tuning.json")


def _device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(torch.cuda.current_device())
    except Exception:
        pass
    return "unknown"


def signature(opts: dict, n: int, batched: bool = False) -> str:
    """Cache key: what changes the relative cost of the candidates."""
    keys = ("ndim", "precision", "imhd", "idust", "iener", "learned_h")
    parts = [f"{k}={opts.get(k, 0)}" for k in keys]
    parts.append(f"ibound={list(opts.get('ibound', [0, 0, 0]))[:opts['ndim']]}")
    parts.append(f"n~2^{int(round(math.log2(max(n, 1))))}")
    parts.append("batched" if batched else "single")
    return f"{_device_name()}|" + ",".join(parts)


def load_cache() -> dict:
    p = _cache_path()
    try:
        with open(p) as f:
            return json.load(f)
    except (OSError, ValueError):
        return {}


def _save(key: str, entry: dict) -> None:
    p = _cache_path()
    data = load_cache()
    data[key] = entry
    try:
        os.makedirs(os.path.dirname(p), exist_ok=True)
        tmp = p + ".tmp"
        with open(tmp, "w") as f:
            json.dump(data, f, indent=1, sort_keys=True)
        os.replace(tmp, p)
    except OSError:
        pass   # a read-only home: the result is still returned


def _time_device(opts: dict, state: dict, tuning: dict, steps: int, warmup: int) -> float:
    from .gpu import GpuSPH
    g = GpuSPH(opts, {k: v.copy() for k, v in state.items()})
    try:
        g.set_tuning(**tuning)
        g.dev_upload()
        g.set_dt(0.0)
        g.dev_step(warmup)
        g.dev_step(steps)
        return g.timing()["total_ms"] / steps
    finally:
        g.close()


def tune_device(opts: dict, state: dict, candidates=None, steps: int = 6, warmup: int = 3,
                use_cache: bool = True) -> dict:
    """Fastest tuning of the device-resident step for this workload.

    ``state`` is a full particle state (after primitive2conservative).
    Returns ``{"tuning": {...}, "ms_per_step": t, "trials": [...],
    "cached": bool}``.
    """
    key = signature(opts, state["x"].shape[0])
    if use_cache:
        hit = load_cache().get(key)
        if hit:
            return dict(hit, cached=True)
    trials = []
    for cand in (candidates or DEVICE_CANDIDATES):
        ms = _time_device(opts, state, cand, steps, warmup)
        trials.append({"tuning": dict(cand), "ms_per_step": round(ms, 4)})
    best = min(trials, key=lambda t: t["ms_per_step"])
    entry = {"tuning": best["tuning"], "ms_per_step": best["ms_per_step"], "trials": trials}
    _save(key, entry)
    return dict(entry, cached=False)


def _time_batched(opts: dict, state: dict, sim, nsim: int, tuning: dict, steps: int, warmup: int) -> float:
    from .gpu import GpuSPH
    g = GpuSPH(opts, {k: v.copy() for k, v in state.items()})
    try:
        g.set_tuning(**tuning)
        g.batch_upload(sim, nsim, initialise=True)
        g.batch_set_graph(2)   # the captured step, whose cells the knobs size
        g.batch_step(warmup)
        g.batch_step(steps)
        return g.timing()["total_ms"] / steps
    finally:
        g.close()


def tune_batched(opts: dict, state: dict, sim, nsim: int, candidates=None, steps: int = 20,
                 warmup: int = 3, use_cache: bool = True) -> dict:
    """Fastest tuning of the batched captured-graph step (cell margin, skin)
    for this batch; ``state`` holds the primitive inputs batch_upload takes.
    (The fused per-tube step of 1D batches has no such knobs: its cells are
    each tube's own.)"""
    key = signature(opts, state["x"].shape[0], batched=True)
    if use_cache:
        hit = load_cache().get(key)
        if hit:
            return dict(hit, cached=True)
    trials = []
    for cand in (candidates or BATCHED_CANDIDATES):
        ms = _time_batched(opts, state, sim, nsim, cand, steps, warmup)
        trials.append({"tuning": dict(cand), "ms_per_step": round(ms, 4)})
    best = min(trials, key=lambda t: t["ms_per_step"])
    entry = {"tuning": best["tuning"], "ms_per_step": best["ms_per_step"], "trials": trials}
    _save(key, entry)
    return dict(entry, cached=False)
