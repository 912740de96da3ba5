"""Autotuner of the solver's launch and work-decomposition knobs.

Sweeps, per workload, the knobs that change speed but not the estimator's
expectation:

* block_threads  -- threads per block of the persistent march (128, 256);
* tile_a         -- packet shape: a warp's packet tiles tile_a x
                    (32 * cells per lane / tile_a) cells of the periodic
                    (j, k) plane (8, 16, 32);
* n_groups       -- band-group count, i.e. band-group size (bands per
                    group) for the spectral stratification (4, 8, 16 bands).

A configuration is scored by its efficiency 1 / (solve time x sum of the
per-cell variances), measured on the caller's own snapshot at a pilot ray
count, so that a faster but noisier decomposition does not win.  When the
caller solves to a target error with a floor on the rays per packet (the
optical-thickness allocation), the score is instead the inverse of the
predicted solve time at that target: the pilot's rays scaled by (pilot
error / target)^2, raised to the floor, times the pilot's time per ray --
more, smaller band groups lower the variance but put every packet at the
floor sooner, which the plain efficiency does not see.  Results are
cached in a JSON file keyed by the workload description and the device name
(DNSMC_AUTOTUNE_CACHE, default ~/.cache/dnsmc_gb300/autotune.json).
"""
from __future__ import annotations

import itertools
import json
import os
import time

import numpy as np

DEFAULT_SPACE = {"block_threads": (128, 256), "tile_a": (8, 16, 32), "group_bands": (4, 8, 16)}


def cache_path() -> str:
    return os.environ.get("DNSMC_AUTOTUNE_CACHE",
                          os.path.join(os.path.expanduser("~"), ".cache", "dnsmc_gb300", "autotune.json"))


def _device_name() -> str:
    try:
        import torch
        if torch.cuda.is_available():
            return torch.cuda.get_device_name(0)
    except Exception:
        pass
    return "unknown"


def _load(path):
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return {}


def autotune(make_solver, set_inputs, workload: str, nbands: int, rays: int = 16, space=None, repeats: int = 2,
             path: str | None = None, force: bool = False, log=None, target_error: float | None = None,
             floor: int | None = None, error_fn=None) -> dict:
    """make_solver(block_threads, tile_a, n_groups) -> Solver;
    set_inputs(solver) sets its fields (and anything else the workload needs).
    With target_error, floor and error_fn(Q, S) -> relative RMS error, the
    configurations are ranked by their predicted solve time at the target.
    Returns {"config": {...}, "results": [...], "cached": bool}."""
    space = dict(DEFAULT_SPACE if space is None else space)
    path = path or cache_path()
    at_target = target_error is not None and floor is not None and error_fn is not None
    key = f"{workload} | {_device_name()} | rays {rays} | " + json.dumps(space, sort_keys=True)
    if at_target:
        key += f" | target {target_error} floor {floor}"
    db = _load(path)
    if not force and key in db:
        out = dict(db[key])
        out["cached"] = True
        return out
    results = []
    for bt, ta, gb in itertools.product(space["block_threads"], space["tile_a"], space["group_bands"]):
        ng = max(1, nbands // gb)
        s = make_solver(bt, ta, ng)
        try:
            set_inputs(s)
            s.set_rays(rays)
            s.solve(timeout_s=600)  # warm-up: sampling tables, buffers
            ms, var, err2 = [], [], []
            for _ in range(repeats):
                Q, S = s.solve(timeout_s=600)
                ms.append(s.timing()[0])
                var.append(float((S ** 2).sum()))
                if at_target:
                    err2.append(float(error_fn(Q, S)) ** 2)
        finally:
            s.close()
        t, v = float(np.median(ms)), float(np.mean(var))
        r = {"block_threads": bt, "tile_a": ta, "group_bands": gb, "n_groups": ng, "solve_ms": t,
             "sum_var": v, "efficiency": 1.0 / (t * v) if t > 0 and v > 0 else 0.0}
        if at_target:
            # rays per packet and group for the target, at least the floor;
            # the solve time scales with the rays
            need = rays * float(np.mean(err2)) / target_error ** 2
            r["error"] = float(np.sqrt(np.mean(err2)))
            r["rays_at_target"] = max(need, float(floor))
            r["ms_at_target"] = t * r["rays_at_target"] / rays
            r["efficiency"] = 1.0 / r["ms_at_target"] if r["ms_at_target"] > 0 else 0.0
        results.append(r)
        if log:
            log(f"autotune {r}")
    best = max(results, key=lambda r: r["efficiency"])
    out = {"config": {k: best[k] for k in ("block_threads", "tile_a", "n_groups", "group_bands")},
           "results": results, "time": time.time()}
    db[key] = out
    os.makedirs(os.path.dirname(path) or ".", exist_ok=True)
    tmp = path + ".tmp"
    with open(tmp, "w") as fh:
        json.dump(db, fh, indent=1)
    os.replace(tmp, path)
    out = dict(out)
    out["cached"] = False
    return out
