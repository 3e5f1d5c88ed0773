"""Autotuner of the batching launch parameters.

Packed batches have two knobs that set how full the GPU stays: the number of
render lanes (batches in flight at once, on their own streams) and the path
slots of each lane (the queue size: camera samples per batch). The
regeneration engine has its pool size and regeneration threshold.
tune_batch() times hasty_batch_render over a calibration set of resident jobs
for every candidate, keeps the fastest by device time, and writes the result
as JSON (one file per GPU name) so later runs reuse it.

    from hastyrenderer_gb300 import autotune
    best = autotune.tune_batch(jobs, passes=4)      # jobs: resident RenderJobs
    batch_render(jobs, spp, **autotune.batch_args(best))
"""
from __future__ import annotations

import json
import os
import time

LANES = [2, 3, 4]
LANE_PATHS = [1 << 22, 1 << 23, 1 << 24]
REGEN_POOLS = [1 << 21, 1 << 22, 1 << 23]
REGEN = [0.75, 0.9, 1.0]
VERSION = 2


def default_path(gpu_name: str = "") -> str:
    base = os.environ.get("HASTY_TUNE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "hastyrenderer_gb300"))
    tag = "".join(c if c.isalnum() else "_" for c in gpu_name) or "gpu"
    return os.path.join(base, f"batch_v{VERSION}_{tag}.json")


def batch_args(result: dict) -> dict:
    """hasty_batch_render keyword arguments of a tuning result."""
    out = {"mode": int(result.get("mode", 0)), "paths_in_flight": int(result["paths_in_flight"])}
    if out["mode"] == 0:
        out["lanes"] = int(result["lanes"])
    else:
        out["regen_fraction"] = float(result["regen_fraction"])
    return out


def candidates(modes=(0, 1)) -> list[dict]:
    out = []
    if 0 in modes:
        out += [{"mode": 0, "lanes": l, "paths_in_flight": p} for l in LANES for p in LANE_PATHS]
    if 1 in modes:
        out += [{"mode": 1, "paths_in_flight": p, "regen_fraction": f} for p in REGEN_POOLS for f in REGEN]
    return out


def tune_batch(jobs, passes: int = 4, cands=None, out_path: str | None = None, repeats: int = 2) -> dict:
    """Times every candidate on `jobs` (each renders `passes` passes per
    trial; the jobs' accumulators are reset before and after) and returns the
    fastest with {"samples_per_s", "trials"}."""
    from .api import batch_render
    cands = cands or candidates()
    trials = []
    n = len(jobs)
    for c in cands:
        best_ms = None
        samples = 0
        for _ in range(repeats):
            for j in jobs:
                j.reset()
            st = batch_render(jobs, [passes] * n, **batch_args(c))
            samples = st["samples"]
            best_ms = st["device_ms"] if best_ms is None else min(best_ms, st["device_ms"])
        trials.append(dict(c, device_ms=best_ms, samples_per_s=samples / (best_ms * 1e-3)))
    for j in jobs:
        j.reset()
    best = max(trials, key=lambda t: t["samples_per_s"])
    result = dict(best, trials=trials, calibration={"jobs": n, "passes": passes}, when=time.time(), version=VERSION)
    if out_path:
        os.makedirs(os.path.dirname(out_path), exist_ok=True)
        with open(out_path, "w") as fh:
            json.dump(result, fh, indent=1)
    return result


def load(path: str) -> dict | None:
    try:
        with open(path) as fh:
            d = json.load(fh)
    except (OSError, ValueError):
        return None
    return d if d.get("version") == VERSION else None
