"""Autotuner of the batching launch parameters.

Packed batches have these knobs: the number of render lanes (batches in
flight at once, on their own streams), the path slots of each lane (the
queue size: camera samples per batch), the block shapes of the two shading
kernels, and the closest-hit grid's blocks per SM while batches overlap. The
regeneration engine has its pool size and regeneration threshold.
tune_batch() times hasty_batch_render over a calibration set of resident
jobs, stage by stage, keeps the fastest by device time, and writes the
result as JSON (one file per GPU name) so later runs reuse it.

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
RESOLVE_THREADS = [128, 256]
SAMPLE_THREADS = [256, 512]
TRACE_BLOCKS = [4, 5, 6]
REGEN_POOLS = [1 << 21, 1 << 22, 1 << 23]
REGEN = [0.75, 0.9, 1.0]
VERSION = 3
KNOBS = ("mode", "lanes", "paths_in_flight", "resolve_threads", "sample_threads", "trace_blocks_per_sm",
         "regen_fraction")


def default_path(gpu_name: str = "") -> str:
    base = os.environ.get("HASTY_TUNE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "hastyrenderer_gb300"))
    tag = "".join(c if c.isalnum() else "_" for c in gpu_name) or "gpu"
    return os.path.join(base, f"batch_v{VERSION}_{tag}.json")


def batch_args(result: dict) -> dict:
    """hasty_batch_render keyword arguments of a tuning result."""
    out = {"mode": int(result.get("mode", 0)), "paths_in_flight": int(result["paths_in_flight"])}
    if out["mode"] == 0:
        for k in ("lanes", "resolve_threads", "sample_threads", "trace_blocks_per_sm"):
            if result.get(k):
                out[k] = int(result[k])
    else:
        out["regen_fraction"] = float(result["regen_fraction"])
    return out


def _time(jobs, passes, cand, repeats):
    from .api import batch_render
    best_ms, samples = None, 0
    for _ in range(repeats):
        for j in jobs:
            j.reset()
        st = batch_render(jobs, [passes] * len(jobs), **batch_args(cand))
        samples = st["samples"]
        best_ms = st["device_ms"] if best_ms is None else min(best_ms, st["device_ms"])
    return dict(cand, device_ms=best_ms, samples_per_s=samples / (best_ms * 1e-3))


def tune_batch(jobs, passes: int = 4, out_path: str | None = None, repeats: int = 2, regen: bool = True) -> dict:
    """Times candidates on `jobs` (each renders `passes` passes per trial; the
    jobs' accumulators are reset before and after), in stages: packed lanes
    x paths per lane (queue size), then the shading kernels' block shapes,
    then the closest-hit grid cap, each stage keeping the best so far; the
    regeneration engine's pool x refill threshold beside them. Returns the
    fastest with {"samples_per_s", "trials"}."""
    trials = []

    def best_of(cands):
        res = [_time(jobs, passes, c, repeats) for c in cands]
        trials.extend(res)
        return max(res, key=lambda t: t["samples_per_s"])

    top = best_of([{"mode": 0, "lanes": l, "paths_in_flight": p} for l in LANES for p in LANE_PATHS])
    base = {k: top[k] for k in ("mode", "lanes", "paths_in_flight")}
    top = best_of([dict(base, resolve_threads=r, sample_threads=t) for r in RESOLVE_THREADS for t in SAMPLE_THREADS])
    base.update(resolve_threads=top["resolve_threads"], sample_threads=top["sample_threads"])
    top = best_of([dict(base, trace_blocks_per_sm=b) for b in TRACE_BLOCKS])
    if regen:
        r = best_of([{"mode": 1, "paths_in_flight": p, "regen_fraction": f} for p in REGEN_POOLS for f in REGEN])
        top = max(top, r, key=lambda t: t["samples_per_s"])
    for j in jobs:
        j.reset()
    result = dict({k: top[k] for k in KNOBS if k in top}, samples_per_s=top["samples_per_s"], trials=trials,
                  calibration={"jobs": len(jobs), "passes": passes}, when=time.time(), version=VERSION)
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
