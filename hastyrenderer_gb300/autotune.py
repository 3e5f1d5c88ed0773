"""Autotuner of the multi-job engine's launch parameters.

The engine has two knobs that set how full its wavefront stays: the size of
the shared path pool (paths in flight) and the regeneration threshold (new
camera samples are issued once fewer than fraction x pool paths are alive).
tune_batch() times hasty_batch_render over a calibration set of resident jobs
for every candidate pair, keeps the fastest by device time, and writes the
result as JSON (one file per GPU name) so later runs reuse it.

    from hastyrenderer_gb300 import autotune
    best = autotune.tune_batch(jobs, passes=2)      # jobs: resident RenderJobs
    batch_render(jobs, spp, **autotune.batch_args(best))
"""
from __future__ import annotations

import json
import os
import time

POOLS = [1 << 20, 1 << 21, 1 << 22, 1 << 23]
REGEN = [0.5, 0.75, 0.9, 1.0]


def default_path(gpu_name: str = "") -> str:
    base = os.environ.get("HASTY_TUNE_DIR", os.path.join(os.path.expanduser("~"), ".cache", "hastyrenderer_gb300"))
    tag = "".join(c if c.isalnum() else "_" for c in gpu_name) or "gpu"
    return os.path.join(base, f"engine_{tag}.json")


def batch_args(result: dict) -> dict:
    return {"paths_in_flight": int(result["paths_in_flight"]), "regen_fraction": float(result["regen_fraction"])}


def tune_batch(jobs, passes: int = 2, pools=None, regen=None, out_path: str | None = None, repeats: int = 2) -> dict:
    """Times every (pool, regen) candidate on `jobs` (each renders `passes`
    passes per trial; the jobs' accumulators are reset before and after) and
    returns {"paths_in_flight", "regen_fraction", "samples_per_s", "trials"}."""
    from .api import batch_render
    pools = pools or POOLS
    regen = regen or REGEN
    trials = []
    n = len(jobs)
    for pool in pools:
        for f in regen:
            best_ms = None
            samples = 0
            for _ in range(repeats):
                for j in jobs:
                    j.reset()
                st = batch_render(jobs, [passes] * n, paths_in_flight=pool, regen_fraction=f)
                samples = st["samples"]
                best_ms = st["device_ms"] if best_ms is None else min(best_ms, st["device_ms"])
            trials.append({"paths_in_flight": pool, "regen_fraction": f, "device_ms": best_ms,
                           "samples_per_s": samples / (best_ms * 1e-3)})
    for j in jobs:
        j.reset()
    best = max(trials, key=lambda t: t["samples_per_s"])
    result = dict(best, trials=trials, calibration={"jobs": n, "passes": passes}, when=time.time())
    if out_path:
        os.makedirs(os.path.dirname(out_path), exist_ok=True)
        with open(out_path, "w") as fh:
            json.dump(result, fh, indent=1)
    return result


def load(path: str) -> dict | None:
    try:
        with open(path) as fh:
            return json.load(fh)
    except (OSError, ValueError):
        return None
