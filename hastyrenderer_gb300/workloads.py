"""Seeded multi-job workloads for batching and serving.

mixed_jobs() draws the mixed-job distribution: each job is either the
procedural Cornell box or the sphere field (50, 200 or 800 subdivision-3
icospheres, i.e. 64k, 256k or 1.02M triangles) with its own seed; resolution
from {128x128, 256x192, 512x512, 1024x768}; samples per pixel log-uniform in
[16, 1024]; max depth uniform in {8..16}. All sphere-field scenes share one
2048x1024 FP32 sky file (the sky does not depend on the seed).

poisson_requests() draws a serving trace: arrival times of a Poisson process
and, per request, a scene from a pool of generated jobs plus its own
resolution, samples per pixel, depth and seed, written as a small
renderJob.json that points at the pooled scene file.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

from . import scenes

RESOLUTIONS = [(128, 128), (256, 192), (512, 512), (1024, 768)]
SPHERE_COUNTS = [50, 200, 800]


def _draw(rng):
    kind = "cornell" if rng.uniform() < 0.5 else "field"
    spheres = int(rng.choice(SPHERE_COUNTS)) if kind == "field" else 0
    w, h = RESOLUTIONS[int(rng.integers(0, len(RESOLUTIONS)))]
    spp = int(round(math.exp(rng.uniform(math.log(16.0), math.log(1024.0)))))
    depth = int(rng.integers(8, 17))
    return kind, spheres, w, h, spp, depth


def mixed_jobs(base_dir: str, n_jobs: int = 64, seed: int = 0) -> list[dict]:
    """Generates (or reuses, when already present) n_jobs scenes under
    base_dir/job_<k>; returns one dict per job: path, kind, spheres, width,
    height, spp, max_depth, seed."""
    os.makedirs(base_dir, exist_ok=True)
    rng = np.random.default_rng(seed)
    sky = os.path.join(base_dir, "sky.pfm")
    jobs = []
    for k in range(n_jobs):
        kind, spheres, w, h, spp, depth = _draw(rng)
        d = os.path.join(base_dir, f"job_{k:03d}")
        meta = {"kind": kind, "spheres": spheres, "width": w, "height": h, "spp": spp, "max_depth": depth,
                "seed": k}
        meta_path = os.path.join(d, "meta.json")
        path = os.path.join(d, "renderJob.json")
        if not (os.path.exists(path) and os.path.exists(meta_path) and json.load(open(meta_path)) == meta):
            if kind == "field" and not os.path.exists(sky):
                scenes.write_pfm(sky, scenes.sky_environment(2048, 1024))
            if kind == "cornell":
                scenes.cornell_box(d, seed=k, width=w, height=h, spp=spp, max_depth=depth)
            else:
                scenes.sphere_field(d, seed=k, n_spheres=spheres, subdiv=3, width=w, height=h, spp=spp,
                                    max_depth=depth, sky_path=sky)
            with open(meta_path, "w") as f:
                json.dump(meta, f)
        jobs.append(dict(meta, path=path))
    return jobs


def job_samples(job: dict) -> int:
    return job["width"] * job["height"] * job["spp"]


def poisson_requests(pool: list[dict], out_dir: str, rate: float, duration: float, seed: int = 1) -> list[dict]:
    """Arrival trace over `duration` seconds at `rate` requests per second.
    Each request draws its settings from the mixed distribution and its scene
    from `pool` (matching kind and sphere count when the pool has one)."""
    os.makedirs(out_dir, exist_ok=True)
    rng = np.random.default_rng(seed)
    t = 0.0
    reqs = []
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            break
        kind, spheres, w, h, spp, depth = _draw(rng)
        same = [p for p in pool if p["kind"] == kind and p["spheres"] == spheres] or pool
        src = same[int(rng.integers(0, len(same)))]
        scene_json = os.path.join(os.path.dirname(src["path"]), "scene.json")
        k = len(reqs)
        path = os.path.join(out_dir, f"req_{k:05d}.json")
        job = {"settings": {"num_samples": spp, "num_threads": 8, "width": w, "height": h,
                            "roulette_start_depth": 3 if kind == "cornell" else 1, "roulette_q": 0.3,
                            "max_depth": depth, "use_mis": True},
               "scene": os.path.abspath(scene_json), "gb300": {"seed": 1000 + k}}
        with open(path, "w") as f:
            json.dump(job, f)
        reqs.append({"t": t, "path": path, "kind": kind, "spheres": spheres, "width": w, "height": h, "spp": spp,
                     "max_depth": depth, "seed": 1000 + k})
    return reqs
