"""The seeded workload generators behind the batched and served benchmarks
(CPU only): the mixed-job distribution's ranges, and the serving trace's
Poisson arrivals and per-request job files."""
import json
import os

import numpy as np

from hastyrenderer_gb300 import workloads


def test_mixed_distribution_ranges():
    rng = np.random.default_rng(0)
    draws = [workloads._draw(rng) for _ in range(2000)]
    kinds = {d[0] for d in draws}
    assert kinds == {"cornell", "field"}
    assert {d[1] for d in draws if d[0] == "field"} == set(workloads.SPHERE_COUNTS)
    assert all(d[1] == 0 for d in draws if d[0] == "cornell")
    assert {(d[2], d[3]) for d in draws} == set(workloads.RESOLUTIONS)
    spp = np.array([d[4] for d in draws])
    assert spp.min() >= 16 and spp.max() <= 1024
    # log-uniform: about half the draws below the geometric mean (128)
    assert 0.4 < np.mean(spp < 128) < 0.6
    assert {d[5] for d in draws} == set(range(8, 17))
    # the same seed gives the same mix
    assert workloads._draw(np.random.default_rng(0)) == draws[0]


def test_poisson_trace(tmp_path):
    pool = [{"kind": "cornell", "spheres": 0, "path": str(tmp_path / "c" / "renderJob.json")},
            {"kind": "field", "spheres": 50, "path": str(tmp_path / "f" / "renderJob.json")}]
    reqs = workloads.poisson_requests(pool, str(tmp_path / "reqs"), rate=20.0, duration=30.0, seed=1)
    t = np.array([r["t"] for r in reqs])
    assert np.all(np.diff(t) > 0) and t[-1] < 30.0
    assert 450 < len(reqs) < 750                   # 600 expected at 20/s for 30 s
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert abs(gaps.mean() - 1 / 20.0) < 0.01      # exponential inter-arrival times
    for r in reqs[:20]:
        job = json.load(open(r["path"]))
        assert job["settings"]["num_samples"] == r["spp"]
        assert (job["settings"]["width"], job["settings"]["height"]) == (r["width"], r["height"])
        assert job["gb300"]["seed"] == r["seed"]
        want = "c" if r["kind"] == "cornell" else "f"   # matching kind where the pool has one
        if r["kind"] == "cornell" or r["spheres"] == 50:
            assert os.path.basename(os.path.dirname(job["scene"])) == want
    again = workloads.poisson_requests(pool, str(tmp_path / "reqs2"), rate=20.0, duration=30.0, seed=1)
    assert [r["t"] for r in again] == [r["t"] for r in reqs]
