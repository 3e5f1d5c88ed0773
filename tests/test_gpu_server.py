"""Serving (hasty_server_*): continuous batching of requests over packed
multi-job batches. A request's sums are bit-identical to hasty_batch_render
and to hasty_job_render_passes of the same job, seed and pass count (passes
are added in order in FP64 whatever they are batched with), under either
batch-formation policy; admission respects the memory budget; scenes are
shared; failures are reported per request."""
import os
import shutil
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["cornell", "field", "room", "room_nomis"]


def _path(name):
    return os.path.join(GOLDEN, "scenes", name, "renderJob.json")


def _batch_sums(name, passes, seed):
    from hastyrenderer_gb300 import RenderJob, batch_render
    j = RenderJob(_path(name))
    j.set_seed(seed)
    batch_render([j], [passes])
    return [j.read_sums(a)[0] for a in (0, 1, 2)], j


def _collect(srv, n, timeout_ms=120000):
    got = {}
    srv.wait_idle(timeout_ms)
    while len(got) < n:
        res = srv.poll(wait_ms=1000)
        assert res, "poll returned nothing although the server is idle"
        for r in res:
            got[r["id"]] = r
    return got


def test_server_results_equal_batch():
    from hastyrenderer_gb300 import Server
    reqs = [("cornell", 3, 11), ("field", 5, 12), ("room", 2, 13), ("room_nomis", 4, 14), ("cornell", 6, 15),
            ("field", 1, 16)]
    with Server(paths_in_flight=1 << 15, max_resident_jobs=4, quantum_samples=3000) as srv:
        ids = [srv.submit(_path(n), passes=p, seed=s) for n, p, s in reqs]
        got = _collect(srv, len(ids))
        st = srv.stats()
        assert st["completed"] == len(reqs) and st["failed"] == 0
        assert st["resident_scenes"] <= len(NAMES)   # the two cornell / field requests share their scene
        for rid, (name, p, seed) in zip(ids, reqs):
            r = got[rid]
            assert r["status"] == 0, r["error"]
            assert r["passes"] == p and r["samples"] == p * r["width"] * r["height"]
            assert r["submit_ms"] <= r["admit_ms"] <= r["finish_ms"]
            ref, job = _batch_sums(name, p, seed)
            for aov in (0, 1, 2):
                assert np.array_equal(srv.read_sums(rid, aov), ref[aov]), (name, aov)
            np.testing.assert_array_equal(srv.read(rid), job.compute_estimate())
            srv.release(rid)


@pytest.mark.parametrize("policy", [0, 1], ids=["round_robin", "shortest_first"])
def test_server_alone_equals_mixed(policy):
    """The same request alone on an idle server and among many others, and
    equal to the single-job path."""
    from hastyrenderer_gb300 import RenderJob, Server
    with Server(paths_in_flight=1 << 14, quantum_samples=2048, policy=policy, lanes=3) as srv:
        rid = srv.submit(_path("room"), passes=3, seed=99)
        _collect(srv, 1)
        alone = srv.read_sums(rid)
        others = [srv.submit(_path(n), passes=4, seed=7) for n in NAMES]
        rid2 = srv.submit(_path("room"), passes=3, seed=99)
        others += [srv.submit(_path(n), passes=2, seed=8) for n in NAMES]
        _collect(srv, len(others) + 1)
        assert np.array_equal(srv.read_sums(rid2), alone)
        plain = RenderJob(_path("room"))
        plain.set_seed(99)
        plain.render_passes(3, sync=True)
        assert np.array_equal(plain.read_sums()[0], alone)


def test_server_memory_budget_admission():
    """A budget that holds the render lanes, one scene and one request at a time:
    requests still all finish, one after another, within the budget."""
    from hastyrenderer_gb300 import Server
    cfg = dict(paths_in_flight=1 << 14, max_resident_jobs=4)
    peaks = []
    for name in ("field", "cornell", "room"):   # footprint of each scene alone, same engine
        with Server(**cfg) as probe:
            probe.submit(_path(name), passes=1)
            _collect(probe, 1)
            peaks.append(probe.stats()["peak_resident_bytes"])
    budget = max(peaks) + 4096
    with Server(memory_budget=budget, max_resident_scenes=1, **cfg) as srv:
        ids = [srv.submit(_path(n), passes=2, seed=5) for n in ("field", "cornell", "field", "room")]
        got = _collect(srv, len(ids))
        assert all(got[i]["status"] == 0 for i in ids), [got[i]["error"] for i in ids]
        st = srv.stats()
        assert st["peak_resident_bytes"] <= budget
        ref, _ = _batch_sums("cornell", 2, 5)
        assert np.array_equal(srv.read_sums(ids[1]), ref[0])


def test_server_failures_reported_per_request():
    from hastyrenderer_gb300 import HastyError, Server
    with tempfile.TemporaryDirectory() as d:
        bad = os.path.join(d, "bad")
        shutil.copytree(os.path.join(GOLDEN, "scenes", "cornell"), bad)
        with open(os.path.join(bad, "scene.obj"), "w") as f:
            f.write("v 0 0 0\nf 1 2 3\n")   # vertex index out of range
        with Server(paths_in_flight=1 << 14) as srv:
            with pytest.raises(HastyError):
                srv.submit(os.path.join(d, "missing", "renderJob.json"))
            rb = srv.submit(os.path.join(bad, "renderJob.json"), passes=1)
            ok = srv.submit(_path("cornell"), passes=1)
            got = _collect(srv, 2)
            assert got[rb]["status"] == -2 and "index" in got[rb]["error"]
            assert got[ok]["status"] == 0
            with pytest.raises(HastyError):
                srv.read_sums(rb)


def test_server_stop_with_work_in_flight():
    from hastyrenderer_gb300 import Server
    srv = Server(paths_in_flight=1 << 14, quantum_samples=1024)
    for n in NAMES * 3:
        srv.submit(_path(n), passes=64)
    srv.stop()   # returns; unfinished requests are dropped
