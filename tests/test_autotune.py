"""The autotuner's staged search on the CPU, with a stand-in for the device
timing: each stage keeps the fastest candidate and carries it into the next
(lanes x paths per lane, then shading block shapes, then the closest-hit grid
cap; the regeneration engine's pool x threshold beside them), the result is
cached as JSON per version, and batch_args turns it into hasty_batch_render
keyword arguments."""
import json

import pytest

from hastyrenderer_gb300 import autotune


class FakeJob:
    def __init__(self):
        self.resets = 0

    def reset(self):
        self.resets += 1


def fake_cost(cand):
    """Samples/s of a candidate: best at 3 lanes of 8M paths, 128/512-thread
    shading, a cap of 6; the regeneration engine always slower."""
    if cand["mode"] == 1:
        return 10.0 + cand["regen_fraction"]
    s = 100.0 - 5 * abs(cand["lanes"] - 3) - 3 * abs(cand["paths_in_flight"].bit_length() - 24)
    s += 2.0 if cand.get("resolve_threads") == 128 else 0.0
    s += 1.0 if cand.get("sample_threads") == 512 else 0.0
    s += {4: 0.0, 5: 0.5, 6: 0.8}.get(cand.get("trace_blocks_per_sm"), 0.0)
    return s


@pytest.fixture
def fake_timing(monkeypatch):
    seen = []

    def _time(jobs, passes, cand, repeats):
        seen.append(dict(cand))
        return dict(cand, device_ms=1.0, samples_per_s=fake_cost(cand))
    monkeypatch.setattr(autotune, "_time", _time)
    return seen


def test_stages_keep_the_best_and_cache_it(tmp_path, fake_timing):
    jobs = [FakeJob(), FakeJob()]
    out = tmp_path / "tune.json"
    res = autotune.tune_batch(jobs, passes=2, out_path=str(out))
    assert res["mode"] == 0 and res["lanes"] == 3 and res["paths_in_flight"] == 1 << 23
    assert (res["resolve_threads"], res["sample_threads"], res["trace_blocks_per_sm"]) == (128, 512, 6)
    n_first = len(autotune.LANES) * len(autotune.LANE_PATHS)
    n_shapes = len(autotune.RESOLVE_THREADS) * len(autotune.SAMPLE_THREADS)
    n_regen = len(autotune.REGEN_POOLS) * len(autotune.REGEN)
    assert len(fake_timing) == n_first + n_shapes + len(autotune.TRACE_BLOCKS) + n_regen
    # later stages keep the earlier stages' choices
    for cand in fake_timing[n_first:n_first + n_shapes]:
        assert (cand["lanes"], cand["paths_in_flight"]) == (3, 1 << 23)
    assert all(j.resets >= 1 for j in jobs)
    cached = autotune.load(str(out))
    assert cached is not None and cached["lanes"] == 3 and cached["version"] == autotune.VERSION
    args = autotune.batch_args(cached)
    assert args == {"mode": 0, "paths_in_flight": 1 << 23, "lanes": 3, "resolve_threads": 128, "sample_threads": 512,
                    "trace_blocks_per_sm": 6}


def test_stale_or_broken_cache_is_ignored(tmp_path):
    p = tmp_path / "old.json"
    p.write_text(json.dumps({"version": autotune.VERSION - 1, "lanes": 2}))
    assert autotune.load(str(p)) is None
    p.write_text("{not json")
    assert autotune.load(str(p)) is None
    assert autotune.load(str(tmp_path / "missing.json")) is None


def test_regen_result_gives_regen_arguments():
    args = autotune.batch_args({"mode": 1, "paths_in_flight": 1 << 22, "regen_fraction": 0.9})
    assert args == {"mode": 1, "paths_in_flight": 1 << 22, "regen_fraction": 0.9}
