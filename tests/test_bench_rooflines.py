"""The rooflines bench.py reports (CPU only): per-class counters weighted by
each scene class's rays and vertices, the issue-rate peak from the SM clock,
and null figures where a class that did work has no capture."""
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
bench = pytest.importorskip("bench")


def _stage(by_class, launches=10, trace_ms=10.0, shade_ms=20.0):
    rays = sum(c["rays"] for c in by_class.values())
    shaded = sum(c["shaded"] for c in by_class.values())
    return {"trace_ms": trace_ms, "shade_ms": shade_ms, "trace_launches": launches, "path_ms": 0.0, "path_launches": 0,
            "rays": rays, "shaded": shaded, "paths": 0, "by_class": by_class}


def test_weighted_counters_and_issue_rate():
    by = {"mix:cornell": {"rays": 3_000_000, "shaded": 1_000_000, "paths": 0},
          "mix:field800": {"rays": 1_000_000, "shaded": 500_000, "paths": 0}}
    kernels, dom = bench.kernel_rooflines(_stage(by), 7000.0, "measured", 2000.0, None)
    k_trace = next(k for k in kernels if k["kernel"] == "k_trace")
    c, f = bench.COUNTERS["mix:cornell"]["k_trace"], bench.COUNTERS["mix:field800"]["k_trace"]
    inst = 3_000_000 * c["warp_inst_per_ray"] + 1_000_000 * f["warp_inst_per_ray"]
    peak = bench.SMS * bench.ISSUE_PER_SM_PER_CLOCK * 2000.0 * 1e-3
    assert k_trace["peak"] == pytest.approx(peak)
    assert k_trace["achieved"] == pytest.approx(inst / 10 / 1e-3 * 1e-9)   # per launch over 1 ms
    assert k_trace["frac"] == pytest.approx(k_trace["achieved"] / peak)
    traffic = (3_000_000 * c["dram_bytes_per_ray"] + 1_000_000 * f["dram_bytes_per_ray"]) / 10
    assert k_trace["traffic"] == pytest.approx(traffic)
    shade = next(k for k in kernels if k["kernel"] == "k_resolve+k_sample")
    assert shade["bytes_per_unit"] == bench.B_SHADE
    assert shade["frac"] == pytest.approx(bench.B_SHADE * 150_000 / 2e-3 * 1e-9 / 7000.0)
    assert 0 < shade["issue"]["frac"] < 1
    assert dom["kernel"] == "k_resolve+k_sample"   # 20 ms of shading against 10 ms of closest hits


def test_uncaptured_class_gives_null_figures():
    by = {"somewhere_else": {"rays": 1000, "shaded": 500, "paths": 0}}
    kernels, _ = bench.kernel_rooflines(_stage(by), 7000.0, "measured", None, None)
    k_trace = next(k for k in kernels if k["kernel"] == "k_trace")
    assert k_trace["frac"] is None and k_trace["traffic"] is None and "note" in k_trace
    shade = next(k for k in kernels if k["kernel"] == "k_resolve+k_sample")
    assert shade["traffic"] is None and "issue" not in shade
    assert shade["frac"] is not None    # the byte model needs no capture


def test_every_counter_class_is_complete():
    for cls, ks in bench.COUNTERS.items():
        assert set(ks["k_trace"]) == {"dram_bytes_per_ray", "warp_inst_per_ray", "thread_inst_per_ray"}, cls
        assert ks["k_trace"]["thread_inst_per_ray"] <= 32 * ks["k_trace"]["warp_inst_per_ray"], cls
        assert set(ks["k_resolve+k_sample"]) == {"dram_bytes_per_vertex", "warp_inst_per_vertex"}, cls
