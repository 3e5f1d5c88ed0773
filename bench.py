"""Benchmarks of the GB300 path tracer. One JSON line per run (rank 0).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

Workloads (seeded synthetic scenes; no external dataset is involved):

* batch (default): 64 render jobs of the mixed distribution (procedural
  Cornell box or sphere field of 50/200/800 subdivision-3 icospheres with the
  2048x1024 FP32 sky; 128x128 .. 1024x768; 16..1024 spp log-uniform; depth
  8..16). One step renders every job's full pass count in one
  hasty_batch_render call (packed batches, parameters from the autotuner).
  `value` is camera samples per second of the batched steps (device time);
  `plain` is the same jobs one after another through
  hasty_job_render_passes (device and wall time), `batched_over_plain` the
  ratios. Every job's image is checked bit-identical between the two.
* plain: one large job, 800 icospheres + ground (1,024,002 triangles),
  1920x1080, thin lens with 6 aperture blades, sky, depth 12; one step = 8
  passes.
* cornell: the procedural Cornell box (34 triangles), 256x256, pinhole, 64
  spp, depth 8, roulette from depth 3; one step = the full 64-pass render.
* serve: Poisson arrivals (20 jobs/s for 120 s) of the mixed distribution
  through hasty_server_*; p50/p95/p99 latency beside throughput.
* stress: 10.36M triangles, 3840x2160, depth 32, one pass per step.
* photon: the photon mapper on a 640x480 textured room.

Inputs stay resident on the device in the timed region; the working sets
(path state of ~7 GB per render lane) are far larger than L2, so no flush is
needed (photon: flushed, its scene fits in L2). `e2e` is the same metric
through the C ABI with host data: scene files loaded (parse, BVH build,
host->device upload) and every image read back to the host inside the timed
region. `cpu_baseline` times the CPU oracle (oracle/, the reference
integrator restated) on this host's cores on a bounded sample of the same
workload; `--impl reference` times the same sample as its own line.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SPP_PER_STEP = 8
WORKLOAD_PLAIN = "sphere_field_800x_icosphere3_1024002tri_1920x1080_dof6_sky2048x1024_depth12"
WORKLOAD_CORNELL = "cornell_box_34tri_256x256_64spp_depth8_rr3"
WORKLOAD_BATCH = "mixed_64_jobs_cornell_or_field50_200_800_128x128_to_1024x768_spp16_1024_depth8_16"
# Algorithmic bytes per shaded vertex: path state read + write (2 x 96 B) and
# the triangle's attributes (92 B); texel reads are not counted.
B_SHADE = 2 * 96 + 92
# Per-unit hardware counters of the wavefront kernels, per scene class, from
# small ncu captures (every k_trace, k_resolve and k_sample launch of a
# one-step run: three batches of 2 passes, of 64 for the Cornell box workload,
# divided by the rays and vertices the process traced and shaded): DRAM
# bytes (dram__bytes_read.sum + dram__bytes_write.sum) per traced ray and
# per shaded vertex, and for the
# closest-hit kernel warp instructions and thread instructions per ray and
# the shading pair's warp instructions per vertex (smsp__inst_executed.sum,
# smsp__thread_inst_executed.sum). Classes: "plain"
# (the 1080p 800-sphere field), "cornell" (the 256x256 box), "mix:<kind>"
# (one job of each scene kind of the 64-job mix, rendered alone; a class
# without a capture gives null). They give each kernel's traffic and the closest-hit kernel's
# issue rate for the units a launch processed; a run covering several classes
# weights them by each class's rays and vertices.
COUNTERS = {
    "plain": {"k_trace": {"dram_bytes_per_ray": 128.67, "warp_inst_per_ray": 227.73, "thread_inst_per_ray": 4535.8},
              "k_resolve+k_sample": {"dram_bytes_per_vertex": 1038.97, "warp_inst_per_vertex": 183.84}},
    "cornell": {"k_trace": {"dram_bytes_per_ray": 80.77, "warp_inst_per_ray": 63.33, "thread_inst_per_ray": 982.99},
                "k_resolve+k_sample": {"dram_bytes_per_vertex": 863.61, "warp_inst_per_vertex": 147.53}},
    "mix:cornell": {"k_trace": {"dram_bytes_per_ray": 73.41, "warp_inst_per_ray": 60.67, "thread_inst_per_ray": 986.99},
                    "k_resolve+k_sample": {"dram_bytes_per_vertex": 819.35, "warp_inst_per_vertex": 146.09}},
    "mix:field50": {"k_trace": {"dram_bytes_per_ray": 78.50, "warp_inst_per_ray": 58.44, "thread_inst_per_ray": 1178.49},
                    "k_resolve+k_sample": {"dram_bytes_per_vertex": 871.84, "warp_inst_per_vertex": 181.70}},
    "mix:field200": {"k_trace": {"dram_bytes_per_ray": 89.84, "warp_inst_per_ray": 100.99,
                                 "thread_inst_per_ray": 1966.27},
                     "k_resolve+k_sample": {"dram_bytes_per_vertex": 916.45, "warp_inst_per_vertex": 189.78}},
    "mix:field800": {"k_trace": {"dram_bytes_per_ray": 134.29, "warp_inst_per_ray": 224.96,
                                 "thread_inst_per_ray": 4318.20},
                     "k_resolve+k_sample": {"dram_bytes_per_vertex": 1016.86, "warp_inst_per_vertex": 188.57}},
}
REF_PASSES_PER_STEP = 64     # reference arm: passes of the CPU sample per step (about 4 s on the mix)
ISSUE_PER_SM_PER_CLOCK = 4   # warp instructions per SM and clock (one per scheduler)
SMS = 152


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.idx = gpu_index
        self.rows = []
        self._stop = threading.Event()
        self._t = None

    def _run(self):
        while not self._stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.idx), f"--query-gpu={self.FIELDS}",
                                      "--format=csv,noheader,nounits"], capture_output=True, text=True, timeout=5)
                if out.returncode == 0:
                    self.rows.append([c.strip() for c in out.stdout.strip().split(",")])
            except Exception:
                pass
            self._stop.wait(0.2)

    def __enter__(self):
        self._t = threading.Thread(target=self._run, daemon=True)
        self._t.start()
        return self

    def __exit__(self, *a):
        self._stop.set()
        if self._t:
            self._t.join(timeout=6)

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = sorted(float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit())
        mx = max((float(r[2]) for r in self.rows if r[2].replace(".", "").isdigit()), default=None)
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            for k, name in enumerate(names):
                if len(r) > 5 + k and r[5 + k].lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": sm[len(sm) // 2] if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(self.rows)}


def make_plain_job(base: str, seed: int = 0) -> str:
    from hastyrenderer_gb300 import scenes
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.sphere_field(base, seed=seed, n_spheres=800, subdiv=3, width=1920, height=1080, spp=256, max_depth=12)
    return path


def make_cornell_job(base: str, seed: int = 0) -> str:
    from hastyrenderer_gb300 import scenes
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.cornell_box(base, seed=seed, width=256, height=256, spp=64, max_depth=8, roulette_start_depth=3)
    return path


def mix_jobs():
    from hastyrenderer_gb300 import workloads
    base = os.environ.get("HASTY_BENCH_MIX", os.path.join(tempfile.gettempdir(), "hasty_bench_mix"))
    return workloads.mixed_jobs(base, n_jobs=64, seed=0)


def scene_class(job: dict) -> str:
    """Scene kind of a mix job: cornell, field50, field200 or field800."""
    return f"{job['kind']}{job['spheres'] or ''}"


def replica_seed(rank: int) -> int:
    """Random streams of rank `rank`'s replica: every rank renders its own
    passes of the same job (weak scaling, no data-path exchange)."""
    return 1000 + rank


def max_over_ranks(value: float, dist, device: str) -> float:
    """The largest of the ranks' values (the job's time is its slowest
    rank's); `dist` None means one rank."""
    if dist is None:
        return value
    import torch
    t = torch.tensor([value], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ---------------------------------------------------------------------------
# CPU oracle on the host cores: bounded, representative samples of each
# workload (shared by cpu_baseline and the reference arm, so both time the
# same pixels).

def strided_rows(h: int, stride: int, phase: int = 0) -> list[int]:
    return list(range(phase % stride, h, stride))


class CpuSampler:
    """Times the CPU oracle on strided full-width rows (every `stride`-th row,
    denser where a frame has fewer than 4 rows per host thread) of one or more jobs,
    pass after pass, and estimates the workload's CPU samples/s.

    jobs: list of (job_path, weight) where weight is the job's share of the
    workload in camera samples; rows of every job are rendered for passes
    0, 1, 2, ... (one round = one pass of every job's row set) until the time
    budget is spent. The estimate is sum(weights) / sum(weight_j * t_j) with
    t_j the measured seconds per camera sample of job j."""

    def __init__(self, jobs, stride: int = 16, threads: int = 0):
        from oracle.oracle import Oracle
        self.threads = threads or (os.cpu_count() or 1)
        self.stride = stride
        self.items = []
        for path, weight in jobs:
            o = Oracle(path)
            info = o.info()
            # at least 4 rows per host thread, so every call keeps all threads busy
            st = max(1, min(stride, info["height"] // (4 * self.threads)))
            self.items.append({"oracle": o, "weight": weight, "w": info["width"], "h": info["height"],
                               "stride": st, "rows": strided_rows(info["height"], st), "time": 0.0, "samples": 0,
                               "rays": 0, "nodes": 0, "tris": 0, "shaded": 0})
        self.rounds = 0

    def run_round(self):
        for it in self.items:
            o = it["oracle"]
            t0 = time.perf_counter()
            r = o.render_rows(self.rounds, 1, it["rows"][0], it["stride"], len(it["rows"]), self.threads)
            st = r["stats"]
            it["rays"] += int(st[0]); it["nodes"] += int(st[2]); it["tris"] += int(st[3]); it["shaded"] += int(st[4])
            it["time"] += time.perf_counter() - t0
            it["samples"] += it["w"] * len(it["rows"])
        self.rounds += 1

    def run(self, budget_s: float, min_rounds: int = 1):
        t0 = time.perf_counter()
        while self.rounds < min_rounds or time.perf_counter() - t0 < budget_s:
            self.run_round()
        return time.perf_counter() - t0

    def estimate(self) -> float:
        wsum = sum(it["weight"] for it in self.items)
        tsum = sum(it["weight"] * it["time"] / max(it["samples"], 1) for it in self.items)
        return wsum / tsum

    def totals(self):
        s = sum(it["samples"] for it in self.items)
        t = sum(it["time"] for it in self.items)
        keys = ("rays", "nodes", "tris", "shaded")
        agg = {k: sum(it[k] for it in self.items) for k in keys}
        return s, t, agg

    def close(self):
        for it in self.items:
            it["oracle"].close()


def cpu_jobs(workload: str):
    """(job_path, weight) pairs of the CPU sample of a workload, with the
    sample's description. For the mixed batch: two jobs of each scene class
    (Cornell box; fields of 50, 200 and 800 icospheres), the first two of the
    mix in job order, each class weighted by its share of the mix's camera
    samples (split evenly over its two jobs)."""
    if workload == "plain":
        return [(make_plain_job(_bench_dir("hasty_bench_c1")), 1.0)], "whole 1920x1080 frame, every 16th row", 16
    if workload == "cornell":
        return [(make_cornell_job(_bench_dir("hasty_bench_c0")), 1.0)], "every row of the 256x256 frame", 1
    jobs = mix_jobs()
    from hastyrenderer_gb300 import workloads
    classes = {}
    for j in jobs:
        classes.setdefault((j["kind"], j["spheres"]), []).append(j)
    out = []
    desc = []
    for key, members in sorted(classes.items()):
        share = sum(workloads.job_samples(j) for j in members)
        picked = members[:2]
        for j in picked:
            out.append((j["path"], share / len(picked)))
        desc.append(f"{key[0]}{key[1] or ''}: jobs {[jobs.index(j) for j in picked]}")
    return out, "every 8th row of " + "; ".join(desc) + ", weighted by class share of the mix's samples", 8


def _bench_dir(name: str) -> str:
    d = os.environ.get("HASTY_BENCH_DIR_" + name.upper(), os.path.join(tempfile.gettempdir(), name))
    os.makedirs(d, exist_ok=True)
    return d


def cpu_baseline(workload: str, budget_s: float):
    jobs, desc, stride = cpu_jobs(workload)
    smp = CpuSampler(jobs, stride=stride)
    dt = smp.run(budget_s)
    v = smp.estimate()
    s, t, agg = smp.totals()
    smp.close()
    line = {"value": v, "unit": "samples/s", "cores": smp.threads, "kind": "port",
            "sample": f"{desc}; {smp.rounds} passes, {s} camera samples, {dt:.1f} s"}
    costs = {"nodes_per_ray": agg["nodes"] / max(agg["rays"], 1), "tris_per_ray": agg["tris"] / max(agg["rays"], 1),
             "rays_per_sample": agg["rays"] / max(s, 1), "shaded_per_sample": agg["shaded"] / max(s, 1)}
    return line, costs


def run_reference_arm(args, rank: int):
    """The reference integrator's CPU path (the oracle, its restatement) on
    this host's cores: the same strided sample as cpu_baseline, one pass of
    every sampled row per step, all host threads. Rank 0 only."""
    if rank != 0:
        return
    workload = args.workload if args.workload in ("plain", "cornell") else "batch"
    jobs, desc, stride = cpu_jobs(workload)
    smp = CpuSampler(jobs, stride=stride)
    for _ in range(args.warmup):
        smp.run_round()
    for it in smp.items:
        it.update(time=0.0, samples=0)
    t0 = time.perf_counter()
    for _ in range(args.steps * REF_PASSES_PER_STEP):
        smp.run_round()
    dt = time.perf_counter() - t0
    v = smp.estimate()
    s, _, _ = smp.totals()
    smp.close()
    wl = {"plain": WORKLOAD_PLAIN, "cornell": WORKLOAD_CORNELL}.get(workload, WORKLOAD_BATCH)
    line = {"impl": "reference", "metric": "samples/s", "value": v, "unit": "samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / max(args.steps, 1) * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded procedural scenes)",
            "config": {"workload": wl, "step": f"{REF_PASSES_PER_STEP} passes of the sampled rows ({desc}) on "
                                               f"{smp.threads} host threads"},
            "cpu_baseline": {"value": v, "unit": "samples/s", "cores": smp.threads, "kind": "port",
                             "sample": f"{desc}; {args.steps * REF_PASSES_PER_STEP} timed passes, {s} camera samples, "
                                       f"{dt:.1f} s"},
            "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# Rooflines of the wavefront kernels from a stage-timed run (one render lane,
# so each kernel's time is its own).

def _weighted(by_class: dict, kernel: str, field: str, unit: str):
    """Sum over scene classes of COUNTERS[class][kernel][field] times the
    class's units; None when a class that did work has no capture."""
    total = 0.0
    for cls, u in by_class.items():
        if not u.get(unit):
            continue
        v = COUNTERS.get(cls, {}).get(kernel, {}).get(field)
        if v is None:
            return None
        total += v * u[unit]
    return total


def kernel_rooflines(stage: dict, hbm: float, peak_kind: str, sm_mhz, costs):
    """stage: trace_ms, shade_ms, trace_launches, path_ms, path_launches,
    rays, shaded, paths and by_class (rays, shaded, paths per scene class) of
    a stage-timed run (wavefront jobs, path-kernel jobs or both). Returns
    (kernels, dominant)."""
    kernels = []
    mhz = sm_mhz or 2070.0
    issue_peak = SMS * ISSUE_PER_SM_PER_CLOCK * mhz * 1e-3
    issue_kind = f"{SMS} SMs x {ISSUE_PER_SM_PER_CLOCK} schedulers x {mhz:.0f} MHz (median under load)"
    by_class = stage["by_class"]
    classes = sorted(by_class)
    if stage["path_launches"]:
        n = stage["path_launches"]
        ms = stage["path_ms"] / n
        k = {"kernel": "k_paths", "unit_of_work": "camera sample", "units_per_launch": stage["paths"] / n,
             "ms_per_launch": ms, "bound": "issue", "unit": "G warp-inst/s"}
        dram = _weighted(by_class, "k_paths", "dram_bytes_per_sample", "paths")
        inst = _weighted(by_class, "k_paths", "warp_inst_per_sample", "paths")
        k["traffic"] = dram / n if dram is not None else None
        if inst is not None:
            ach = inst / n / (ms * 1e-3) * 1e-9
            k.update(achieved=ach, peak=issue_peak, frac=ach / issue_peak, peak_kind=issue_kind)
        else:
            k.update(achieved=None, peak=None, frac=None, note="instruction counts not captured for these scenes")
        kernels.append(k)
    if not stage["trace_launches"]:
        dominant = dict(max(kernels, key=lambda k: k["ms_per_launch"] * 1.0))
        dominant["note"] = "dominant kernel by device time, timed alone (stage timing keeps one render lane)"
        return kernels, dominant
    n = max(stage["trace_launches"], 1)
    rays_l = stage["rays"] / n
    trace_ms = stage["trace_ms"] / n
    k_trace = {"kernel": "k_trace", "unit_of_work": "traced ray", "units_per_launch": rays_l,
               "ms_per_launch": trace_ms, "scene_classes": classes}
    dram = _weighted(by_class, "k_trace", "dram_bytes_per_ray", "rays")
    k_trace["traffic"] = dram / n if dram is not None else None
    inst = _weighted(by_class, "k_trace", "warp_inst_per_ray", "rays")
    tinst = _weighted(by_class, "k_trace", "thread_inst_per_ray", "rays")
    if inst is not None:
        achieved = inst / n / (trace_ms * 1e-3) * 1e-9
        k_trace.update(bound="issue", achieved=achieved, peak=issue_peak, unit="G warp-inst/s",
                       frac=achieved / issue_peak, peak_kind=issue_kind,
                       warp_inst_per_ray=inst / max(stage["rays"], 1),
                       active_lanes_per_inst=tinst / inst if tinst else None)
    else:
        k_trace.update(bound="issue", achieved=None, peak=None, unit="G warp-inst/s", frac=None,
                       note="instruction counts not captured for these scenes")
    if costs:
        model = 32 + 16 + 64 * costs["nodes_per_ray"] + 48 * costs["tris_per_ray"]
        k_trace["hbm_model"] = {"bytes_per_ray": model, "note": "ray + hit + 64 B per binary-BVH node visit and 48 B per "
                                "triangle test counted by the CPU oracle: an upper bound on traffic, not a bound "
                                "on this kernel (its upper tree levels stay in L1/L2)",
                                "gbs": model * rays_l / (trace_ms * 1e-3) * 1e-9}
    verts_l = stage["shaded"] / n
    shade_ms = stage["shade_ms"] / n
    alg = B_SHADE * verts_l
    ach = alg / (shade_ms * 1e-3) * 1e-9
    dram = _weighted(by_class, "k_resolve+k_sample", "dram_bytes_per_vertex", "shaded")
    k_shade = {"kernel": "k_resolve+k_sample", "unit_of_work": "shaded vertex", "units_per_launch": verts_l,
               "ms_per_launch": shade_ms, "bound": "hbm", "achieved": ach, "peak": hbm, "unit": "GB/s",
               "frac": ach / hbm, "peak_kind": peak_kind, "bytes_per_unit": B_SHADE,
               "algorithmic_bytes_per_launch": alg, "traffic": dram / n if dram is not None else None}
    # the same launches against the issue rate (the pair is latency-bound: neither bound is reached)
    inst = _weighted(by_class, "k_resolve+k_sample", "warp_inst_per_vertex", "shaded")
    if inst is not None:
        ach_i = inst / n / (shade_ms * 1e-3) * 1e-9
        k_shade["issue"] = {"achieved": ach_i, "peak": issue_peak, "unit": "G warp-inst/s", "frac": ach_i / issue_peak,
                            "warp_inst_per_vertex": inst / max(stage["shaded"], 1), "peak_kind": issue_kind}
    kernels += [k_trace, k_shade]
    # dominant by total device time of the run
    totals = {"k_paths": stage["path_ms"], "k_trace": stage["trace_ms"], "k_resolve+k_sample": stage["shade_ms"]}
    dominant = dict(max(kernels, key=lambda k: totals[k["kernel"]]))
    dominant["note"] = "dominant kernel by device time, timed alone (stage timing keeps one render lane)"
    return kernels, dominant


def stage_split(job_list, passes_list, classes):
    """Renders the jobs one after another with stage timing and returns the
    summed stage times and work for the rooflines: rays and shaded vertices
    of the wavefront jobs, camera samples of the path-kernel jobs, in total
    and per scene class (classes[i] names job i's)."""
    out = {"trace_ms": 0.0, "shade_ms": 0.0, "trace_launches": 0, "rays": 0, "shaded": 0, "kernel_ms": 0.0,
           "path_ms": 0.0, "path_launches": 0, "paths": 0, "by_class": {}}
    for job, p, cls in zip(job_list, passes_list, classes):
        path_kernel = job.info.path_kernel
        job.set_stage_timing(True)
        s0 = job.stats()
        job.render_passes(p, sync=True)
        s1 = job.stats()
        job.set_stage_timing(False)
        for k in ("trace_ms", "shade_ms", "trace_launches", "kernel_ms", "path_ms", "path_launches"):
            out[k] += s1[k] - s0[k]
        c = out["by_class"].setdefault(cls, {"rays": 0, "shaded": 0, "paths": 0})
        if path_kernel:
            for k in ("paths",):
                out[k] += s1[k] - s0[k]
                c[k] += s1[k] - s0[k]
        else:
            for k in ("rays", "shaded"):
                out[k] += s1[k] - s0[k]
                c[k] += s1[k] - s0[k]
    return out


def tuned_batch_args(args, jobs, ctx):
    """Batching parameters from the autotuner (cached per GPU name), tuned on
    16 jobs spread over the mix, 8 passes each."""
    import torch
    from hastyrenderer_gb300 import RenderJob, autotune
    if args.no_tune:
        return {"mode": 0, "lanes": 2, "paths_in_flight": 1 << 24}, {"source": "defaults"}
    path = autotune.default_path(torch.cuda.get_device_name())
    res = autotune.load(path)
    if res:
        res["source"] = path
    else:
        calib = [RenderJob(j["path"], ctx) for j in jobs[::4]]
        res = autotune.tune_batch(calib, passes=8, out_path=path)
        for c in calib:
            c.close()
        res["source"] = "tuned now"
    info = {k: res[k] for k in autotune.KNOBS + ("samples_per_s", "source") if k in res}
    info["candidates"] = len(res.get("trials", []))
    return autotune.batch_args(res), info


# ---------------------------------------------------------------------------

def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (default: 3 batch, 16 plain/cornell)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="batch", choices=["batch", "plain", "cornell", "serve", "stress", "photon"])
    ap.add_argument("--spp-per-step", type=int, default=SPP_PER_STEP, help="plain: passes per step")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--bvh", default="wide", choices=["wide", "binary"])
    ap.add_argument("--rate", type=float, default=20.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=120.0, help="serve: seconds of arrivals")
    ap.add_argument("--policy", type=int, default=0, help="serve: 0 round robin, 1 shortest remaining first")
    ap.add_argument("--no-tune", action="store_true", help="batch/serve: skip the autotuner (defaults)")
    ap.add_argument("--serve-stress", action="store_true", help="stress: also serve the job through hasty_server_*")
    ap.add_argument("--jobs", type=int, default=64, help="batch: the first N jobs of the 64-job mix (profiling)")
    ap.add_argument("--mix-job", type=int, default=-1, help="plain: render job K of the 64-job mix instead (profiling)")
    ap.add_argument("--lane-paths", type=int, default=0,
                    help="batch/serve: path slots per render lane instead of the tuned value (profiling small batches)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 3 if args.workload == "batch" else 16
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        dist = None
        if world > 1:
            import torch.distributed as dist
            dist.init_process_group("gloo")     # the reference arm runs on the host cores only
        run_reference_arm(args, rank)
        if dist is not None:
            dist.destroy_process_group()
        return
    if args.workload == "stress":
        return run_stress(args)
    if args.workload == "photon":
        return run_photon(args)
    if args.workload == "serve":
        return run_serve(args)
    if args.workload == "batch":
        return run_batch(args)
    return run_single(args)


def _dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if world <= 1:
        return None, 0, 1, local_rank
    import torch
    import torch.distributed as dist
    torch.cuda.set_device(local_rank)
    dist.init_process_group("nccl")
    return dist, dist.get_rank(), world, local_rank


def run_single(args):
    """plain (the 1080p sphere field, SPP_PER_STEP passes per step) or
    cornell (the 256x256 box, the whole 64-pass render per step): replicas on
    every rank (weak scaling)."""
    import torch
    from hastyrenderer_gb300 import Context, RenderJob
    dist, rank, world, local_rank = _dist_setup(args)
    if args.workload == "plain" and args.mix_job >= 0:
        mj = mix_jobs()[args.mix_job] if rank == 0 else None
        wl, passes, cls = f"mix_job_{args.mix_job}", args.spp_per_step, None
    elif args.workload == "plain":
        job_path = make_plain_job(_bench_dir("hasty_bench_c1")) if rank == 0 else None
        wl, passes, cls = WORKLOAD_PLAIN, args.spp_per_step, "plain"
    else:
        job_path = make_cornell_job(_bench_dir("hasty_bench_c0")) if rank == 0 else None
        wl, passes, cls = WORKLOAD_CORNELL, 64, "cornell"
    if dist is not None:
        dist.barrier()
    if args.workload == "plain" and args.mix_job >= 0:
        mj = mix_jobs()[args.mix_job]
        job_path, cls = mj["path"], "mix:" + scene_class(mj)
    else:
        job_path = os.path.join(_bench_dir("hasty_bench_c1" if args.workload == "plain" else "hasty_bench_c0"),
                                "renderJob.json")
    torch.cuda.init()
    ctx = Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0)

    # end to end through the C ABI: load (parse, BVH, upload) + steps, each
    # step's colour estimate read back to the host while the next renders
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    job = RenderJob(job_path, ctx)
    info = job.info
    load_ms = (time.perf_counter() - t0) * 1e3
    W, H = info.width, info.height
    for k in range(args.steps):
        job.render_passes(passes)
        if k:
            job.snapshot_get()
        job.snapshot()
    est, n_est = job.snapshot_get()
    e2e_s = time.perf_counter() - t0
    assert n_est == args.steps * passes
    del est
    job.sync()
    # every ray and vertex this process shades (for per-unit ncu counters,
    # which cover all launches of the process)
    work = {k: job.stats()[k] for k in ("rays", "shaded", "paths")}

    # device-resident timing (both render lanes, as a user's render runs)
    job.reset()
    job.set_seed(replica_seed(rank))
    for _ in range(args.warmup):
        job.render_passes(passes)
    job.sync()
    s0 = job.stats()
    sampler = ClockSampler(local_rank)
    with sampler:
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            job.render_passes(passes)
        job.sync()
        torch.cuda.synchronize()
        wall = time.perf_counter() - w0
        if dist is not None:
            dist.barrier()
    s1 = job.stats()
    s2 = job.stats()
    stage = stage_split([job] * args.steps, [passes] * args.steps, [cls] * args.steps)
    for k in work:
        work[k] += s2[k] + stage[k]
    t = max_over_ranks(max((s1["kernel_ms"] - s0["kernel_ms"]) * 1e-3, 1e-9), dist, "cuda")
    samples = args.steps * passes * W * H
    clocks = sampler.summary()
    if rank == 0:
        hbm, peak_kind = peaks()
        cpu, costs = (None, None)
        if not args.no_cpu_baseline:
            cpu, costs = cpu_baseline(args.workload, args.cpu_budget)
        kernels, roof = kernel_rooflines(stage, hbm, peak_kind, clocks.get("sm_mhz"), costs)
        line = {
            "metric": "samples/s", "value": samples * world / t, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": wl, "passes_per_step": passes, "width": W, "height": H, "bvh": args.bvh,
                       "max_depth": info.max_depth, "triangles": info.n_triangles,
                       "l2": "working set > L2 (path state + scene), no flush", "parallelism": f"replicas x{world}"},
            "mrays_per_s": (s1["rays"] - s0["rays"]) * world / t * 1e-6,
            "stage_ms_per_step": {"trace": stage["trace_ms"] / args.steps, "shade": stage["shade_ms"] / args.steps,
                                  "path_kernel": stage["path_ms"] / args.steps,
                                  "one_lane_total": stage["kernel_ms"] / args.steps,
                                  "note": "same steps with stage timing (one render lane); the timed run uses two"},
            "wall_ms_per_step": wall / args.steps * 1e3,
            "gpu_launches": s1["kernel_launches"] - s0["kernel_launches"],
            "roofline": roof, "kernels": kernels, "cpu_baseline": cpu,
            "work_in_process": work,
            "e2e": {"value": samples * world / e2e_s, "unit": "samples/s",
                    "h2d_bytes_per_step": int(info.device_bytes // args.steps), "d2h_bytes_per_step": W * H * 3 * 4,
                    "includes": "job load (parse, BVH build, upload) + steps + a colour read-back per step",
                    "load_ms": {"total": load_ms, "parse": info.parse_ms, "bvh_build": info.bvh_build_ms,
                                "upload": info.upload_ms}},
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    job.close()
    if dist is not None:
        dist.destroy_process_group()


def run_batch(args):
    """The 64-job mix: batched (packed batches) against the same jobs one by
    one through the single-job path, with bit-identical images."""
    import numpy as np
    import torch
    from hastyrenderer_gb300 import Context, batch_render, load_jobs, workloads
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return
    torch.cuda.init()
    t_gen = time.perf_counter()
    jobs = mix_jobs()[: max(1, args.jobs)]
    gen_s = time.perf_counter() - t_gen
    ctx = Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0)
    spp = [j["spp"] for j in jobs]
    total = sum(workloads.job_samples(j) for j in jobs)
    hbm, peak_kind = peaks()

    # end to end through the C ABI: load every job (parse, BVH build, upload),
    # one batched render, every job's colour estimate read to the host
    t0 = time.perf_counter()
    resident = load_jobs([j["path"] for j in jobs], ctx)   # parse, BVH build, upload on all host threads
    load_s = time.perf_counter() - t0
    eargs, tune = tuned_batch_args(args, jobs, ctx)   # (tuning is not part of the end-to-end time)
    if args.lane_paths:
        eargs = dict(eargs, mode=0, lanes=eargs.get("lanes", 2), paths_in_flight=args.lane_paths)
    for r in resident:
        r.reset()
    t1 = time.perf_counter()
    batch_render(resident, spp, **eargs)
    images = [r.compute_estimate() for r in resident]
    e2e_s = load_s + (time.perf_counter() - t1)
    h2d = sum(r.info.device_bytes for r in resident)
    d2h = sum(im.nbytes for im in images)
    del images

    # plain: one job after another (device time from each job's own events)
    plain_sums, per_class = [], {}
    plain_ms, plain_rays = 0.0, 0
    for r in resident:
        r.reset()
    sampler = ClockSampler(local_rank)
    with sampler:
        w0 = time.perf_counter()
        for j, r, p in zip(jobs, resident, spp):
            s0 = r.stats()
            r.render_passes(p, sync=True)
            s1 = r.stats()
            ms = s1["kernel_ms"] - s0["kernel_ms"]
            plain_ms += ms
            plain_rays += s1["rays"] - s0["rays"]
            key = scene_class(j)
            c = per_class.setdefault(key, {"samples": 0, "plain_ms": 0.0})
            c["samples"] += workloads.job_samples(j)
            c["plain_ms"] += ms
            plain_sums.append(r.read_sums()[0])
            r.release_paths()
        plain_wall = time.perf_counter() - w0
        # batched: warm-up steps, then the timed steps
        for _ in range(args.warmup):
            for r in resident:
                r.reset()
            batch_render(resident, spp, **eargs)
        torch.cuda.synchronize()
        dev_ms, wall_ms, rays, launches, batches = 0.0, 0.0, 0, 0, 0
        identical = True
        for _ in range(args.steps):
            for r in resident:
                r.reset()
            torch.cuda.synchronize()
            w1 = time.perf_counter()
            st = batch_render(resident, spp, **eargs)
            torch.cuda.synchronize()
            wall_ms += (time.perf_counter() - w1) * 1e3
            dev_ms += st["device_ms"]
            rays += st["rays"]
            launches += st["kernel_launches"]
            batches += st["iterations"]
            identical = identical and all(np.array_equal(r.read_sums()[0], ps) for r, ps in zip(resident, plain_sums))
    clocks = sampler.summary()
    # stage split on 1/8 of every job's passes (one render lane, for the rooflines)
    for r in resident:
        r.reset()
    stage = stage_split(resident, [max(1, p // 8) for p in spp], ["mix:" + scene_class(j) for j in jobs])
    for r in resident:
        r.release_paths()
        r.close()
    cpu, costs = (None, None)
    if not args.no_cpu_baseline:
        cpu, costs = cpu_baseline("batch", args.cpu_budget)
    kernels, roof = kernel_rooflines(stage, hbm, peak_kind, clocks.get("sm_mhz"), costs)
    batch_sps = total * args.steps / (dev_ms * 1e-3)
    plain_sps = total / (plain_ms * 1e-3)
    for c in per_class.values():
        c["plain_samples_per_s"] = c["samples"] / (c["plain_ms"] * 1e-3)
    line = {
        "metric": "samples/s", "value": batch_sps, "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": dev_ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
        "config": {"workload": WORKLOAD_BATCH if len(jobs) == 64 else f"first_{len(jobs)}_jobs_of_the_mix",
                   "jobs": len(jobs), "samples_per_step": total,
                   "step": "every job's full pass count in one hasty_batch_render call",
                   "batching": eargs, "l2": "working set > L2 (path state + scenes), no flush",
                   "parallelism": "one GPU"},
        "mrays_per_s": rays / (dev_ms * 1e-3) * 1e-6,
        "wall_ms_per_step": wall_ms / args.steps,
        "plain": {"value": plain_sps, "unit": "samples/s", "device_ms": plain_ms, "wall_ms": plain_wall * 1e3,
                  "mrays_per_s": plain_rays / (plain_ms * 1e-3) * 1e-6, "per_class": per_class,
                  "note": "the same jobs one after another through hasty_job_render_passes"},
        "batched_over_plain": {"device": plain_ms / (dev_ms / args.steps),
                               "wall": plain_wall * 1e3 / (wall_ms / args.steps)},
        "images_bit_identical_to_plain": identical,
        "batches_per_step": batches / args.steps,
        "gpu_launches": launches,
        "roofline": roof, "kernels": kernels,
        "stage_ms_per_step": {"trace": stage["trace_ms"] * 8, "shade": stage["shade_ms"] * 8,
                              "path_kernel": stage["path_ms"] * 8,
                              "note": "1/8 of every job's passes with stage timing (one render lane), scaled by 8"},
        "cpu_baseline": cpu,
        "e2e": {"value": total / e2e_s, "unit": "samples/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "includes": "loading all the jobs (hasty_jobs_load on all host threads: parse, BVH build, upload) + "
                            "one batched render + every colour estimate read to the host", "load_s": load_s,
                "scene_generation_s": gen_s},
        "autotune": tune, "clocks": clocks, "peak_hbm_gbs": hbm, "peak_kind": peak_kind,
    }
    print(json.dumps(line), flush=True)


def run_serve(args):
    """Serving: Poisson arrivals of the mixed distribution over a warm pool of
    32 scenes, through hasty_server_* (packed batches on the tuned lanes)."""
    import numpy as np
    import torch
    from hastyrenderer_gb300 import Context, Server, workloads
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return
    torch.cuda.init()
    jobs = mix_jobs()
    ctx = Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0)
    eargs, tune = tuned_batch_args(args, jobs, ctx)
    lanes = eargs.get("lanes", 2)
    paths = eargs.get("paths_in_flight", 1 << 24) if eargs.get("mode", 0) == 0 else 1 << 24
    shapes = {k: eargs[k] for k in ("resolve_threads", "sample_threads", "trace_blocks_per_sm") if k in eargs}
    pool = jobs[: max(1, len(jobs) // 2)]
    base = os.path.dirname(os.path.dirname(pool[0]["path"]))
    reqs = workloads.poisson_requests(pool, os.path.join(base, f"requests_{args.rate:g}_{args.duration:g}"),
                                      rate=args.rate, duration=args.duration, seed=1)
    cfg = dict(memory_budget=120 << 30, max_resident_jobs=32, max_resident_scenes=32, lanes=lanes,
               paths_in_flight=paths, policy=args.policy, **shapes)
    srv = Server(ctx, **cfg)
    t0 = time.perf_counter()
    for j in pool:                       # warm the scene cache: one cheap request per scene
        srv.submit(j["path"], passes=1)
    srv.wait_idle(-1)
    for r in srv.poll(max_results=len(pool) + 8, wait_ms=0):
        srv.release(r["id"])
    warm_s = time.perf_counter() - t0
    st0 = srv.stats()
    results = []
    sampler = ClockSampler(local_rank)
    with sampler:
        t0 = time.perf_counter()
        k = 0
        while k < len(reqs) or len(results) < len(reqs):
            now = time.perf_counter() - t0
            while k < len(reqs) and reqs[k]["t"] <= now:
                srv.submit(reqs[k]["path"], passes=reqs[k]["spp"], seed=reqs[k]["seed"])
                k += 1
            wait = 0 if k >= len(reqs) else max(0, int((reqs[k]["t"] - (time.perf_counter() - t0)) * 1e3))
            for r in srv.poll(wait_ms=max(1, min(wait, 50)) if k < len(reqs) else 200):
                if r["status"] == 0:
                    img = srv.read(r["id"])   # host result as a caller reads it
                    del img
                srv.release(r["id"])
                results.append(r)
        span = time.perf_counter() - t0
    st1 = srv.stats()
    srv.stop()
    ok = [r for r in results if r["status"] == 0]
    lat = np.array([r["latency_ms"] for r in ok]) if ok else np.zeros(1)
    samples = sum(r["samples"] for r in ok)
    dev_ms = st1["device_ms"] - st0["device_ms"]
    offered = sum(r["width"] * r["height"] * r["spp"] for r in reqs) / args.duration
    line = {
        "metric": "samples/s", "value": samples / span, "unit": "samples/s", "n_gpus": 1, "steps": len(reqs),
        "warmup": len(pool), "ms_per_step": span * 1e3 / max(len(reqs), 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
        "config": {"workload": f"serving_poisson_{args.rate:g}_per_s_{args.duration:g}_s", "requests": len(reqs),
                   "scene_pool": len(pool), "server": cfg},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                       "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
        "completed": len(ok), "failed": len(results) - len(ok),
        "device_samples_per_s": samples / max(dev_ms * 1e-3, 1e-9),
        "mrays_per_s": (st1["rays"] - st0["rays"]) / max(dev_ms * 1e-3, 1e-9) * 1e-6,
        "offered_samples_per_s": offered, "offered_over_served": offered / max(samples / span, 1e-9),
        "batches": st1["batches"] - st0["batches"], "gpu_launches": st1["kernel_launches"] - st0["kernel_launches"],
        "peak_resident_bytes": st1["peak_resident_bytes"], "warm_s": warm_s, "span_s": span,
        "autotune": tune, "clocks": sampler.summary(),
    }
    print(json.dumps(line), flush=True)


PHOTON_WORKLOAD = "photon_mapping_textured_room_640x480_tex256_depth8_caustics_map"


def run_photon(args):
    """The photon mapper (hasty_pm_render) on the textured room (area light,
    smooth glass sphere, glossy and anisotropic metal, texture maps) at
    640x480, depth 8: one stochastic progressive iteration per step (photon
    tracing until 0.5*W*H caustic photons are stored, photon-map build, gather
    of every pixel). value = pixels gathered per second by the wall clock (the
    host part of an iteration is real work); the CPU baseline is the oracle's
    photon mapper (one thread, as one reference render thread) on the same
    scene at 160x120."""
    import numpy as np
    import torch
    from hastyrenderer_gb300 import Context, RenderJob, scenes
    torch.cuda.init()
    base = os.environ.get("HASTY_BENCH_PHOTON", os.path.join(tempfile.gettempdir(), "hasty_bench_photon"))
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.textured_room(base, seed=5, width=640, height=480, spp=64, max_depth=8, tex_size=256)
    job = RenderJob(path, Context(0))
    info = job.info
    W, H = info.width, info.height
    for _ in range(args.warmup):
        job.pm_render(1)
    s0 = job.pm_stats()
    # the scene and the photon map fit in L2: a 256 MB write between
    # iterations evicts them, so every iteration starts from cold caches
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")
    flush.zero_()                       # the first launch of torch's kernel loads its module
    torch.cuda.synchronize()
    sampler = ClockSampler(0)
    with sampler:
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            job.pm_render(1)
            flush.zero_()
            torch.cuda.synchronize()
        wall = time.perf_counter() - t0
    s1 = job.pm_stats()
    est = job.pm_read(0)
    dev_ms = s1["device_ms"] - s0["device_ms"]
    host_ms = s1["host_ms"] - s0["host_ms"]
    cpu = None
    if not args.no_cpu_baseline:
        from oracle.oracle import PhotonMapper
        small = os.path.join(base + "_small", "renderJob.json")
        if not os.path.exists(small):
            scenes.textured_room(os.path.dirname(small), seed=5, width=160, height=120, spp=64, max_depth=8, tex_size=256)
        pm = PhotonMapper(small)
        pm.iterate(1)
        t0 = time.perf_counter()
        k = 0
        while time.perf_counter() - t0 < min(args.cpu_budget, 10.0) or k == 0:
            pm.iterate(1)
            k += 1
        dt = time.perf_counter() - t0
        pm.close()
        cpu = {"value": k * 160 * 120 / dt, "unit": "pixels/s", "cores": 1, "kind": "port",
               "sample": f"{k} iterations of the same scene at 160x120 after one warm-up iteration, {dt:.1f} s"}
    line = {
        "metric": "pixels/s", "value": args.steps * W * H / wall, "unit": "pixels/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": wall / args.steps * 1e3, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": PHOTON_WORKLOAD, "width": W, "height": H, "max_depth": info.max_depth,
                   "triangles": info.n_triangles, "step": "one progressive photon-mapping iteration",
                   "l2": "working set < L2 (small scene); L2 flushed between iterations (256 MB write, inside the timed region)"},
        "device_ms_per_step": dev_ms / args.steps, "host_ms_per_step": host_ms / args.steps,
        "photon_ms_per_step": (s1["photon_ms"] - s0["photon_ms"]) / args.steps,
        "gather_ms_per_step": (s1["gather_ms"] - s0["gather_ms"]) / args.steps,
        "cell_size_host_ms_per_step": (s1["cell_ms"] - s0["cell_ms"]) / args.steps,
        "map_build_ms_per_step": (s1["map_ms"] - s0["map_ms"]) / args.steps,
        "photons_emitted_per_step": s1["photons_emitted"], "photons_stored_per_step": s1["photons_stored"],
        "photons_traced_per_s": s1["photons_emitted"] * args.steps / wall,
        "estimate_finite": bool(np.isfinite(est).all()), "media_overflow": s1["media_overflow"],
        "cpu_baseline": cpu, "clocks": sampler.summary(),
    }
    print(json.dumps(line), flush=True)
    job.close()


STRESS_WORKLOAD = "stress_8000x_icosphere3_10000_cuboids_10360016tri_3840x2160_rgba8tex4096_cauchy_depth32"


def run_stress(args):
    """The stress scene through the plain drop-in: one pass (8.29M camera
    samples) per step, FP64 cross-pass accumulation, device-timed."""
    import numpy as np
    import torch
    from hastyrenderer_gb300 import Context, RenderJob, scenes
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if int(os.environ.get("RANK", "0")) != 0:
        return
    torch.cuda.init()
    base = os.environ.get("HASTY_BENCH_STRESS", os.path.join(tempfile.gettempdir(), "hasty_bench_stress"))
    path = os.path.join(base, "renderJob.json")
    t0 = time.perf_counter()
    if not os.path.exists(path):
        scenes.stress_scene(base, seed=4)
    gen_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    job = RenderJob(path, Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0))
    load_s = time.perf_counter() - t0
    info = job.info
    for _ in range(args.warmup):
        job.render_passes(1)
    job.sync()
    s0 = job.stats()
    sampler = ClockSampler(local_rank)
    with sampler:
        w0 = time.perf_counter()
        for _ in range(args.steps):
            job.render_passes(1)
        job.sync()
        wall = time.perf_counter() - w0
    s1 = job.stats()
    ms = s1["kernel_ms"] - s0["kernel_ms"]
    # stage split: the same steps with stage timing (one render lane)
    job.set_stage_timing(True)
    job.sync()
    t0s = job.stats()
    for _ in range(args.steps):
        job.render_passes(1)
    job.sync()
    t1s = job.stats()
    job.set_stage_timing(False)
    samples = args.steps * info.width * info.height
    est = job.compute_estimate()
    line = {
        "metric": "samples/s", "value": samples / (ms * 1e-3), "unit": "samples/s", "n_gpus": 1, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
        "config": {"workload": STRESS_WORKLOAD, "width": info.width, "height": info.height, "max_depth": info.max_depth,
                   "triangles": info.n_triangles, "bvh": args.bvh, "accumulation": "fp64 across passes",
                   "l2": "working set > L2, no flush"},
        "mrays_per_s": (s1["rays"] - s0["rays"]) / (ms * 1e-3) * 1e-6,
        "stage_ms_per_step": {"trace": (t1s["trace_ms"] - t0s["trace_ms"]) / args.steps,
                              "shade": (t1s["shade_ms"] - t0s["shade_ms"]) / args.steps,
                              "one_lane_total": (t1s["kernel_ms"] - t0s["kernel_ms"]) / args.steps,
                              "note": "same steps with stage timing (one render lane); the timed run uses two"},
        "wall_ms_per_step": wall / args.steps * 1e3, "bvh_build_ms": info.bvh_build_ms, "bvh_tree_ms": info.bvh_tree_ms, "bvh_depth": info.bvh_depth,
        "load_s": load_s, "scene_generation_s": gen_s, "device_bytes": info.device_bytes,
        "estimate_finite": bool(np.isfinite(est).all()), "media_overflow": s1["media_overflow"],
        "trial_cap": s1["trial_cap"], "clocks": sampler.summary(),
    }
    if args.serve_stress:
        line["served"] = serve_stress(job, path, args.steps)
    print(json.dumps(line), flush=True)
    job.close()


def serve_stress(job, path, passes):
    """The stress job served: one request of `passes` passes through
    hasty_server_* (scene loaded by the server's loader threads), its latency
    and rate, and its sums against the single-job path's for the same passes
    and seed (bit-identical expected)."""
    import numpy as np
    from hastyrenderer_gb300 import Server
    job.reset()
    job.render_passes(passes, sync=True)
    plain = job.read_sums()[0]
    seed = job.info.seed
    with Server(paths_in_flight=1 << 24, lanes=2) as srv:
        t0 = time.perf_counter()
        rid = srv.submit(path, passes=passes, seed=seed)
        srv.wait_idle(-1)
        res = srv.poll(wait_ms=0)
        wall = time.perf_counter() - t0
        st = srv.stats()
        sums = srv.read_sums(rid)
    r = res[0]
    return {"status": r["status"], "latency_ms": r["latency_ms"], "wall_s": wall,
            "samples_per_s_device": r["samples"] / max(st["device_ms"] * 1e-3, 1e-9),
            "samples_per_s_wall": r["samples"] / wall, "equal_to_single_job_path": bool(np.array_equal(sums, plain)),
            "note": "latency includes the server's scene load (parse, BVH build, upload)"}



if __name__ == "__main__":
    main()
