"""Benchmark of the plain single-job path tracer on the large seeded workload.

Workload: 800 subdivision-3 icospheres + ground (1,024,002 triangles), FP32
2048x1024 procedural sky (importance sampled), 1920x1080, thin lens with 6
aperture blades, max depth 12; one step = SPP_PER_STEP passes (camera samples
per pixel) over the full frame, rendered as one batch of 16.6M paths. Inputs
stay resident on the device; the working set (path state ~7 GB per render
lane, BVH + triangles ~0.3 GB) is far larger than L2, so no explicit flush is
done between steps.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints one JSON line (rank 0). `value` is camera samples per second over all
ranks (each rank renders its own pass range of the same job: weak scaling);
`e2e` is the same metric through the C ABI including the job load (host
parse, BVH build, host->device upload) and a device->host read of the colour
estimate of every step (hasty_job_snapshot: copied while the next step
renders, as a progressive viewer reads it). `cpu_baseline` times the CPU oracle (oracle/)
on this host's cores on a bounded crop of the same job.
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
WORKLOAD = "sphere_field_800x_icosphere3_1024002tri_1920x1080_dof6_sky2048x1024_depth12"
# Algorithmic bytes per shaded vertex: path state read + write (2 x 96 B) and
# the triangle's attributes (92 B); texel reads are not counted.
B_SHADE = 2 * 96 + 92
# DRAM bytes per launch (dram__bytes_read.sum + dram__bytes_write.sum, averaged
# over the 12 bounces of one 8-pass batch of 16,588,800 paths, wide BVH) from
# one ncu capture of `bench.py --steps 1 --warmup 3 --spp-per-step 8`, the
# batches of the default run (captures of 2- and 4-pass batches gave 1/4 and
# 1/2 of these bytes). The
# shading stage is one k_resolve and one k_sample launch per bounce.
MEASURED_TRAFFIC = {"wide": {"k_trace": 461.4e6, "k_resolve+k_sample": 939.9e6 + 738.9e6}}
MEASURED_TRAFFIC_PASSES = 8


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


def make_job(base: str, seed: int = 0) -> str:
    from hastyrenderer_gb300 import scenes
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.sphere_field(base, seed=seed, n_spheres=800, subdiv=3, width=1920, height=1080, spp=256, max_depth=12)
    return path


def cpu_baseline(job_path: str, budget_s: float = 12.0, threads: int = 0):
    """CPU oracle on this host's cores: rows of a centred 128-pixel-wide crop,
    one pass each, until the time budget is spent. Also returns the BVH node
    visits and triangle tests per ray of the oracle's binary BVH."""
    from oracle.oracle import Oracle
    ora = Oracle(job_path)
    info = ora.info()
    threads = threads or (os.cpu_count() or 1)
    W, H = info["width"], info["height"]
    cw = 128
    x0 = (W - cw) // 2
    y = H // 2 - 32
    samples = 0
    rays = nodes = tris = shaded = 0
    t0 = time.perf_counter()
    k = 0
    while time.perf_counter() - t0 < budget_s:
        r = ora.render(k // 8, 1, x0, y + 8 * (k % 8), cw, 8, threads)
        st = r["stats"]
        samples += cw * 8
        rays += int(st[0]); nodes += int(st[2]); tris += int(st[3]); shaded += int(st[4])
        k += 1
    dt = time.perf_counter() - t0
    ora.close()
    return {"value": samples / dt, "unit": "samples/s", "cores": threads, "kind": "port",
            "sample": f"{samples} camera samples of a centred {cw}x64 crop (passes 0..{k // 8}), {dt:.1f} s",
            "mrays_per_s": rays / dt * 1e-6}, {"nodes_per_ray": nodes / max(rays, 1), "tris_per_ray": tris / max(rays, 1),
                                               "shaded_per_sample": shaded / max(samples, 1), "rays_per_sample": rays / max(samples, 1)}


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


def run_reference_arm(args, job_path: str, rank: int):
    if rank != 0:
        return
    from oracle.oracle import Oracle
    threads = os.cpu_count() or 1
    ora = Oracle(job_path)
    info = ora.info()
    cw, ch = 96, 16
    x0, y0 = (info["width"] - cw) // 2, info["height"] // 2 - ch
    for _ in range(args.warmup):
        ora.render(0, 1, x0, y0, cw, ch, threads)
    t0 = time.perf_counter()
    for k in range(args.steps):
        ora.render(k, 1, x0, y0, cw, ch, threads)
    dt = time.perf_counter() - t0
    v = args.steps * cw * ch / dt
    line = {"impl": "reference", "metric": "samples/s", "value": v, "unit": "samples/s", "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": WORKLOAD, "step": f"{cw}x{ch} crop x 1 pass on {threads} host threads"},
            "cpu_baseline": {"value": v, "unit": "samples/s", "cores": threads, "kind": "port",
                             "sample": f"{cw}x{ch} centred crop, 1 pass per step, {args.steps} steps"},
            "e2e": {"value": v, "unit": "samples/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=32)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp-per-step", type=int, default=SPP_PER_STEP)
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--bvh", default="wide", choices=["wide", "binary"])
    ap.add_argument("--workload", default="plain", choices=["plain", "batch", "serve", "stress", "photon"],
                    help="plain: the large single job (default); batch: the 64-job mix batched vs one by one; "
                         "serve: Poisson arrivals over the server; stress: 10.36M-triangle 4K scene, one pass per step; "
                         "photon: the photon mapper on the textured room, one progressive iteration per step")
    ap.add_argument("--jobs", type=int, default=64, help="batch/serve: jobs in the mix (serve: scene pool = half)")
    ap.add_argument("--rate", type=float, default=20.0, help="serve: arrivals per second")
    ap.add_argument("--duration", type=float, default=120.0, help="serve: seconds of arrivals")
    ap.add_argument("--no-tune", action="store_true", help="batch/serve: skip the autotuner (engine defaults)")
    args = ap.parse_args()
    if args.workload == "stress":
        return run_stress(args)
    if args.workload == "photon":
        return run_photon(args)
    if args.workload != "plain":
        return run_mixed(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        if args.impl == "ours":
            torch.cuda.set_device(local_rank)
        # the reference arm runs on the host cores only (gloo, no device)
        dist.init_process_group("nccl" if args.impl == "ours" else "gloo")

    base = os.environ.get("HASTY_BENCH_DIR", os.path.join(tempfile.gettempdir(), "hasty_bench_c1"))
    if rank == 0:
        os.makedirs(base, exist_ok=True)
        job_path = make_job(base)
    if dist is not None:
        dist.barrier()
    job_path = os.path.join(base, "renderJob.json")

    if args.impl == "reference":
        run_reference_arm(args, job_path, rank)
        if dist is not None:
            dist.destroy_process_group()
        return

    import torch
    from hastyrenderer_gb300 import Context, RenderJob
    torch.cuda.init()
    ctx = Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0)

    # ---- end to end through the C ABI: load (parse, BVH, upload) + steps with read-back
    if dist is not None:
        dist.barrier()
    t0 = time.perf_counter()
    job = RenderJob(job_path, ctx)
    info = job.info
    load_ms = (time.perf_counter() - t0) * 1e3
    W, H = info.width, info.height
    # each step's colour estimate is read back while the next step renders
    # (hasty_job_snapshot: estimate behind the step, copy on a copy stream)
    est_sum = 0.0
    for k in range(args.steps):
        job.render_passes(args.spp_per_step)
        if k:
            est, _ = job.snapshot_get()
            est_sum += float(est[0, 0, 0])
        job.snapshot()
    est, n_est = job.snapshot_get()
    e2e_s = time.perf_counter() - t0
    assert n_est == args.steps * args.spp_per_step
    e2e_bytes_up = info.device_bytes
    del est

    # ---- device-resident timing (both render lanes, as a user's render runs)
    job.reset()
    job.set_seed(replica_seed(rank))
    for _ in range(args.warmup):
        job.render_passes(args.spp_per_step)
    job.sync()
    s0 = job.stats()
    sampler = ClockSampler(local_rank)
    start = torch.cuda.Event(enable_timing=True)
    end = torch.cuda.Event(enable_timing=True)
    with sampler:
        if dist is not None:
            dist.barrier()
        torch.cuda.synchronize()
        start.record()
        w0 = time.perf_counter()
        for _ in range(args.steps):
            job.render_passes(args.spp_per_step)
        job.sync()
        torch.cuda.synchronize()
        end.record()
        end.synchronize()
        wall = time.perf_counter() - w0
        if dist is not None:
            dist.barrier()
    s1 = job.stats()
    # Per-stage split for the roofline: the same steps with stage timing,
    # which keeps one render lane so that kernel times are not shared.
    job.set_stage_timing(True)
    job.render_passes(args.spp_per_step)
    job.sync()
    st0 = job.stats()
    for _ in range(args.steps):
        job.render_passes(args.spp_per_step)
    job.sync()
    st1 = job.stats()
    job.set_stage_timing(False)
    dev_s = (s1["kernel_ms"] - s0["kernel_ms"]) * 1e-3
    t = max(dev_s, 1e-9)
    t = max_over_ranks(t, dist, "cuda")
    samples = args.steps * args.spp_per_step * W * H
    rays = s1["rays"] - s0["rays"]
    shaded = s1["shaded"] - s0["shaded"]
    trace_ms = st1["trace_ms"] - st0["trace_ms"]
    shade_ms = st1["shade_ms"] - st0["shade_ms"]
    one_lane_ms = st1["kernel_ms"] - st0["kernel_ms"]
    launches = s1["kernel_launches"] - s0["kernel_launches"]
    trace_launches = st1["trace_launches"] - st0["trace_launches"]
    clocks = sampler.summary()

    if rank == 0:
        hbm, peak_kind = peaks()
        cpu, bvh_costs = (None, None)
        if not args.no_cpu_baseline:
            cpu, bvh_costs = cpu_baseline(job_path, args.cpu_budget)
        roof, kernels = None, []
        if bvh_costs is not None:
            b_ray = 32 + 16 + 64 * bvh_costs["nodes_per_ray"] + 48 * bvh_costs["tris_per_ray"]
            # the measured bytes scale with the passes in a batch
            batch_passes = min(args.spp_per_step, max(1, info.paths_in_flight // (W * H)))
            traffic = {k: v * batch_passes / MEASURED_TRAFFIC_PASSES
                       for k, v in MEASURED_TRAFFIC.get(args.bvh, {}).items()}
            n_launch = max(trace_launches, 1)
            rays_st, shaded_st = st1["rays"] - st0["rays"], st1["shaded"] - st0["shaded"]
            for name, work, unit_bytes, ms in (("k_trace", rays_st, b_ray, trace_ms),
                                                ("k_resolve+k_sample", shaded_st, B_SHADE, shade_ms)):
                per_launch_bytes = work * unit_bytes / n_launch
                achieved = per_launch_bytes / (ms * 1e-3 / n_launch) / 1e9
                kernels.append({"bound": "hbm", "kernel": name, "achieved": achieved, "peak": hbm, "unit": "GB/s",
                                "frac": achieved / hbm, "peak_kind": peak_kind,
                                "traffic": traffic.get(name), "algorithmic_bytes_per_launch": per_launch_bytes,
                                "ms_per_launch": ms / n_launch,
                                "bytes_per_unit": unit_bytes, "unit_of_work": "ray" if name == "k_trace" else "shaded vertex"})
            kernels[0].update({"bvh_nodes_per_ray": bvh_costs["nodes_per_ray"], "tris_per_ray": bvh_costs["tris_per_ray"]})
            roof = dict(max(kernels, key=lambda k: k["ms_per_launch"]))
            roof["note"] = ("dominant kernel by device time, timed alone (one render lane); traffic = measured DRAM "
                            "bytes per launch (ncu), well below the algorithmic bytes because L1/L2 hold the upper "
                            "BVH levels")
        line = {
            "metric": "samples/s", "value": samples * world / t, "unit": "samples/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": t / args.steps * 1e3, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scene)",
            "config": {"workload": WORKLOAD, "spp_per_step": args.spp_per_step, "width": W, "height": H, "bvh": args.bvh,
                       "max_depth": info.max_depth, "triangles": info.n_triangles,
                       "l2": "working set > L2 (path state + BVH), no flush", "parallelism": f"replicas x{world}"},
            "mrays_per_s": rays * world / t * 1e-6,
            "stage_ms_per_step": {"trace": trace_ms / args.steps, "shade": shade_ms / args.steps,
                                  "one_lane_total": one_lane_ms / args.steps,
                                  "note": "same steps with stage timing, which keeps one render lane; the timed "
                                          "run uses two lanes, one batch's trace overlapping the other's shading"},
            "wall_ms_per_step": wall / args.steps * 1e3,
            "gpu_launches": launches,
            "roofline": roof,
            "kernels": kernels,
            "cpu_baseline": cpu,
            "e2e": {"value": args.steps * args.spp_per_step * W * H * world / e2e_s, "unit": "samples/s",
                    "h2d_bytes_per_step": int(e2e_bytes_up // args.steps), "d2h_bytes_per_step": W * H * 3 * 4,
                    "includes": "job load (parse, BVH build, upload) + steps + a colour read-back per step, each copied while the next step renders",
                    "load_ms": {"total": load_ms, "parse": info.parse_ms, "bvh_build": info.bvh_build_ms,
                                "upload": info.upload_ms}},
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    job.close()
    if dist is not None:
        dist.destroy_process_group()


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
    print(json.dumps(line), flush=True)
    job.close()


def _rel_diff(a, b):
    import numpy as np
    den = float(np.linalg.norm(b.astype(np.float64)))
    return float(np.linalg.norm(a.astype(np.float64) - b.astype(np.float64))) / max(den, 1e-30)


def _tuned(args, jobs, ctx):
    """Engine parameters from the autotuner (cached per GPU name)."""
    import torch
    from hastyrenderer_gb300 import RenderJob, autotune
    path = autotune.default_path(torch.cuda.get_device_name())
    if args.no_tune:
        return {"paths_in_flight": 1 << 22, "regen_fraction": 0.9, "source": "defaults"}
    cached = autotune.load(path)
    if cached:
        cached["source"] = path
        return cached
    calib = [RenderJob(j["path"], ctx) for j in jobs[:16]]
    res = autotune.tune_batch(calib, passes=2, out_path=path)
    for c in calib:
        c.close()
    res["source"] = "tuned now"
    return res


def run_mixed(args):
    """Mixed-job workloads: batching (the same jobs one by one through
    hasty_job_render_passes, then all at once through hasty_batch_render) or
    serving (Poisson arrivals through hasty_server_*)."""
    import numpy as np
    import torch
    from hastyrenderer_gb300 import Context, RenderJob, Server, autotune, batch_render, workloads
    rank = int(os.environ.get("RANK", "0"))
    local_rank = int(os.environ.get("LOCAL_RANK", "0"))
    if rank != 0:
        return
    torch.cuda.init()
    base = os.environ.get("HASTY_BENCH_MIX", os.path.join(tempfile.gettempdir(), "hasty_bench_mix"))
    t_gen = time.perf_counter()
    jobs = workloads.mixed_jobs(base, n_jobs=args.jobs, seed=0)
    gen_s = time.perf_counter() - t_gen
    ctx = Context(local_rank, Context.BINARY_BVH if args.bvh == "binary" else 0)
    tune = _tuned(args, jobs, ctx)
    engine_args = autotune.batch_args(tune)
    hbm, peak_kind = peaks()
    sampler = ClockSampler(local_rank)

    if args.workload == "batch":
        total = sum(workloads.job_samples(j) for j in jobs)
        t0 = time.perf_counter()
        resident = [RenderJob(j["path"], ctx) for j in jobs]
        load_s = time.perf_counter() - t0
        spp = [j["spp"] for j in jobs]
        plain_est = []
        with sampler:
            # plain drop-in, one job after another (device time from the job's own CUDA events)
            plain_ms = 0.0
            plain_rays = 0
            w0 = time.perf_counter()
            for job, p in zip(resident, spp):
                s0 = job.stats()
                job.render_passes(p, sync=True)
                s1 = job.stats()
                plain_ms += s1["kernel_ms"] - s0["kernel_ms"]
                plain_rays += s1["rays"] - s0["rays"]
                plain_est.append(job.compute_estimate())
                job.release_paths()
                job.reset()
            plain_wall = time.perf_counter() - w0
            for _ in range(max(args.warmup - 2, 0)):   # the autotuner's trials already warmed the engine
                batch_render(resident[:8], [2] * 8, **engine_args)
                for job in resident[:8]:
                    job.reset()
            w0 = time.perf_counter()
            st = batch_render(resident, spp, **engine_args)
            batch_wall = time.perf_counter() - w0
        diffs = [_rel_diff(job.compute_estimate(), ref) for job, ref in zip(resident, plain_est)]
        batch_sps = total / (st["device_ms"] * 1e-3)
        plain_sps = total / (plain_ms * 1e-3)
        line = {
            "metric": "samples/s", "value": batch_sps, "unit": "samples/s", "n_gpus": 1, "steps": 1,
            "warmup": args.warmup, "ms_per_step": st["device_ms"], "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
            "config": {"workload": f"mixed_{len(jobs)}_jobs_batched", "jobs": len(jobs), "samples": total,
                       "engine": engine_args, "l2": "working set > L2 (path pool + scenes), no flush"},
            "mrays_per_s": st["rays"] / (st["device_ms"] * 1e-3) * 1e-6,
            "plain": {"value": plain_sps, "unit": "samples/s", "device_ms": plain_ms, "wall_ms": plain_wall * 1e3,
                      "mrays_per_s": plain_rays / (plain_ms * 1e-3) * 1e-6},
            "batched_over_plain": batch_sps / plain_sps,
            "wall": {"batched_ms": batch_wall * 1e3, "plain_ms": plain_wall * 1e3, "load_s": load_s,
                     "scene_generation_s": gen_s},
            "equal_estimate": {"max_rel_l2_diff_vs_plain": max(diffs), "note": "same samples; fixed-point vs FP64 sums"},
            "engine_iterations": st["iterations"], "engine_bytes": st["engine_bytes"],
            "autotune": {k: tune[k] for k in ("paths_in_flight", "regen_fraction", "samples_per_s", "source") if k in tune},
            "clocks": sampler.summary(), "peak_hbm_gbs": hbm, "peak_kind": peak_kind,
        }
        print(json.dumps(line), flush=True)
        return

    # serving: Poisson arrivals over a warm scene pool
    pool = jobs[: max(1, len(jobs) // 2)]
    reqs = workloads.poisson_requests(pool, os.path.join(base, f"requests_{args.rate:g}_{args.duration:g}"),
                                      rate=args.rate, duration=args.duration, seed=1)
    srv = Server(ctx, memory_budget=120 << 30, max_resident_jobs=32, max_resident_scenes=32, **engine_args)
    t0 = time.perf_counter()
    for j in pool:                       # warm the scene cache: one cheap request per scene
        srv.submit(j["path"], passes=1)
    srv.wait_idle(-1)
    for r in srv.poll(max_results=len(pool) + 8, wait_ms=0):
        srv.release(r["id"])
    warm_s = time.perf_counter() - t0
    st0 = srv.stats()
    results = []
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
    line = {
        "metric": "samples/s", "value": samples / span, "unit": "samples/s", "n_gpus": 1, "steps": len(reqs),
        "warmup": len(pool), "ms_per_step": span * 1e3 / max(len(reqs), 1), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded procedural scenes)",
        "config": {"workload": f"serving_poisson_{args.rate:g}_per_s_{args.duration:g}_s", "requests": len(reqs),
                   "scene_pool": len(pool), "engine": engine_args, "max_resident_jobs": 32, "memory_budget": 120 << 30},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p95": float(np.percentile(lat, 95)),
                       "p99": float(np.percentile(lat, 99)), "max": float(lat.max())},
        "completed": len(ok), "failed": len(results) - len(ok),
        "device_samples_per_s": samples / max(dev_ms * 1e-3, 1e-9),
        "mrays_per_s": (st1["rays"] - st0["rays"]) / max(dev_ms * 1e-3, 1e-9) * 1e-6,
        "offered_samples_per_s": sum(r["width"] * r["height"] * r["spp"] for r in reqs) / args.duration,
        "peak_resident_bytes": st1["peak_resident_bytes"], "warm_s": warm_s, "span_s": span,
        "autotune": {k: tune[k] for k in ("paths_in_flight", "regen_fraction", "samples_per_s", "source") if k in tune},
        "clocks": sampler.summary(),
    }
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
