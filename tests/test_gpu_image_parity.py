"""Image parity at the benchmark configurations: per-pixel z-tests of GPU
images against the CPU oracle (the reference's estimateRadiance,
core/src/PathTracing.cpp:21-95, restated and pinned bit-for-bit to the
reference build) on the same seeded scenes.

The GPU renders S samples per pixel (passes 0..S-1); the oracle renders the
reference, N = 16 S samples on passes S..S+N-1, and a null image, S samples
on passes S+N..S+N+S-1. Each GPU image passes zstat.ztest: per pixel and
channel, its 4-sigma exceedances, block exceedances and mean z must match
the null image's (the reference compared with itself), as zstat explains.
"""
import os
import tempfile

import numpy as np
import pytest

from zstat import gpu_moments, oracle_ref_and_null, ztest

pytestmark = pytest.mark.gpu


def _scene(name, make):
    base = os.path.join(tempfile.gettempdir(), "hasty_parity_" + name)
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        make(base)
    return path


def _pick_blocks(gs, gs2, S, size, n, key):
    """Corners of n non-overlapping size x size blocks maximising key(block
    mean, block variance) (deterministic: the GPU's own moments)."""
    m = gs / S
    v = np.maximum(gs2 / S - m * m, 0.0)
    h, w = m.shape[:2]
    scores = []
    for y in range(0, h - size + 1, size):
        for x in range(0, w - size + 1, size):
            scores.append((key(m[y:y + size, x:x + size], v[y:y + size, x:x + size]), x, y))
    scores.sort(reverse=True)
    return [(x, y, size, size) for _, x, y in scores[:n]]


def test_c0_cornell_full_frame():
    """Benchmark configuration 0 in full: Cornell box 256x256, 64 spp,
    depth 8, roulette from depth 3; the oracle at 1024 spp."""
    from hastyrenderer_gb300 import RenderJob, scenes
    from oracle.oracle import Oracle
    path = _scene("c0", lambda d: scenes.cornell_box(d, seed=0, width=256, height=256, spp=64, max_depth=8,
                                                     roulette_start_depth=3))
    S, N = 64, 1024
    job = RenderJob(path)
    (gs, gs2), = gpu_moments(job, S, [(0, 0, 256, 256)])
    ora = Oracle(path)
    cs, cs2, nulls = oracle_ref_and_null(ora, S, N, 0, 0, 256, 256)
    ztest("C0 cornell 256x256", gs, gs2, S, cs, cs2, N, nulls)


def test_c1_sphere_field_crops():
    """Benchmark configuration 1 (800 icospheres, 1,024,002 triangles,
    1920x1080, thin lens with 6 blades, 2048x1024 sky with the sun, depth 12)
    rendered in full on the GPU at 64 spp; three 16x16 crops tested against
    the oracle at 1024 spp: the two blocks of highest variance (sun through
    glass, caustics) and the block with the largest spread of the mean
    (object edges, blurred by the lens)."""
    from hastyrenderer_gb300 import RenderJob, scenes
    from oracle.oracle import Oracle
    path = _scene("c1", lambda d: scenes.sphere_field(d, seed=0))
    S, N = 64, 1024
    job = RenderJob(path)
    W, H = job.width, job.height
    (fs, fs2), = gpu_moments(job, 8, [(0, 0, W, H)])
    crops = _pick_blocks(fs, fs2, 8, 16, 2, lambda m, v: float(v.mean()))
    crops += [c for c in _pick_blocks(fs, fs2, 8, 16, 3, lambda m, v: float(m.std())) if c not in crops][:1]
    job.reset()
    moments = gpu_moments(job, S, crops)
    ora = Oracle(path)
    for (x, y, w, h), (gs, gs2) in zip(crops, moments):
        cs, cs2, nulls = oracle_ref_and_null(ora, S, N, x, y, w, h)
        ztest(f"C1 crop at ({x}, {y})", gs, gs2, S, cs, cs2, N, nulls)


def test_c4_stress_crop():
    """Benchmark configuration 4 (10,360,016 triangles, 3840x2160, Cauchy
    dispersive glass, RGBA8 albedo/normal maps, three area lights and the
    sky, depth 32) rendered in full on the GPU at 16 spp; the 16x16 block of
    highest variance and the block with the largest spread of the mean tested
    against the oracle at 256 spp. The medium stack must not overflow."""
    from hastyrenderer_gb300 import RenderJob, scenes
    from oracle.oracle import Oracle
    path = _scene("c4", lambda d: scenes.stress_scene(d, seed=4))
    S, N = 16, 256
    job = RenderJob(path)
    W, H = job.width, job.height
    (fs, fs2), = gpu_moments(job, 4, [(0, 0, W, H)])
    crops = _pick_blocks(fs, fs2, 4, 16, 1, lambda m, v: float(v.mean()))
    crops += [c for c in _pick_blocks(fs, fs2, 4, 16, 3, lambda m, v: float(m.std())) if c not in crops][:1]
    job.reset()
    moments = gpu_moments(job, S, crops)
    assert job.stats()["media_overflow"] == 0
    ora = Oracle(path)
    for (x, y, w, h), (gs, gs2) in zip(crops, moments):
        cs, cs2, nulls = oracle_ref_and_null(ora, S, N, x, y, w, h)
        ztest(f"C4 crop at ({x}, {y})", gs, gs2, S, cs, cs2, N, nulls)


def _small_mix():
    """Six jobs of the mixed distribution's scene kinds at 64x48: three
    Cornell boxes and fields of 50, 200 and 800 icospheres, 64 spp."""
    from hastyrenderer_gb300 import scenes
    out = []
    for k in range(3):
        out.append(_scene(f"mix_cornell{k}", lambda d, k=k: scenes.cornell_box(d, seed=10 + k, width=64, height=48,
                                                                               spp=64, max_depth=8 + 4 * k)))
    for k, n in enumerate((50, 200, 800)):
        out.append(_scene(f"mix_field{n}", lambda d, k=k, n=n: scenes.sphere_field(
            d, seed=20 + k, n_spheres=n, width=64, height=48, spp=64, max_depth=10 + 2 * k, env_size=(512, 256))))
    return out


def test_batched_and_served_images():
    """A small mix batched (hasty_batch_render) and served (hasty_server_*):
    every image passes the z-test against the oracle (the oracle's variance
    for both sides), equals the single-job path's image, and so has the same
    RMSE against a converged single-job image (1024 spp) as the single-job
    path has (difference 0, within the 1% asked for); the converged image
    passes the z-test too, against a null image of as many oracle samples."""
    from hastyrenderer_gb300 import RenderJob, Server, batch_render
    from oracle.oracle import Oracle
    paths = _small_mix()
    S, N = 64, 1024
    batched = [RenderJob(p) for p in paths]
    batch_render(batched, [S] * len(paths), paths_in_flight=1 << 18, lanes=2)
    with Server(paths_in_flight=1 << 18, quantum_samples=1 << 16) as srv:
        ids = [srv.submit(p, passes=S) for p in paths]
        srv.wait_idle(600000)
        served = {}
        while len(served) < len(ids):
            for r in srv.poll(wait_ms=1000):
                assert r["status"] == 0, r["error"]
                served[r["id"]] = srv.read_sums(r["id"])
    for p, jb, rid in zip(paths, batched, ids):
        name = os.path.basename(os.path.dirname(p))
        ora = Oracle(p)
        w, h = jb.width, jb.height
        cs, cs2, nulls = oracle_ref_and_null(ora, S, N, 0, 0, w, h)
        vc = np.maximum(cs2 / N - (cs / N) ** 2, 0.0)

        def second(sums, n):
            # the reference's per-sample variance for a side whose squares are not kept
            return (vc + (sums / n) ** 2) * n
        for label, sums in (("batched", jb.read_sums()[0]), ("served", served[rid])):
            ztest(f"{name} {label}", sums, second(sums, S), S, cs, cs2, N, [(ns, second(ns, S)) for ns, _ in nulls])
        plain = RenderJob(p)
        plain.render_passes(S, sync=True)
        assert np.array_equal(plain.read_sums()[0], jb.read_sums()[0])
        assert np.array_equal(plain.read_sums()[0], served[rid])
        conv = RenderJob(p)
        conv.set_seed(999)
        C = N
        conv.render_passes(C, sync=True)
        ref = conv.read_sums()[0] / C
        # the converged image (C samples on the streams of seed 999) against two
        # null images of as many oracle samples (passes after the others)
        conv_nulls = [ora.render(S + N + 3 * S + k * C, C, 0, 0, w, h)["color"] for k in range(2)]
        ztest(f"{name} converged", ref * C, second(ref * C, C), C, cs, cs2, N,
              [(n2, second(n2, C)) for n2 in conv_nulls])
        rmse_b = np.sqrt(np.mean((jb.read_sums()[0] / S - ref) ** 2))
        rmse_p = np.sqrt(np.mean((plain.read_sums()[0] / S - ref) ** 2))
        assert abs(rmse_b - rmse_p) <= 0.01 * rmse_p, (name, rmse_b, rmse_p)
        print(f"[{name}] RMSE vs converged: batched {rmse_b:.6g}, single-job {rmse_p:.6g}")
