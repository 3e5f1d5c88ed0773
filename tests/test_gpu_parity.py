"""CUDA path against the reference's own outputs (golden fixtures written by
the reference build, tests/golden/) and against the CPU oracle (oracle/) on
the same seeded scenes and per-path random streams. All calls go through the
C ABI (hastyrenderer_gb300.native)."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
SCENES = ["cornell", "field", "room", "room_nomis"]


def golden_job(name):
    return os.path.join(GOLDEN, "scenes", name, "renderJob.json")


def _job(path):
    from hastyrenderer_gb300 import RenderJob
    return RenderJob(path)


def _random_rays(n, rng, lo, hi):
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def _check_hits(g, c):
    g_tri, g_t = g[0], g[1]
    c_tri, c_t = c[0], c[1]
    agree = g_tri == c_tri
    assert agree.mean() >= 0.9999, agree.mean()
    both = agree & (c_tri >= 0)
    rel = np.abs(g_t[both] - c_t[both]) / np.maximum(np.abs(c_t[both]), 1e-30)
    assert rel.max() <= 1e-5, rel.max()
    return agree.mean()


@pytest.mark.parametrize("name,lo,hi", [("cornell", -1.0, 2.0), ("field", -3.0, 4.0), ("room", -2.0, 3.0)])
def test_intersect_matches_oracle(name, lo, hi):
    """Closest hits: triangle ids agree on >= 99.99% of rays (exactly, in
    practice), t within 1e-5 relative; the oracle's BVH answer is the same
    as a brute-force scan with the same FP32 triangle test."""
    job = _job(golden_job(name))
    ora = Oracle(golden_job(name))
    rays = _random_rays(50000, np.random.default_rng(5), lo, hi)
    g = job.intersect(rays)
    c = ora.intersect(rays)
    b = ora.intersect(rays, brute=True)
    assert np.array_equal(c[0], b[0])
    assert _check_hits(g, c) == 1.0
    assert (c[0] >= 0).mean() > 0.2


def test_intersect_full_size_scene(tmp_path):
    """The 1,024,002-triangle benchmark scene: camera-like and random rays."""
    from hastyrenderer_gb300 import scenes
    path = scenes.sphere_field(str(tmp_path / "c1"), seed=0)
    job = _job(path)
    ora = Oracle(path)
    rng = np.random.default_rng(11)
    rays = _random_rays(30000, rng, -10.0, 10.0)
    rays[:, 1] = np.abs(rays[:, 1]) + 0.01
    g = job.intersect(rays)
    c = ora.intersect(rays)
    _check_hits(g, c)
    assert job.info.n_triangles == 1024002


@pytest.mark.parametrize("name", SCENES)
def test_first_pass_matches_reference(name):
    """Pass 0 of each golden job: every camera sample follows the same random
    stream as in the reference's own estimateRadiance, so nearly every pixel
    equals the reference's value (1e-3 relative); AOVs likewise."""
    g = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    job = _job(golden_job(name))
    job.render_passes(1, sync=True)
    col, n = job.read_sums()
    nrm, _ = job.read_sums(1)
    alb, _ = job.read_sums(2)
    assert n == 1
    ref = g["sample_color"]
    ref = np.where(np.isnan(ref).any(-1, keepdims=True), 0.0, ref)
    close = np.all(np.abs(col - ref) <= 1e-3 * np.maximum(1.0, np.abs(ref)), axis=-1)
    assert close.mean() >= 0.97, close.mean()
    for ours, key in ((nrm, "sample_normal"), (alb, "sample_albedo")):
        c2 = np.all(np.abs(ours - g[key]) <= 1e-4 + 1e-4 * np.abs(g[key]), axis=-1)
        assert c2.mean() >= 0.99, (key, c2.mean())


@pytest.mark.parametrize("name", SCENES)
def test_sixteen_passes_match_reference(name):
    """16 passes against the reference's sums over the same 16 streams."""
    g = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    job = _job(golden_job(name))
    P = int(g["passes"])
    job.render_passes(P, sync=True)
    col, n = job.read_sums()
    assert n == P
    rel = np.abs(col - g["color"]) / np.maximum(1.0, np.abs(g["color"]))
    assert (rel.max(-1) <= 1e-3).mean() >= 0.9, (rel.max(-1) <= 1e-3).mean()
    assert abs(col.mean() - g["color"].mean()) <= 0.02 * abs(g["color"].mean()) + 1e-6


@pytest.mark.parametrize("name", ["cornell", "field", "room"])
def test_image_ztest(name):
    """Per-pixel means at S = 64 spp against the oracle at 16*S spp from the
    same streams: |mean_gpu - mean_cpu| <= 4 sigma per pixel, sigma from the
    per-sample variance of the oracle's 16*S samples for both estimates (its
    own Monte Carlo noise included). Sun and caustic paths make the radiance
    heavy-tailed, so the sample variance can underestimate sigma on a few
    pixels: at most 0.5% of pixels may exceed 4 sigma, and the signed
    z-scores must show no bias."""
    S = 64
    job = _job(golden_job(name))
    job.set_seed(777)
    job.render_passes(S, sync=True)
    g, n = job.read_sums()
    assert n == S
    ora = Oracle(golden_job(name))
    ora.set_seed(777)
    w, h = job.width, job.height
    N = 16 * S
    r = ora.render(0, N, 0, 0, w, h)
    # per-pixel channel mean
    sc = r["color"].mean(-1)
    mc = sc / N
    # variance of the channel mean of one sample, from the per-channel second moments (upper bound)
    var_c = np.maximum((r["color_sq"] / N - (r["color"] / N) ** 2).mean(-1), 0.0)
    mg = g.mean(-1) / S
    sig = np.sqrt(var_c / S + var_c / N) + 1e-6 + 1e-5 * np.abs(mc)
    z = (mg - mc) / sig
    assert (np.abs(z) > 4.0).mean() <= 0.005, ((np.abs(z) > 4.0).mean(), np.abs(z).max())
    assert abs(z.mean()) <= 0.25, z.mean()


def test_device_bsdf_matches_reference():
    """Device PrincipledBRDF sample/evaluate/pdf on the reference's
    known-answer cases (replayed uniforms): within 1e-5 relative on >= 99.5%
    of cases (CUDA's sinf/cosf/powf differ from glibc's by an ulp or two)."""
    from hastyrenderer_gb300 import debug_bsdf
    g = np.load(os.path.join(GOLDEN, "kat_bsdf.npz"))
    for which, name, cols in ((0, "sample", 11), (1, "evaluate", 9), (2, "pdf", 1)):
        ours = debug_bsdf(which, g["inputs"], g["replay"])[:, :cols]
        ref = g[name][:, :cols]
        ok = np.isfinite(ref).all(1)
        rel = np.abs(ours - ref) / np.maximum(1e-3, np.abs(ref))
        good = (rel <= 1e-5).all(1) | ~ok
        assert good.mean() >= 0.995, (name, good.mean())
        if which == 0:
            assert (debug_bsdf(0, g["inputs"], g["replay"])[:, 11] == g["sample"][:, 11]).mean() >= 0.995
