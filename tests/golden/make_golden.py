"""Writes the golden fixtures under tests/golden/ from the reference's own
integrator code, built under oracle/_ref by `make -C oracle ref` (needs the
reference sources, so this runs on the development machine only; the
fixtures are committed and travel with the tests).

  HASTY_REFERENCE_DIR=<reference checkout> python -m hastyrenderer_gb300.build --oracle
  python tests/golden/make_golden.py

Fixtures:
  * kat_bsdf.npz    - PrincipledBRDF::sample / evaluate / evaluateSamplePDF
                      (core/src/BRDF.cpp:630-742) on random inputs with
                      replayed uniform streams.
  * kat_sampling.npz - Sample.cpp / BRDF.cpp sampling routines (aperture
                      polygon, cosine hemisphere, triangle, GGX VNDF, Fresnel,
                      refraction, sphere, Rodrigues rotation, Smith/GGX D).
  * scenes/<name>/  - small seeded render jobs (OBJ/MTL/JSON/images): a
                      Cornell box; a sphere field with sky, DoF and
                      dispersive glass; a textured room (maps, anisotropy,
                      glass), with and without MIS; six nested glass shells
                      (the medium stack deeper than four) with a textured wall
                      that has no texture coordinates.
  * render_<name>.npz - estimateRadiance (core/src/PathTracing.cpp:21-95)
                      sums over passes 0..P-1 and pass-0 per-sample values,
                      with the project's per-(seed, pixel, pass) PCG streams.
  * rng_streams.npz - first outputs of a few path streams (the stream spec).

Input layout of the BSDF known-answer cases (33 floats): x(3), Ng(3),
Ns(3), tangent(3), bitangent(3), albedo(3), metallic, specular, roughness,
anisotropy, transmission, IOR, vary-IOR flag, wo(3), wi(3), wavelength,
outside IOR. Outputs (12 floats): sample = outside, dir(3), thrDiffuse(3),
thrConcentrated(3), pdf, draws; evaluate = fDiffuse(3), fConcentrated(3),
shading normal(3); pdf = pdf.
"""
from __future__ import annotations

import os
import shutil
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from hastyrenderer_gb300 import scenes  # noqa: E402
from oracle.oracle import ReferenceBuild, kat, rng_stream  # noqa: E402

N_KAT = 1500
N_REPLAY = 64
RENDER_PASSES = 16

GOLDEN_SCENES = {
    "cornell": lambda d: scenes.cornell_box(d, seed=0, width=32, height=32, spp=4, max_depth=8, roulette_start_depth=3),
    "field": lambda d: scenes.sphere_field(d, seed=1, n_spheres=12, subdiv=1, width=24, height=24, spp=4,
                                           env_size=(64, 32), vary_glass_ior=True, box=4.0),
    "room": lambda d: scenes.textured_room(d, seed=2, width=32, height=24, spp=4),
    "room_nomis": lambda d: scenes.textured_room(d, seed=3, width=32, height=24, spp=4, use_mis=False),
    "nested": lambda d: scenes.nested_media(d, seed=5, width=32, height=24, spp=4),
}


def unit(v):
    return v / np.linalg.norm(v, axis=-1, keepdims=True)


def replay_streams(rng, n, k):
    out = np.empty((n, k), np.uint32)
    for i in range(n):
        out[i] = rng.choice(np.iinfo(np.uint32).max, size=k, replace=False).astype(np.uint32)
    return out


def bsdf_cases(rng, n):
    c = np.zeros((n, 33), np.float32)
    ng = unit(rng.normal(size=(n, 3)))
    smooth = rng.uniform(size=n) < 0.5
    ns = unit(ng + np.where(smooth[:, None], 0.3 * rng.normal(size=(n, 3)), 0.0))
    t = unit(np.cross(ng, rng.normal(size=(n, 3))))
    b = np.cross(ng, t)
    c[:, 0:3] = rng.uniform(-3, 3, (n, 3))
    c[:, 3:6] = ng; c[:, 6:9] = ns; c[:, 9:12] = t; c[:, 12:15] = b
    c[:, 15:18] = rng.uniform(0.0, 1.0, (n, 3))
    kind = rng.integers(0, 4, n)           # 0 rough dielectric, 1 metal, 2 glass, 3 smooth (delta) dielectric
    rough = np.where(kind >= 2, 0.0, rng.uniform(0.0, 1.0, n))
    metal = np.where(kind == 1, 1.0, np.where(kind == 0, rng.uniform(0, 1, n) * (rng.uniform(size=n) < 0.3), 0.0))
    trans = np.where(kind == 2, 1.0, np.where(kind == 3, rng.uniform(0, 1, n) * (rng.uniform(size=n) < 0.5), 0.0))
    c[:, 18] = metal; c[:, 19] = rng.uniform(0, 1, n); c[:, 20] = rough
    c[:, 21] = np.where(rng.uniform(size=n) < 0.3, rng.uniform(0, 1, n), 0.0)
    c[:, 22] = trans; c[:, 23] = rng.uniform(1.2, 1.8, n)
    vary = (rng.uniform(size=n) < 0.4) & (trans > 0)
    c[:, 24] = vary
    wo = unit(rng.normal(size=(n, 3)))
    c[:, 25:28] = wo
    c[:, 28:31] = unit(rng.normal(size=(n, 3)))
    c[:, 31] = np.where(vary, rng.integers(0, 3, n), -1)
    c[:, 32] = np.where(rng.uniform(size=n) < 0.6, 1.0, rng.uniform(1.0, 1.6, n))
    return c


def sampling_cases(rng, which, n):
    if which == 3:   # aperture polygon: blades, rotation
        return np.stack([rng.integers(3, 10, n), rng.uniform(-3.0, 3.0, n)], 1).astype(np.float32)
    if which == 4:   # cosine hemisphere around n
        return unit(rng.normal(size=(n, 3))).astype(np.float32)
    if which == 5:
        return np.zeros((n, 1), np.float32)
    if which == 6:   # VNDF: n, at, ab, t, b, wo (wo above n)
        nn = unit(rng.normal(size=(n, 3)))
        t = unit(np.cross(nn, rng.normal(size=(n, 3))))
        b = np.cross(nn, t)
        wo = unit(rng.normal(size=(n, 3)))
        wo = np.where((np.sum(wo * nn, 1) < 0)[:, None], -wo, wo)
        a = np.maximum(1e-2, rng.uniform(0, 1, (n, 2)))
        return np.concatenate([nn, a, t, b, wo], 1).astype(np.float32)
    if which == 7:   # Fresnel: cos_i, cos_t, eta_i, eta_t
        return np.stack([rng.uniform(0, 1, n), rng.uniform(0, 1, n), rng.uniform(1, 2, n), rng.uniform(1, 2, n)], 1).astype(np.float32)
    if which == 8:   # refraction: wi, n (wi on the normal's side), eta_i, eta_t
        nn = unit(rng.normal(size=(n, 3)))
        wi = unit(rng.normal(size=(n, 3)))
        wi = np.where((np.sum(wi * nn, 1) < 0)[:, None], -wi, wi)
        return np.concatenate([wi, nn, rng.uniform(1, 2, (n, 1)), rng.uniform(1, 2, (n, 1))], 1).astype(np.float32)
    if which == 9:
        return np.zeros((n, 1), np.float32)
    if which == 10:  # rotation: from, to, x
        return np.concatenate([unit(rng.normal(size=(n, 3))), unit(rng.normal(size=(n, 3))), rng.uniform(-1, 1, (n, 3))], 1).astype(np.float32)
    if which == 11:  # smith G1 and D: nv, tv, bv, at, ab
        return np.concatenate([rng.uniform(0.05, 1, (n, 1)), rng.uniform(-1, 1, (n, 2)), np.maximum(1e-2, rng.uniform(0, 1, (n, 2)))], 1).astype(np.float32)
    if which == 12:  # isotropic GGX sampling: n, alpha, d1
        nn = unit(rng.normal(size=(n, 3)))
        d1 = unit(rng.normal(size=(n, 3)))
        d1 = np.where((np.sum(d1 * nn, 1) < 0)[:, None], -d1, d1)
        return np.concatenate([nn, np.maximum(1e-2, rng.uniform(0, 1, (n, 1))), d1], 1).astype(np.float32)
    if which == 13:  # cosine lobe: lobe, exponent
        return np.concatenate([unit(rng.normal(size=(n, 3))), 1 + 10 * rng.uniform(0, 1, (n, 1))], 1).astype(np.float32)
    if which == 14:
        return unit(rng.normal(size=(n, 3))).astype(np.float32)
    if which == 15:  # cosine pdf: n, d
        return np.concatenate([unit(rng.normal(size=(n, 3))), unit(rng.normal(size=(n, 3)))], 1).astype(np.float32)
    raise ValueError(which)


def main():
    if not ReferenceBuild.available():
        raise SystemExit("oracle/_ref/libhasty_ref.so missing: run `make -C oracle ref` first")
    rng = np.random.default_rng(20261203)

    cases = bsdf_cases(rng, N_KAT)
    replay = replay_streams(rng, N_KAT, N_REPLAY)
    out = {"inputs": cases, "replay": replay}
    for which, name in ((0, "sample"), (1, "evaluate"), (2, "pdf")):
        out[name] = kat(which, cases, replay, reference=True)
    np.savez_compressed(os.path.join(HERE, "kat_bsdf.npz"), **out)

    samp = {}
    for which in range(3, 16):
        x = sampling_cases(rng, which, 400)
        r = replay_streams(rng, 400, N_REPLAY)
        # pad inputs to a common width
        xp = np.zeros((x.shape[0], 33), np.float32); xp[:, :x.shape[1]] = x
        samp[f"in_{which}"] = xp
        samp[f"replay_{which}"] = r
        samp[f"out_{which}"] = kat(which, xp, r, reference=True)
    np.savez_compressed(os.path.join(HERE, "kat_sampling.npz"), **samp)

    sdir = os.path.join(HERE, "scenes")
    for name, gen in GOLDEN_SCENES.items():
        d = os.path.join(sdir, name)
        if os.path.isdir(d):
            shutil.rmtree(d)
        job = gen(d)
        ref = ReferenceBuild(job)
        import json
        with open(job) as f:
            js = json.load(f)
        w, h = js["settings"]["width"], js["settings"]["height"]
        r = ref.render(0, RENDER_PASSES, 0, 0, w, h, 8)
        c0, n0, a0 = ref.render_samples(0, 0, 0, w, h)
        np.savez_compressed(os.path.join(HERE, f"render_{name}.npz"), color=r["color"], color_sq=r["color_sq"],
                            normal=r["normal"], albedo=r["albedo"], passes=RENDER_PASSES, sample_color=c0,
                            sample_normal=n0, sample_albedo=a0)
        ref.close()

    streams = {}
    for seed, pixel, p in ((0, 0, 0), (0, 1, 0), (0, 0, 1), (7, 12345, 99), (2**40 + 3, 2**31 + 5, 2**31 + 7)):
        streams[f"s{seed}_{pixel}_{p}"] = rng_stream(seed, pixel, p, 16)
    np.savez_compressed(os.path.join(HERE, "rng_streams.npz"), **streams)
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    main()
