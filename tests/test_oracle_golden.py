"""The CPU oracle (oracle/port) against fixtures written by the reference's
own code (tests/golden/make_golden.py, from the build under oracle/_ref), and
the reference's unit tests (apps/Tests.cpp) run on the oracle."""
import os

import numpy as np
import pytest

from oracle.oracle import Oracle, kat, property_test, rng_stream

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rel(a, b):
    return np.abs(a - b) / np.maximum(1.0, np.abs(b))


def test_bsdf_kat_matches_reference():
    """PrincipledBRDF sample/evaluate/pdf on 1500 random cases with replayed
    uniforms: the restatement reproduces the reference to 1e-6 relative
    (bit-identical in practice) and consumes the same number of uniforms."""
    g = np.load(os.path.join(GOLDEN, "kat_bsdf.npz"))
    for which, name in ((0, "sample"), (1, "evaluate"), (2, "pdf")):
        ours = kat(which, g["inputs"], g["replay"])
        ref = g[name]
        cols = 11 if which == 0 else (9 if which == 1 else 1)
        assert np.array_equal(np.isnan(ours[:, :cols]), np.isnan(ref[:, :cols])), name
        ok = ~np.isnan(ref[:, :cols])
        assert _rel(ours[:, :cols][ok], ref[:, :cols][ok]).max() <= 1e-6, name
        if which == 0:
            assert np.array_equal(ours[:, 11], ref[:, 11]), "uniform draws differ"


@pytest.mark.parametrize("which", list(range(3, 16)))
def test_sampling_kat_matches_reference(which):
    g = np.load(os.path.join(GOLDEN, "kat_sampling.npz"))
    ours = kat(which, g[f"in_{which}"], g[f"replay_{which}"])
    ref = g[f"out_{which}"]
    ok = ~np.isnan(ref)
    assert np.array_equal(np.isnan(ours), np.isnan(ref))
    assert _rel(ours[ok], ref[ok]).max() <= 1e-6


@pytest.mark.parametrize("name", ["cornell", "field", "room", "room_nomis", "nested"])
def test_render_matches_reference(name):
    """estimateRadiance over 16 passes of a seeded job: per-pixel sums equal to
    the reference's own integrator on the same streams."""
    g = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    job = os.path.join(GOLDEN, "scenes", name, "renderJob.json")
    ora = Oracle(job)
    h, w = g["color"].shape[:2]
    r = ora.render(0, int(g["passes"]), 0, 0, w, h, 4)
    for k in ("color", "normal", "albedo"):
        assert np.allclose(r[k], g[k], rtol=1e-6, atol=1e-9), k
    c, n, a = ora.render_samples(0, 0, 0, w, h)
    assert np.array_equal(np.isnan(c), np.isnan(g["sample_color"]))
    m = ~np.isnan(c)
    assert np.allclose(c[m], g["sample_color"][m], rtol=1e-6, atol=1e-9)
    assert r["stats"][0] > 0


def test_rng_stream_spec():
    g = np.load(os.path.join(GOLDEN, "rng_streams.npz"))
    for key in g.files:
        seed, pixel, p = (int(x) for x in key[1:].split("_"))
        assert np.array_equal(rng_stream(seed, pixel, p, 16), g[key])


# ---- the reference's unit tests (apps/Tests.cpp), run on the oracle -------
def test_rodrigues_rotation():                      # Tests.cpp:40-52
    assert property_test(0, 200)[0] <= 1e-4 * np.sqrt(3)


def test_spherical_coordinates():                   # Tests.cpp:54-74
    m, tmin, tmax, pmin, pmax = property_test(1, 50)
    assert m <= 1e-4 * np.sqrt(3)
    assert tmin >= 0 and tmax <= np.pi + 1e-6 and pmin >= 0 and pmax <= 2 * np.pi + 1e-6


def test_sample_cosine_lobe():                      # Tests.cpp:76-90
    rel, ln = property_test(2, 50)
    assert rel <= 1e-5 and ln <= 1e-5


def test_sample_hemisphere_cos_importance():        # Tests.cpp:93-106
    rel, ln = property_test(3, 50)
    assert rel <= 1e-4 and ln <= 1e-4


def test_dggx_normalisation():                      # Tests.cpp:107-131
    est, mind = property_test(4, 50000)
    assert abs(est - 1.0) <= 1e-2 and mind >= 0.0


def test_sample_dggx_density():                     # Tests.cpp:132-147
    assert property_test(5, 50)[0] <= 1e-2


def test_sample_dggx_expectation():                 # Tests.cpp:148-168
    est, minp = property_test(6, 500000)
    assert abs(est - np.pi) <= 1e-2 * np.pi and minp >= 0.0


def test_sample_ggx_vndf_density():                 # Tests.cpp:169-187
    rel, minp = property_test(7, 50)
    assert rel <= 1e-2 and minp >= 0.0


def test_sample_ggx_vndf_expectation():             # Tests.cpp:188-210
    est, minp = property_test(8, 5000000)
    assert abs(est - np.pi) <= 1e-2 * np.pi and minp >= 0.0


def test_refraction_roundtrip_and_fresnel_reciprocity():   # Tests.cpp:212-232
    d, f = property_test(9, 1)
    assert d <= 1e-5 * np.sqrt(3) and f <= 1e-5


@pytest.mark.parametrize("name", ["cornell", "room", "field"])
def test_photon_mapper_matches_reference(name):
    """The restated photon mapper (oracle/port/oracle_pm.cpp) against the
    reference's own (PhotonMapping.cpp through oracle/ref_pm_harness.cpp):
    every progressive iteration's colour, normal, albedo and radius images and
    photon counts, bit for bit."""
    from oracle.oracle import PhotonMapper
    g = np.load(os.path.join(GOLDEN, f"pm_{name}.npz"))
    pm = PhotonMapper(os.path.join(GOLDEN, "scenes", name, "renderJob.json"))
    try:
        for it in range(g["color"].shape[0]):
            r = pm.iterate(1)
            assert r["emitted"] == g["emitted"][it] and r["stored"] == g["stored"][it], it
            for k in ("color", "normal", "albedo", "radii"):
                assert np.array_equal(r[k], g[k][it], equal_nan=True), (k, it)
    finally:
        pm.close()
