"""Host-side loader, BVH builders and the traversal code (the same source the
GPU runs, compiled for the host) against the CPU oracle: no GPU needed."""
import os

import numpy as np
import pytest

from hastyrenderer_gb300.api import host_trace
from oracle.oracle import Oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rays(n, seed, lo, hi):
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


@pytest.mark.parametrize("kind", [0, 1])
@pytest.mark.parametrize("name,lo,hi", [("cornell", -1.0, 2.0), ("field", -3.0, 4.0), ("room", -2.0, 3.0)])
def test_traversal_exact(kind, name, lo, hi):
    """Binary (0) and compressed 8-wide (1) BVH answer every ray exactly as a
    brute-force scan with the same FP32 triangle test."""
    job = os.path.join(GOLDEN, "scenes", name, "renderJob.json")
    rays = _rays(30000, 5, lo, hi)
    tri, t, _, _, info = host_trace(job, rays, kind)
    o = Oracle(job)
    b = o.intersect(rays, brute=True)
    assert np.array_equal(tri, b[0])
    hit = tri >= 0
    assert np.array_equal(t[hit], b[1][hit])
    assert info["triangles"] == o.info()["n_tris"]


def test_full_size_scene(tmp_path):
    """The 1,024,002-triangle benchmark scene: both trees agree with the
    oracle's BVH; the wide tree is shallower and has fewer nodes."""
    from hastyrenderer_gb300 import scenes
    job = scenes.sphere_field(str(tmp_path / "c1"), seed=0)
    rays = _rays(8000, 11, -10.0, 10.0)
    rays[:, 1] = np.abs(rays[:, 1]) + 0.01
    o = Oracle(job)
    c = o.intersect(rays)
    res = {}
    for kind in (0, 1):
        tri, t, _, _, info = host_trace(job, rays, kind)
        assert np.array_equal(tri, c[0])
        res[kind] = info
    assert res[0]["triangles"] == 1024002
    assert res[1]["depth"] < res[0]["depth"] and res[1]["depth"] <= 30
    assert res[1]["nodes"] < res[0]["nodes"]


def test_loader_rejects_bad_inputs(tmp_path):
    from hastyrenderer_gb300 import native
    bad = tmp_path / "renderJob.json"
    bad.write_text('{"settings": {}, "scene": "missing.json"}')
    with pytest.raises(native.HastyError) as e:
        host_trace(str(bad), np.zeros((1, 6), np.float32))
    assert e.value.code == -2
    (tmp_path / "s.json").write_text('{"camera": {"position": [0,0,0]}, "world": {"background_color": [0,0,0]}, '
                                     '"mesh": "m.obj"}')
    (tmp_path / "m.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    bad.write_text('{"settings": {}, "scene": "s.json"}')
    with pytest.raises(native.HastyError) as e:           # face without material (Scene.cpp:155-159)
        host_trace(str(bad), np.zeros((1, 6), np.float32))
    assert "material" in str(e.value)
