"""GPU binned-SAH BVH builder: trees built on the device answer every ray
exactly like trees built on the host (closest hit is tree-independent), for
both layouts, on the golden scenes and the 1.02M-triangle sphere field."""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def _rays(job_path, n, seed):
    """Seeded rays from points in the scene's vertex bounds, random directions."""
    d0 = os.path.dirname(job_path)
    obj = [f for f in os.listdir(d0) if f.endswith(".obj")][0]
    v = np.array([[float(x) for x in ln.split()[1:4]] for ln in open(os.path.join(d0, obj)) if ln.startswith("v ")])
    lo, hi = v.min(0), v.max(0)
    rng = np.random.default_rng(seed)
    o = rng.uniform(lo, hi, (n, 3))
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return np.concatenate([o, d], 1).astype(np.float32)


def _hits(path, flags, rays):
    from hastyrenderer_gb300 import Context, RenderJob
    ctx = Context(0, flags)
    job = RenderJob(path, ctx)
    tri, t, u, v = job.intersect(rays)
    info = job.info
    job.close()
    return tri, t, u, v, info


@pytest.mark.parametrize("name", ["cornell", "field", "room"])
@pytest.mark.parametrize("binary", [False, True])
def test_device_tree_equals_host_tree(name, binary):
    from hastyrenderer_gb300 import Context
    path = os.path.join(GOLDEN, "scenes", name, "renderJob.json")
    rays = _rays(path, 20000, 3)
    base = Context.BINARY_BVH if binary else 0
    g = _hits(path, base, rays)
    h = _hits(path, base | Context.HOST_BVH, rays)
    for a, b in zip(g[:4], h[:4]):
        assert np.array_equal(a, b)
    assert (g[0] >= 0).mean() > 0.05


def _sphere_field_800():
    """The 1,024,002-triangle sphere field (800 icospheres), generated once."""
    from hastyrenderer_gb300 import scenes
    base = os.path.join(tempfile.gettempdir(), "hasty_test_sphere_field_800")
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.sphere_field(base, seed=0, n_spheres=800, subdiv=3, width=1920, height=1080, spp=256, max_depth=12)
    return path


def test_device_tree_full_size():
    """1,024,002 triangles: identical hits on random rays; the device build
    is the default and reports its time."""
    from hastyrenderer_gb300 import Context
    path = _sphere_field_800()
    rng = np.random.default_rng(11)
    o = rng.uniform([-10, 0, -10], [10, 20, 10], (200000, 3))
    d = rng.normal(size=(200000, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    rays = np.concatenate([o, d], 1).astype(np.float32)
    g = _hits(path, 0, rays)
    h = _hits(path, Context.HOST_BVH, rays)
    for a, b in zip(g[:4], h[:4]):
        assert np.array_equal(a, b)
    print(f"wide BVH build: device {g[4].bvh_build_ms:.0f} ms, host {h[4].bvh_build_ms:.0f} ms; "
          f"depth {g[4].bvh_depth} / {h[4].bvh_depth}")
    assert g[4].bvh_depth <= 30


@pytest.mark.parametrize("name", ["cornell", "field", "room", "full"])
def test_device_layout_equals_host_layout(name):
    """The compressed 8-wide layout written on the device is byte-identical
    to the host writer's for the same device-built tree, and two device
    builds are identical."""
    import ctypes
    from hastyrenderer_gb300 import native
    if name == "full":
        path = _sphere_field_800()
    else:
        path = os.path.join(GOLDEN, "scenes", name, "renderJob.json")
    info = (ctypes.c_int64 * 8)()
    same = ctypes.c_int32()
    native.check(native.lib().hasty_debug_wide_emit_check(0, path.encode(), info, ctypes.byref(same)))
    assert info[0] > 0
    assert same.value == 1, list(info)
    assert info[7] == 1, list(info)
