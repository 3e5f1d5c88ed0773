"""The path kernel (one persistent thread per camera sample, path state in
an L2-sized slot pool) against the wavefront kernels: the same bounce code
and per-sample random streams, so every sum and statistic is bit-identical.
Contexts pick the kernel (HASTY_CTX_WAVEFRONT / HASTY_CTX_PATH_KERNEL); by
default every scene takes the wavefront (measured faster on GB300)."""
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["cornell", "field", "room", "room_nomis"]


def _path(name):
    return os.path.join(GOLDEN, "scenes", name, "renderJob.json")


def _sums(job):
    return [job.read_sums(a)[0] for a in (0, 1, 2)]


def _big_field(width=64, height=48):
    """The 1,024,002-triangle sphere field at a small frame."""
    from hastyrenderer_gb300 import scenes
    base = os.path.join(tempfile.gettempdir(), f"hasty_test_field800_{width}x{height}")
    path = os.path.join(base, "renderJob.json")
    if not os.path.exists(path):
        scenes.sphere_field(base, seed=0, n_spheres=800, subdiv=3, width=width, height=height, spp=4, max_depth=12)
    return path


@pytest.mark.parametrize("name", NAMES + ["big_field"])
def test_path_kernel_equals_wavefront(name):
    from hastyrenderer_gb300 import Context, RenderJob
    path = _big_field() if name == "big_field" else _path(name)
    wf = RenderJob(path, Context(0, Context.WAVEFRONT))
    pk = RenderJob(path, Context(0, Context.PATH_KERNEL))
    assert wf.info.path_kernel == 0 and pk.info.path_kernel == 1
    for n in (3, 2):      # two calls: the second continues the pass sequence
        wf.render_passes(n, sync=True)
        pk.render_passes(n, sync=True)
    for a, b in zip(_sums(pk), _sums(wf)):
        assert np.array_equal(a, b), name
    s_wf, s_pk = wf.stats(), pk.stats()
    for k in ("rays", "shaded", "paths", "nan_samples", "media_overflow", "trial_cap"):
        assert s_wf[k] == s_pk[k], (name, k, s_wf[k], s_pk[k])
    assert s_pk["path_launches"] >= 1 and s_wf["path_launches"] == 0


def test_default_context_is_the_wavefront():
    from hastyrenderer_gb300 import RenderJob
    assert RenderJob(_path("cornell")).info.path_kernel == 0
    assert RenderJob(_big_field()).info.path_kernel == 0


def test_packed_batch_on_the_path_kernel():
    """Packed batches run on the path kernel equal each job's single-job
    wavefront path."""
    from hastyrenderer_gb300 import Context, RenderJob, batch_render
    paths = [_path(n) for n in NAMES] + [_big_field(), _big_field(48, 32)]
    passes = [4, 3, 5, 2, 3, 4]
    pk, wf = Context(0, Context.PATH_KERNEL), Context(0, Context.WAVEFRONT)
    batched = [RenderJob(p, pk) for p in paths]
    assert {j.info.path_kernel for j in batched} == {1}
    batch_render(batched, passes, paths_in_flight=9000, lanes=3)
    for p, n, jb in zip(paths, passes, batched):
        plain = RenderJob(p, wf)
        plain.render_passes(n, sync=True)
        for a, b in zip(_sums(jb), _sums(plain)):
            assert np.array_equal(a, b), p


MIXED_CLASSES = r"""
import os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from hastyrenderer_gb300 import Context, RenderJob, batch_render
paths = sys.argv[2:]
passes = [4, 3, 5, 2, 3, 4][:len(paths)]
batched = [RenderJob(p) for p in paths]
assert {j.info.path_kernel for j in batched} == {0, 1}, [j.info.path_kernel for j in batched]
batch_render(batched, passes, paths_in_flight=9000, lanes=3)
wf = Context(0, Context.WAVEFRONT)
for p, n, jb in zip(paths, passes, batched):
    plain = RenderJob(p, wf)
    plain.render_passes(n, sync=True)
    for a in (0, 1, 2):
        assert np.array_equal(jb.read_sums(a)[0], plain.read_sums(a)[0]), p
print("mixed ok")
"""


def test_packed_batch_of_both_kernel_classes():
    """With the path kernel taking scenes up to 100k triangles
    (HASTY_PATH_KERNEL_TRIS, read once per process, so in a child process),
    one batch_render call over small and large scenes runs path-kernel and
    wavefront batches side by side; every job equals its single-job path."""
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    paths = [_path(n) for n in NAMES] + [_big_field(), _big_field(48, 32)]
    env = dict(os.environ, HASTY_PATH_KERNEL_TRIS="100000")
    r = subprocess.run([sys.executable, "-c", MIXED_CLASSES, root] + paths, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "mixed ok" in r.stdout, r.stdout + r.stderr
