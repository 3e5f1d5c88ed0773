"""hasty_job_render_pass_static: one pass rendered with scratch from a static
device array (no device allocation in the call), compared with the regular
hasty_job_render_passes path on the same job, seed and pass indices.

Tolerance: both paths run the same kernels on the same sample streams and add
one FP64 sample per pixel to zero, so the sums are expected to be equal; the
test allows rtol 1e-9 / atol 1e-12 per value.

Named to run last: the static array is shared by every call in the process,
so this file also checks that calls made after the rest of the suite start
from a clean state.
"""
import ctypes
import os
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
RTOL, ATOL = 1e-9, 1e-12
MAX_PIXELS = 16384


def _job(path):
    from hastyrenderer_gb300 import RenderJob
    return RenderJob(path)


def _scene(name):
    return os.path.join(GOLDEN, "scenes", name, "renderJob.json")


def _static_pass(job, pass_index):
    """Calls the entry point through the C ABI into a NaN-filled device buffer."""
    import torch
    from hastyrenderer_gb300 import native
    n = job.width * job.height * 3
    buf = torch.full((n,), float("nan"), dtype=torch.float64, device="cuda")
    torch.cuda.synchronize()
    rc = native.lib().hasty_job_render_pass_static(job._h, int(pass_index), ctypes.c_void_p(buf.data_ptr()))
    native.check(rc)
    job.sync()
    return buf.cpu().numpy().reshape(job.height, job.width, 3)


def _regular_sums(path, n_passes):
    ref = _job(path)
    ref.render_passes(n_passes, sync=True)
    sums, done = ref.read_sums(0)
    assert done == n_passes
    return sums


@pytest.mark.parametrize("name", ["cornell", "field", "room"])
def test_two_calls_match_regular_path(name):
    path = _scene(name)
    job = _job(path)
    s0 = _static_pass(job, 0)
    s1 = _static_pass(job, 1)
    r1 = _regular_sums(path, 1)
    r2 = _regular_sums(path, 2)
    assert np.isfinite(s0).all() and np.isfinite(s1).all()
    np.testing.assert_allclose(s0, r1, rtol=RTOL, atol=ATOL)
    np.testing.assert_allclose(s0 + s1, r2, rtol=RTOL, atol=ATOL)
    # the job's own accumulators are untouched
    assert job.read_sums(0)[1] == 0
    assert not job.read_sums(0)[0].any()
    # a repeated call sees none of the previous calls' scratch contents
    np.testing.assert_array_equal(_static_pass(job, 0), s0)


def test_largest_frame_and_rejection():
    from hastyrenderer_gb300 import native, scenes
    with tempfile.TemporaryDirectory() as d:
        ok = os.path.join(d, "max")
        scenes.cornell_box(ok, seed=3, width=128, height=MAX_PIXELS // 128, spp=1)
        path = os.path.join(ok, "renderJob.json")
        job = _job(path)
        a = _static_pass(job, 5)
        b = _static_pass(job, 5)
        ref = _job(path)
        ref.render_passes(6, sync=True)
        r5 = ref.read_sums(0)[0]
        ref5 = _job(path)
        ref5.render_passes(5, sync=True)
        r4 = ref5.read_sums(0)[0]
        np.testing.assert_array_equal(a, b)
        np.testing.assert_allclose(r4 + a, r5, rtol=RTOL, atol=ATOL)

        big = os.path.join(d, "big")
        scenes.cornell_box(big, seed=3, width=129, height=128, spp=1)
        jb = _job(os.path.join(big, "renderJob.json"))
        import torch
        buf = torch.zeros(129 * 128 * 3, dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        rc = native.lib().hasty_job_render_pass_static(jb._h, 0, ctypes.c_void_p(buf.data_ptr()))
        assert rc == -1   # HASTY_ERR_ARG
        with pytest.raises(native.HastyError, match="static scratch limit"):
            native.check(rc)
        jb.sync()
        assert not buf.any().item()   # rejected before anything was launched
