"""Multi-job engine (batching): results independent of the mix, equal to the
single-job path, robust to heavy slot regeneration."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
NAMES = ["cornell", "field", "room", "room_nomis"]


def _job(name):
    from hastyrenderer_gb300 import RenderJob
    return RenderJob(os.path.join(GOLDEN, "scenes", name, "renderJob.json"))


def _sums(job):
    return [job.read_sums(a)[0] for a in (0, 1, 2)]


def test_alone_equals_mixed():
    """Each job's image is bit-identical rendered alone or batched with others."""
    from hastyrenderer_gb300.api import batch_render
    passes = [3, 5, 2, 4]
    mixed = [_job(n) for n in NAMES]
    st = batch_render(mixed, passes)
    assert st["samples"] == sum(p * j.width * j.height for p, j in zip(passes, mixed))
    for name, p, jm in zip(NAMES, passes, mixed):
        alone = _job(name)
        batch_render([alone], [p])
        for a, b in zip(_sums(jm), _sums(alone)):
            assert np.array_equal(a, b), name
        assert jm.read_sums()[1] == p


def test_batch_matches_single_job_path():
    """Same streams as hasty_job_render_passes: sums agree to fixed-point
    resolution (2^-32 per sample), AOVs too."""
    from hastyrenderer_gb300.api import batch_render
    for name in NAMES:
        jb, jp = _job(name), _job(name)
        batch_render([jb], [4])
        jp.render_passes(4, sync=True)
        for a, b in zip(_sums(jb), _sums(jp)):
            close = np.isclose(a, b, rtol=1e-6, atol=1e-8)
            assert close.mean() >= 0.999, (name, close.mean())


def test_small_pool_regeneration():
    """A pool far smaller than the work forces thousands of refills; the
    result is still bit-identical to the default pool."""
    from hastyrenderer_gb300.api import batch_render
    a, b = _job("field"), _job("field")
    st_a = batch_render([a], [8])
    st = batch_render([b], [8], paths_in_flight=700, regen_fraction=1.0)
    # 4608 samples through 700 slots: several refills, so more iterations
    # than one wave of max_depth bounces needs
    assert st["samples"] == st_a["samples"] == 8 * 24 * 24
    assert st["iterations"] > st_a["iterations"]
    assert st["iterations"] > 12
    for x, y in zip(_sums(a), _sums(b)):
        assert np.array_equal(x, y)


def test_release_paths_between_renders():
    """Freeing the path state between renders changes nothing in the result."""
    a, b = _job("room"), _job("room")
    a.render_passes(3, sync=True)
    b.render_passes(1, sync=True)
    b.release_paths()
    b.render_passes(2, sync=True)
    for x, y in zip(_sums(a), _sums(b)):
        assert np.array_equal(x, y)
