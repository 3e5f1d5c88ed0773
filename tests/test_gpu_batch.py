"""Batching (hasty_batch_render), both modes.

Packed batches run the single-job path's kernels over chunks of several jobs
and add each pass to the job's FP64 sums in pass order, so a job's sums are
bit-identical to hasty_job_render_passes of the same passes, alone or in any
mix, for any batch size and lane count. The regeneration engine sums in
int64 fixed point: bit-identical alone or mixed, equal to the FP64 path to
fixed-point resolution."""
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


@pytest.mark.parametrize("mode", [0, 1], ids=["packed", "regen"])
def test_alone_equals_mixed(mode):
    """Each job's image is bit-identical rendered alone or batched with others."""
    from hastyrenderer_gb300.api import batch_render
    passes = [3, 5, 2, 4]
    mixed = [_job(n) for n in NAMES]
    st = batch_render(mixed, passes, mode=mode)
    assert st["samples"] == sum(p * j.width * j.height for p, j in zip(passes, mixed))
    for name, p, jm in zip(NAMES, passes, mixed):
        alone = _job(name)
        batch_render([alone], [p], mode=mode)
        for a, b in zip(_sums(jm), _sums(alone)):
            assert np.array_equal(a, b), name
        assert jm.read_sums()[1] == p


@pytest.mark.parametrize("lanes,paths,shapes", [(2, 0, (0, 0, 0)), (1, 3000, (128, 256, 4)), (2, 2500, (0, 0, 0)),
                                                (3, 4000, (256, 256, 6)), (4, 1100, (128, 512, 0))])
def test_packed_equals_single_job_path(lanes, paths, shapes):
    """Packed batches (small lanes force many batches, chunks split across
    batches and several jobs per batch; the tuner's block shapes) give
    exactly the single-job path's sums, a second call continuing the pass
    sequence."""
    from hastyrenderer_gb300.api import batch_render
    passes = [5, 7, 3, 6]
    packed = [_job(n) for n in NAMES]
    kw = dict(paths_in_flight=paths, lanes=lanes, resolve_threads=shapes[0], sample_threads=shapes[1],
              trace_blocks_per_sm=shapes[2])
    st = batch_render(packed, passes, **kw)
    batch_render(packed, [2, 1, 3, 2], **kw)
    assert st["samples"] == sum(p * j.width * j.height for p, j in zip(passes, packed))
    if paths:
        assert st["iterations"] >= st["samples"] // paths     # batches
    for name, p, p2, jb in zip(NAMES, passes, [2, 1, 3, 2], packed):
        plain = _job(name)
        plain.render_passes(p, sync=True)
        plain.render_passes(p2, sync=True)
        assert jb.read_sums()[1] == p + p2
        for a, b in zip(_sums(jb), _sums(plain)):
            assert np.array_equal(a, b), (name, lanes, paths)


def test_regen_matches_single_job_path():
    """Regeneration engine against hasty_job_render_passes: the same streams;
    sums agree to fixed-point resolution (2^-32 per sample), AOVs too."""
    from hastyrenderer_gb300.api import batch_render
    for name in NAMES:
        jb, jp = _job(name), _job(name)
        batch_render([jb], [4], mode=1)
        jp.render_passes(4, sync=True)
        for a, b in zip(_sums(jb), _sums(jp)):
            np.testing.assert_allclose(a, b, rtol=1e-6, atol=4 * 2.0 ** -32 * 4)


def test_small_pool_regeneration():
    """A pool far smaller than the work forces thousands of refills; the
    result is still bit-identical to the default pool."""
    from hastyrenderer_gb300.api import batch_render
    a, b = _job("field"), _job("field")
    st_a = batch_render([a], [8], mode=1)
    st = batch_render([b], [8], paths_in_flight=700, regen_fraction=1.0, mode=1)
    # 4608 samples through 700 slots: several refills, so more iterations
    # than one wave of max_depth bounces needs
    assert st["samples"] == st_a["samples"] == 8 * 24 * 24
    assert st["iterations"] > st_a["iterations"]
    assert st["iterations"] > 12
    for x, y in zip(_sums(a), _sums(b)):
        assert np.array_equal(x, y)


def test_regen_iteration_bound_then_recovers():
    """The engine's device-side loop guard: a batch that needs more
    iterations than max_iterations stops with HASTY_ERR_CUDA ("iteration
    bound") instead of running on, and the context stays usable: the next
    batch on it renders normally."""
    from hastyrenderer_gb300 import HastyError
    from hastyrenderer_gb300.api import batch_render
    j = _job("cornell")
    with pytest.raises(HastyError) as e:
        batch_render([j], [4], max_iterations=3, mode=1)
    assert e.value.code == -3 and "iteration bound" in str(e.value)
    ok, ref = _job("cornell"), _job("cornell")
    st = batch_render([ok], [4], mode=1)
    assert st["samples"] == 4 * 32 * 32
    batch_render([ref], [4], mode=1)
    for x, y in zip(_sums(ok), _sums(ref)):
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


def test_jobs_loaded_together_equal_loaded_alone(tmp_path):
    """hasty_jobs_load (several host threads) gives jobs whose renders equal
    those of jobs loaded one by one; a missing file fails the whole call with
    HASTY_ERR_LOAD and returns no job."""
    from hastyrenderer_gb300 import HastyError, load_jobs
    paths = [os.path.join(GOLDEN, "scenes", n, "renderJob.json") for n in NAMES + NAMES]
    together = load_jobs(paths, threads=4)
    assert len(together) == len(paths)
    for p, jt in zip(paths, together):
        alone = _job(os.path.basename(os.path.dirname(p)))
        assert (jt.width, jt.height, jt.info.n_triangles) == (alone.width, alone.height, alone.info.n_triangles)
        jt.render_passes(2, sync=True)
        alone.render_passes(2, sync=True)
        for a, b in zip(_sums(jt), _sums(alone)):
            assert np.array_equal(a, b), p
        jt.close()
        alone.close()
    with pytest.raises(HastyError) as err:
        load_jobs(paths[:2] + [str(tmp_path / "missing" / "renderJob.json")] + paths[2:3], threads=2)
    assert err.value.code == -2, err.value   # HASTY_ERR_LOAD
