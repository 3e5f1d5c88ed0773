"""The packed-batch plan (hasty_debug_pack; no device needed): the schedule
hasty_batch_render and the server follow when they pack several jobs' passes
into shared batches. Every job's passes are planned once, in order; a batch
fits its slots and the chunk table, holds jobs of one kernel class, and
keeps the per-job cap; kernel classes take turns while several have passes
left."""
import ctypes

import numpy as np
import pytest

from hastyrenderer_gb300 import native

MAX_CHUNKS = 64   # chunks per batch (the kernel-parameter table)


def plan(npix, passes, cls, slots, job_samples=0):
    n = len(npix)
    a = lambda v: (ctypes.c_int32 * max(n, 1))(*v)   # noqa: E731
    cap = 1 << 16
    out = (ctypes.c_int32 * (4 * cap))()
    n_out = ctypes.c_size_t()
    native.check(native.lib().hasty_debug_pack(a(npix), a(passes), a(cls), n, slots, job_samples, out, cap,
                                               ctypes.byref(n_out)))
    assert n_out.value <= cap
    return np.frombuffer(out, dtype=np.int32, count=4 * n_out.value).reshape(-1, 4)


def check_plan(chunks, npix, passes, cls, slots, job_samples):
    n = len(npix)
    nxt = [0] * n
    for b in np.unique(chunks[:, 0]):
        rows = chunks[chunks[:, 0] == b]
        assert len(rows) <= MAX_CHUNKS
        assert sum(int(p) * npix[j] for _, j, _, p in rows) <= slots
        assert len({cls[j] for _, j, _, _ in rows}) == 1, "a batch mixes kernel classes"
        for _, j, first, p in rows:
            assert p >= 1 and first == nxt[j], "passes out of order or repeated"
            nxt[j] += p
            if job_samples:
                assert p <= max(1, job_samples // npix[j])
    assert nxt == list(passes), "every pass planned once"
    assert list(np.unique(chunks[:, 0])) == list(range(len(np.unique(chunks[:, 0]))))


@pytest.mark.parametrize("seed", range(8))
def test_random_mixes(seed):
    rng = np.random.default_rng(seed)
    n = int(rng.integers(1, 70))
    npix = [int(x) for x in rng.choice([128 * 128, 256 * 192, 512 * 512, 1024 * 768, 37], size=n)]
    passes = [int(x) for x in rng.integers(0, 300, size=n)]
    cls = [int(x) for x in rng.integers(0, 3, size=n)]
    slots = int(rng.choice([1 << 20, 1 << 22, 1 << 24]))
    job_samples = int(rng.choice([0, 1 << 16, 1 << 20]))
    chunks = plan(npix, passes, cls, slots, job_samples)
    check_plan(chunks, npix, passes, cls, slots, job_samples)


def test_classes_take_turns():
    # two classes with many passes each: consecutive batches alternate
    npix, passes, cls = [1000, 1000], [100, 100], [0, 1]
    chunks = plan(npix, passes, cls, slots=10_000)
    batch_cls = [cls[int(chunks[chunks[:, 0] == b][0, 1])] for b in np.unique(chunks[:, 0])]
    assert batch_cls[:6] == [0, 1, 0, 1, 0, 1]
    check_plan(chunks, npix, passes, cls, 10_000, 0)


def test_small_jobs_fill_a_batch():
    # one batch holds several small jobs' passes (up to the chunk-table size)
    npix, passes, cls = [100] * 10, [3] * 10, [0] * 10
    chunks = plan(npix, passes, cls, slots=100_000)
    assert set(chunks[:, 0]) == {0} and len(chunks) == 10


def test_bad_arguments():
    out = (ctypes.c_int32 * 4)()
    n_out = ctypes.c_size_t()
    one = (ctypes.c_int32 * 1)(1000)
    passes = (ctypes.c_int32 * 1)(1)
    bad_cls = (ctypes.c_int32 * 1)(3)
    assert native.lib().hasty_debug_pack(one, passes, bad_cls, 1, 10_000, 0, out, 1, ctypes.byref(n_out)) != 0
    ok_cls = (ctypes.c_int32 * 1)(0)
    assert native.lib().hasty_debug_pack(one, passes, ok_cls, 1, 10, 0, out, 1, ctypes.byref(n_out)) != 0   # frame > slots
