"""Output surface on the GPU: the progressive read-back (hasty_job_snapshot*,
the reference viewer's computeEstimate loop, apps/PathTracingViewer.cpp:88-139),
the asynchronous output writer, and the headless CLI end to end
(apps/PathTracingViewer.cpp:17-175, apps/ViewerUtils.cpp:137-152). Snapshots
and files must equal hasty_job_read of the same pass count bit for bit."""
import os
import struct
import subprocess

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

AOVS = (0, 1, 2)
NAMES = ("output", "outputNormal", "outputAlbedo")


def read_exr(path):
    """Reader for the single-part, uncompressed FLOAT scanline files the
    library writes (channels in header order, one line per chunk)."""
    with open(path, "rb") as f:
        b = f.read()
    assert struct.unpack_from("<II", b, 0) == (20000630, 2)
    p, chans, box = 8, [], None
    while b[p] != 0:
        e = b.index(b"\0", p); name = b[p:e].decode(); p = e + 1
        e = b.index(b"\0", p); typ = b[p:e].decode(); p = e + 1
        (size,) = struct.unpack_from("<I", b, p); p += 4
        val = b[p:p + size]; p += size
        if name == "channels":
            q = 0
            while val[q] != 0:
                e = val.index(b"\0", q); chans.append(val[q:e].decode()); q = e + 1
                assert struct.unpack_from("<I", val, q)[0] == 2        # FLOAT
                q += 16
        elif name == "compression":
            assert val[0] == 0
        elif name == "dataWindow":
            box = struct.unpack_from("<iiii", val, 0)
        assert typ
    p += 1
    w, h = box[2] - box[0] + 1, box[3] - box[1] + 1
    offsets = struct.unpack_from("<%dQ" % h, b, p)
    img = np.empty((h, w, 3), np.float32)
    for y, off in enumerate(offsets):
        ly, n = struct.unpack_from("<iI", b, off)
        assert ly == y and n == w * 4 * len(chans)
        planes = np.frombuffer(b, np.float32, w * len(chans), off + 8).reshape(len(chans), w)
        for c, name in enumerate(chans):
            img[y, :, "RGB".index(name)] = planes[c]
    return img


@pytest.fixture(scope="module")
def cornell(tmp_path_factory):
    from hastyrenderer_gb300 import scenes
    d = tmp_path_factory.mktemp("cornell")
    return scenes.cornell_box(str(d), seed=3, width=256, height=192, spp=12)


def _job(path):
    from hastyrenderer_gb300 import RenderJob
    return RenderJob(path)


def test_snapshot_equals_read(cornell):
    job = _job(cornell)
    job.render_passes(4)
    job.snapshot(AOVS)
    snaps = [job.snapshot_get(a) for a in AOVS]
    assert job.snapshot_ready()
    for a, (img, n) in zip(AOVS, snaps):
        assert n == 4
        np.testing.assert_array_equal(img, job.compute_estimate(a))


def test_snapshot_while_rendering_continues(cornell):
    job = _job(cornell)
    job.render_passes(3)
    job.snapshot((0,))
    job.render_passes(5)              # enqueued before the snapshot is waited for
    s3, n3 = job.snapshot_get(0)
    job.snapshot((0, 2))
    job.render_passes(4)
    s8, n8 = job.snapshot_get(0)
    a8, _ = job.snapshot_get(2)
    assert (n3, n8) == (3, 8)
    ref = _job(cornell)
    ref.render_passes(3)
    np.testing.assert_array_equal(s3, ref.compute_estimate(0))
    ref.render_passes(5)
    np.testing.assert_array_equal(s8, ref.compute_estimate(0))
    np.testing.assert_array_equal(a8, ref.compute_estimate(2))
    np.testing.assert_array_equal(job.compute_estimate(0), (ref.render_passes(4), ref.compute_estimate(0))[1])


def test_snapshot_errors(cornell):
    from hastyrenderer_gb300.native import HastyError
    job = _job(cornell)
    with pytest.raises(HastyError):
        job.snapshot_get(0)               # none taken
    with pytest.raises(HastyError):
        job.snapshot(())                  # empty mask
    job.render_passes(1)
    job.snapshot((1,))
    with pytest.raises(HastyError):
        job.snapshot_get(0)               # colour not captured
    assert job.snapshot_get(1)[1] == 1


def test_async_outputs_equal_sync(cornell, tmp_path):
    a, b = tmp_path / "async", tmp_path / "sync"
    a.mkdir(); b.mkdir()
    job = _job(cornell)
    job.render_passes(6)
    job.write_outputs_async(str(a), write_pfm=True)
    job.render_passes(6)                  # renders while the files are written
    job.outputs_wait()
    ref = _job(cornell)
    ref.render_passes(6)
    ref.write_outputs(str(b), write_pfm=True)
    for name in NAMES:
        for ext in (".exr", ".pfm"):
            assert (a / (name + ext)).read_bytes() == (b / (name + ext)).read_bytes(), name + ext
    for aov, name in zip(AOVS, NAMES):
        np.testing.assert_array_equal(read_exr(str(a / (name + ".exr"))), ref.compute_estimate(aov))


def test_async_outputs_missing_directory(cornell, tmp_path):
    from hastyrenderer_gb300.native import HastyError
    job = _job(cornell)
    job.render_passes(1)
    with pytest.raises(HastyError) as e:
        job.write_outputs_async(str(tmp_path / "missing"))
    assert e.value.code == -5


@pytest.mark.parametrize("every", [0, 5])
def test_cli_end_to_end(cornell, tmp_path, every):
    from hastyrenderer_gb300 import native
    exe = os.path.join(os.path.dirname(native.LIB_PATH), "hasty_gpu_render")
    env = dict(os.environ)
    env.pop("HASTY_WRITE_EVERY", None)
    if every:
        env["HASTY_WRITE_EVERY"] = str(every)
    r = subprocess.run([exe, cornell, str(tmp_path)], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    ref = _job(cornell)
    ref.render_passes(ref.info.num_samples)
    for aov, name in zip(AOVS, NAMES):
        np.testing.assert_array_equal(read_exr(str(tmp_path / (name + ".exr"))), ref.compute_estimate(aov))


def test_job_info_load_times_and_paths(cornell):
    """hasty_job_info reports the load's parts and the paths-in-flight
    setting (whole passes, up to 16M paths); path buffers follow a change."""
    job = _job(cornell)
    i = job.info
    npix = i.width * i.height
    assert i.parse_ms > 0 and i.upload_ms >= 0 and i.bvh_build_ms > 0
    assert i.paths_in_flight % npix == 0 and npix <= i.paths_in_flight <= max(npix, 1 << 24)
    job.set_paths_in_flight(3 * npix + 5)
    assert job.info.paths_in_flight == 3 * npix
    job.render_passes(7)
    ref = _job(cornell)
    ref.render_passes(7)
    np.testing.assert_array_equal(job.compute_estimate(0), ref.compute_estimate(0))
