"""Extensions beyond the reference's job surface, checked against the CPU
oracle (which implements the same extensions): RGBA8 (PAM) textures kept as
bytes on the device, and Cauchy dispersion bands."""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _render(path, passes):
    from hastyrenderer_gb300 import RenderJob
    job = RenderJob(path)
    job.render_passes(passes, sync=True)
    out = [job.read_sums(a)[0] for a in (0, 1, 2)]
    job.close()
    return out


def test_rgba8_textures_equal_float_textures(tmp_path):
    """8-bit textures (bytes + per-texture value table) give exactly the
    texel values of the same maps loaded as floats, so the images match bit
    for bit."""
    from hastyrenderer_gb300 import scenes
    a = scenes.textured_room(str(tmp_path / "ppm"), seed=4, width=48, height=32)
    b = scenes.textured_room(str(tmp_path / "pam"), seed=4, width=48, height=32, rgba8=True)
    for x, y in zip(_render(a, 4), _render(b, 4)):
        assert np.array_equal(x, y)


@pytest.mark.parametrize("rgba8,dispersion", [(True, None), (False, {"model": "cauchy", "b": 0.0042}),
                                             (True, {"model": "cauchy", "b": 0.0042, "wavelengths": [0.7, 0.55, 0.4]})])
def test_extensions_match_oracle(tmp_path, rgba8, dispersion):
    """Pass 0 camera samples on the GPU equal the CPU oracle's (1e-3 relative)."""
    from hastyrenderer_gb300 import RenderJob, scenes
    from oracle.oracle import Oracle
    path = scenes.textured_room(str(tmp_path / "room"), seed=9, width=48, height=32, rgba8=rgba8, dispersion=dispersion)
    job = RenderJob(path)
    job.render_passes(1, sync=True)
    gpu, n = job.read_sums()
    job.close()
    ora = Oracle(path)
    cpu, _, _ = ora.render_samples(0, 0, 0, 48, 32)
    ora.close()
    cpu = np.where(np.isnan(cpu).any(-1, keepdims=True), 0.0, cpu)
    close = np.all(np.abs(gpu - cpu) <= 1e-3 * np.maximum(1.0, np.abs(cpu)), axis=-1)
    assert n == 1 and close.mean() >= 0.97, close.mean()


def test_cauchy_changes_the_glass(tmp_path):
    """The Cauchy bands differ from the reference's ratios, and the image
    differs where the dispersive glass is seen."""
    from hastyrenderer_gb300 import scenes
    a = scenes.textured_room(str(tmp_path / "ratio"), seed=9, width=48, height=32)
    b = scenes.textured_room(str(tmp_path / "cauchy"), seed=9, width=48, height=32,
                             dispersion={"model": "cauchy", "b": 0.05})
    ca, cb = _render(a, 8)[0], _render(b, 8)[0]
    assert not np.array_equal(ca, cb)
