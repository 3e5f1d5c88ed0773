"""The bounds-checked build (HASTY_DEBUG_BOUNDS: every queue entry, ray id,
BVH node, leaf triangle, hit triangle, material, texture, light triangle and
medium-stack block the kernels read through is checked on the device; a bad
index sets a status bit and the access is skipped, never a trap) on the
golden scenes through every executor: no bit set, and the sums equal the
regular build's bit for bit (the checks change nothing else). It stands in
for a memory checker, which this pool does not run. The checked library is
built here if missing and loaded in a child process (HASTY_LIB)."""
import os
import subprocess
import sys

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
NAMES = ["cornell", "field", "room", "room_nomis", "nested"]
BOUNDS_LIB = os.path.join(ROOT, "hastyrenderer_gb300", "lib", "bounds", "libhasty_gb300.so")

RENDER = r"""
import os, sys
import numpy as np
sys.path.insert(0, sys.argv[1])
from hastyrenderer_gb300 import Context, RenderJob, batch_render, native
out, names = sys.argv[2], sys.argv[3:]
paths = [os.path.join(sys.argv[1], "tests", "golden", "scenes", n, "renderJob.json") for n in names]
res = {}
for n, p in zip(names, paths):
    j = RenderJob(p)
    j.render_passes(4, sync=True)
    res["plain_" + n] = j.read_sums()[0]
    k = RenderJob(p, Context(0, Context.PATH_KERNEL))
    k.render_passes(2, sync=True)
    res["path_" + n] = k.read_sums()[0]
jobs = [RenderJob(p) for p in paths]
batch_render(jobs, [3] * len(jobs), paths_in_flight=2500, lanes=3)
for n, j in zip(names, jobs):
    res["packed_" + n] = j.read_sums()[0]
jobs = [RenderJob(p) for p in paths]
batch_render(jobs, [2] * len(jobs), mode=1, paths_in_flight=4096)
for n, j in zip(names, jobs):
    res["regen_" + n] = j.read_sums()[0]
pm = RenderJob(paths[names.index("room")])
pm.pm_render(1)
res["photon_room"] = pm.pm_read(0)
if native.LIB_PATH.endswith(os.path.join("bounds", "libhasty_gb300.so")):
    import ctypes
    flags = ctypes.c_uint32(0xFFFFFFFF)
    native.check(native.lib().hasty_debug_bounds_status(ctypes.byref(flags)))
    res["bounds_flags"] = np.array([flags.value], np.uint32)
np.savez(out, **res)
print("rendered")
"""


def _render(tmp_path, lib):
    out = str(tmp_path / ("checked.npz" if lib else "regular.npz"))
    env = dict(os.environ)
    if lib:
        env["HASTY_LIB"] = lib
    else:
        env.pop("HASTY_LIB", None)
    r = subprocess.run([sys.executable, "-c", RENDER, ROOT, out] + NAMES, env=env, capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0 and "rendered" in r.stdout, r.stdout + r.stderr
    return dict(np.load(out))


def test_bounds_checked_build_on_goldens(tmp_path):
    if not os.path.exists(BOUNDS_LIB):
        b = subprocess.run([sys.executable, "-m", "hastyrenderer_gb300.build", "--debug-bounds"], cwd=ROOT,
                           capture_output=True, text=True, timeout=900)
        assert b.returncode == 0, b.stdout + b.stderr
    checked = _render(tmp_path, BOUNDS_LIB)
    regular = _render(tmp_path, None)
    assert int(checked["bounds_flags"][0]) == 0, hex(int(checked["bounds_flags"][0]))
    for key, val in regular.items():
        assert np.array_equal(checked[key], val), key
