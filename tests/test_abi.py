"""The C-ABI library loads, exports every entry point include/hasty_gpu.h
declares, and reports errors without a device; no compute is attempted."""
import ctypes
import os
import subprocess

import pytest

from hastyrenderer_gb300 import native


def test_header_declares_the_boundary():
    syms = native.declared_symbols()
    for s in ("hasty_ctx_create", "hasty_job_load", "hasty_job_render_passes", "hasty_job_read",
              "hasty_job_write_outputs", "hasty_debug_intersect", "hasty_debug_bsdf", "hasty_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    lib = native.lib()
    missing = [s for s in native.declared_symbols() if not hasattr(lib, s)]
    assert not missing, missing
    out = subprocess.run(["nm", "-D", "--defined-only", native.LIB_PATH], capture_output=True, text=True).stdout
    exported = {ln.split()[-1] for ln in out.splitlines() if ln.strip()}
    assert set(native.declared_symbols()) <= exported


def test_errors_are_status_codes():
    lib = native.lib()
    assert lib.hasty_job_render_passes(None, 1) == -1          # HASTY_ERR_ARG, no exception
    buf = ctypes.create_string_buffer(256)
    assert lib.hasty_last_error(buf, 256) == 0
    assert b"null" in buf.value
    assert lib.hasty_job_stop(None) == -1
    assert lib.hasty_debug_bsdf(7, None, 0, None, 0, None) == -1
    # progressive read-back entry points
    assert lib.hasty_job_snapshot(None, 1) == -1
    assert lib.hasty_job_snapshot_query(None, None) == -1
    assert lib.hasty_job_snapshot_get(None, 0, None, None) == -1
    assert lib.hasty_job_write_outputs_async(None, b".", 0) == -1
    assert lib.hasty_job_outputs_wait(None) == -1
    # several jobs at once: a null context or path list is an argument error
    out = (ctypes.c_void_p * 2)()
    paths = (ctypes.c_char_p * 2)(b"a/renderJob.json", b"b/renderJob.json")
    assert lib.hasty_jobs_load(None, paths, 2, 0, out) == -1
    assert lib.hasty_debug_pack(None, None, None, 1, 10, 0, None, 0, None) == -1


def test_static_scratch_holds_its_largest_frame():
    """The no-allocation entry point's static array holds the path state and
    sums of the largest frame it accepts, carved exactly as a call carves it
    (the same sizes and 256-byte alignment as every path pool)."""
    lib = native.lib()
    mx, need, cap = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_int64()
    assert lib.hasty_debug_static_scratch(ctypes.byref(mx), ctypes.byref(need), ctypes.byref(cap)) == 0
    assert mx.value >= 128 * 128
    assert 0 < need.value <= cap.value, (need.value, cap.value)
    assert lib.hasty_debug_static_scratch(None, None, None) == -1


def test_bounds_status_only_in_the_checked_build():
    """The regular library answers the bounds-status query with
    HASTY_ERR_MISSING (the checks are compiled into the checked build only)."""
    lib = native.lib()
    flags = ctypes.c_uint32(0)
    if native.LIB_PATH.endswith(os.path.join("bounds", "libhasty_gb300.so")):
        pytest.skip("the bounds-checked library is loaded")
    assert lib.hasty_debug_bounds_status(ctypes.byref(flags)) == -7


def test_cli_argument_errors(tmp_path):
    exe = os.path.join(os.path.dirname(native.LIB_PATH), "hasty_gpu_render")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stdout
    r = subprocess.run([exe, "job.json", str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 1 and "not a directory" in r.stdout


def _obj_digest(path, chunks):
    lib = native.lib()
    d, nt, ns = ctypes.c_uint64(), ctypes.c_int64(), ctypes.c_int64()
    assert lib.hasty_debug_obj_digest(str(path).encode(), chunks, ctypes.byref(d), ctypes.byref(nt), ctypes.byref(ns)) == 0
    return d.value, nt.value, ns.value


def _edge_obj(tmp_path):
    """An OBJ with the reader's edge cases: polygons of 2 to 6 corners (fans,
    quads split along the shorter diagonal, degenerate faces skipped),
    negative and partial indices, o/g cuts including empty shapes, usemtl of
    unknown names, a second mtllib mid-file, smoothing groups and 'off'."""
    import random
    rnd = random.Random(7)
    lines = ["mtllib a.mtl", "o first", "usemtl red"]
    nv = 0
    faces = 0
    for i in range(6000):
        r = rnd.random()
        if r < 0.05:
            lines.append(rnd.choice(["o obj%d" % i, "g g%d" % i, "usemtl red", "usemtl blue", "usemtl nope",
                                     "s %d" % rnd.randint(0, 3), "s off", "mtllib b.mtl", "# comment", "o", "g a b"]))
        elif r < 0.4 or nv < 3:
            for _ in range(rnd.randint(1, 3)):
                lines.append("v %g %g %g" % tuple(rnd.uniform(-5, 5) for _ in range(3)))
                nv += 1
        else:
            n = rnd.choice([3, 3, 3, 4, 4, 5, 6, 2])
            idx = [rnd.randint(1, nv) if rnd.random() < 0.8 else -rnd.randint(1, nv) for _ in range(n)]
            form = rnd.choice(["%d", "%d/1", "%d//2", "%d/2/1"])
            lines.append("f " + " ".join(form % x for x in idx))
            faces += max(0, n - 2)
    lines = lines[:3] + ["vt 0.5 0.5", "vt 0.1 0.9", "vn 0 1 0", "vn 1 0 0"] + lines[3:]
    (tmp_path / "a.mtl").write_text("newmtl red\nKd 1 0 0\nnewmtl blue\nKd 0 0 1\n")
    (tmp_path / "b.mtl").write_text("newmtl green\nKd 0 1 0\n")
    p = tmp_path / "edge.obj"
    p.write_text("\n".join(lines) + "\n")
    return p, faces


def test_obj_reader_independent_of_chunking(tmp_path):
    """The mesh reader parses a file's lines in chunks on all host threads and
    assembles triangles per chunk at offsets from a pass over the directives;
    the triangles (corners, materials, smoothing groups, shapes) must be the
    ones a single pass gives, for any number of chunks."""
    p, tris = _edge_obj(tmp_path)
    ref = _obj_digest(p, 1)
    assert ref[1] == tris and ref[2] > 10
    for chunks in (2, 3, 5, 8, 13, 16, 31, 64, 0):
        assert _obj_digest(p, chunks) == ref, chunks
    golden = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "scenes")
    for name in ("cornell", "field", "room"):
        q = os.path.join(golden, name, "scene.obj")
        one = _obj_digest(q, 1)
        assert all(_obj_digest(q, c) == one for c in (2, 7, 16))
