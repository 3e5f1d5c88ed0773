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


def test_cli_argument_errors(tmp_path):
    exe = os.path.join(os.path.dirname(native.LIB_PATH), "hasty_gpu_render")
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 1 and "usage" in r.stdout
    r = subprocess.run([exe, "job.json", str(tmp_path / "missing")], capture_output=True, text=True)
    assert r.returncode == 1 and "not a directory" in r.stdout
