"""ctypes binding of the C ABI declared in include/hasty_gpu.h.

The library is built in-tree (``python -m hastyrenderer_gb300.build``) at
``hastyrenderer_gb300/lib/libhasty_gb300.so``. Loading fails loudly when it is
missing: there is no CPU fallback.
"""
from __future__ import annotations

import ctypes
import os
import re

# HASTY_LIB selects another build of the library (the bounds-checked one, in tests).
LIB_PATH = os.environ.get("HASTY_LIB") or os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib",
                                                        "libhasty_gb300.so")
HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "hasty_gpu.h")

HASTY_OK = 0
ERRORS = {-1: "HASTY_ERR_ARG", -2: "HASTY_ERR_LOAD", -3: "HASTY_ERR_CUDA", -4: "HASTY_ERR_MEMORY",
          -5: "HASTY_ERR_IO", -6: "HASTY_ERR_STOPPED", -7: "HASTY_ERR_MISSING"}
AOV_COLOR, AOV_NORMAL, AOV_ALBEDO = 0, 1, 2


class HastyError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class JobInfo(ctypes.Structure):
    _fields_ = [("width", ctypes.c_int32), ("height", ctypes.c_int32), ("num_samples", ctypes.c_int32),
                ("max_depth", ctypes.c_int32), ("roulette_start_depth", ctypes.c_int32), ("roulette_q", ctypes.c_float),
                ("use_mis", ctypes.c_int32), ("seed", ctypes.c_uint64), ("n_triangles", ctypes.c_int64),
                ("n_light_triangles", ctypes.c_int64), ("n_shapes", ctypes.c_int32), ("n_materials", ctypes.c_int32),
                ("env_is_texture", ctypes.c_int32), ("exposure", ctypes.c_float), ("samples_done", ctypes.c_int32),
                ("bvh_depth", ctypes.c_int32), ("bvh_build_ms", ctypes.c_double), ("device_bytes", ctypes.c_int64),
                ("bvh_tree_ms", ctypes.c_double), ("parse_ms", ctypes.c_double), ("upload_ms", ctypes.c_double),
                ("paths_in_flight", ctypes.c_int64), ("path_kernel", ctypes.c_int32), ("pad", ctypes.c_int32)]


class Stats(ctypes.Structure):
    _fields_ = [("rays", ctypes.c_uint64), ("shaded", ctypes.c_uint64), ("paths", ctypes.c_uint64),
                ("nan_samples", ctypes.c_uint64), ("media_overflow", ctypes.c_uint64), ("trial_cap", ctypes.c_uint64),
                ("kernel_ms", ctypes.c_double), ("trace_ms", ctypes.c_double), ("shade_ms", ctypes.c_double),
                ("trace_launches", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64), ("path_ms", ctypes.c_double),
                ("path_launches", ctypes.c_uint64), ("stack_overflow", ctypes.c_uint64)]


class BatchConfig(ctypes.Structure):
    _fields_ = [("paths_in_flight", ctypes.c_int64), ("regen_fraction", ctypes.c_float),
                ("max_iterations", ctypes.c_int32), ("mode", ctypes.c_int32), ("lanes", ctypes.c_int32),
                ("resolve_threads", ctypes.c_int32), ("sample_threads", ctypes.c_int32),
                ("trace_blocks_per_sm", ctypes.c_int32), ("pad", ctypes.c_int32)]


class BatchStats(ctypes.Structure):
    _fields_ = [("device_ms", ctypes.c_double), ("wall_ms", ctypes.c_double), ("samples", ctypes.c_uint64),
                ("rays", ctypes.c_uint64), ("shaded", ctypes.c_uint64), ("nan_samples", ctypes.c_uint64),
                ("saturated", ctypes.c_uint64), ("iterations", ctypes.c_uint64), ("paths_in_flight", ctypes.c_int64),
                ("engine_bytes", ctypes.c_int64), ("kernel_launches", ctypes.c_uint64),
                ("media_overflow", ctypes.c_uint64)]


class PmStats(ctypes.Structure):
    _fields_ = [("iterations", ctypes.c_int32), ("photons_emitted", ctypes.c_int64), ("photons_stored", ctypes.c_int64),
                ("cell_size", ctypes.c_float), ("device_ms", ctypes.c_double), ("host_ms", ctypes.c_double),
                ("media_overflow", ctypes.c_uint64), ("trial_cap", ctypes.c_uint64), ("photon_ms", ctypes.c_double),
                ("gather_ms", ctypes.c_double), ("cell_ms", ctypes.c_double), ("map_ms", ctypes.c_double)]


class ServerConfig(ctypes.Structure):
    _fields_ = [("paths_in_flight", ctypes.c_int64), ("lanes", ctypes.c_int32), ("max_resident_jobs", ctypes.c_int32),
                ("max_resident_scenes", ctypes.c_int32), ("loader_threads", ctypes.c_int32),
                ("memory_budget", ctypes.c_int64), ("quantum_samples", ctypes.c_int64), ("policy", ctypes.c_int32),
                ("resolve_threads", ctypes.c_int32), ("sample_threads", ctypes.c_int32),
                ("trace_blocks_per_sm", ctypes.c_int32)]


class ServerResult(ctypes.Structure):
    _fields_ = [("id", ctypes.c_int64), ("status", ctypes.c_int32), ("width", ctypes.c_int32),
                ("height", ctypes.c_int32), ("passes", ctypes.c_int32), ("samples", ctypes.c_uint64),
                ("submit_ms", ctypes.c_double), ("admit_ms", ctypes.c_double), ("finish_ms", ctypes.c_double),
                ("latency_ms", ctypes.c_double), ("error", ctypes.c_char * 160)]


class ServerStats(ctypes.Structure):
    _fields_ = [("submitted", ctypes.c_uint64), ("admitted", ctypes.c_uint64), ("completed", ctypes.c_uint64),
                ("failed", ctypes.c_uint64), ("samples", ctypes.c_uint64), ("rays", ctypes.c_uint64),
                ("shaded", ctypes.c_uint64), ("batches", ctypes.c_uint64), ("kernel_launches", ctypes.c_uint64),
                ("device_ms", ctypes.c_double), ("uptime_ms", ctypes.c_double), ("resident_bytes", ctypes.c_int64),
                ("peak_resident_bytes", ctypes.c_int64), ("engine_bytes", ctypes.c_int64),
                ("resident_jobs", ctypes.c_int32), ("resident_scenes", ctypes.c_int32), ("pending", ctypes.c_int32)]


def declared_symbols(header: str = HEADER) -> list[str]:
    """Function names declared in the C header."""
    text = open(header).read()
    return sorted(set(re.findall(r"^\s*int\s+(hasty_\w+)\s*\(", text, flags=re.M)))


_lib = None


def lib() -> ctypes.CDLL:
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"native library missing: {LIB_PATH} (run python -m hastyrenderer_gb300.build)")
    L = ctypes.CDLL(LIB_PATH)
    P, I, U64, I64, SZ = ctypes.c_void_p, ctypes.c_int, ctypes.c_uint64, ctypes.c_int64, ctypes.c_size_t
    sig = {
        "hasty_last_error": [ctypes.c_char_p, SZ],
        "hasty_version": [P, P],
        "hasty_ctx_create": [I, ctypes.c_uint32, P],
        "hasty_ctx_destroy": [P],
        "hasty_job_load": [P, ctypes.c_char_p, P],
        "hasty_jobs_load": [P, P, SZ, ctypes.c_int32, P],
        "hasty_job_destroy": [P],
        "hasty_job_info_get": [P, P],
        "hasty_job_set_seed": [P, U64],
        "hasty_job_reset": [P],
        "hasty_job_set_paths_in_flight": [P, I64],
        "hasty_job_render_passes": [P, I],
        "hasty_job_release_paths": [P],
        "hasty_job_sync": [P],
        "hasty_job_stop": [P],
        "hasty_job_stats_get": [P, P],
        "hasty_job_set_stage_timing": [P, I],
        "hasty_job_read": [P, I, P, SZ, SZ, P],
        "hasty_job_read_sums": [P, I, P, SZ, SZ, P],
        "hasty_job_write_outputs": [P, ctypes.c_char_p, I],
        "hasty_job_snapshot": [P, ctypes.c_uint32],
        "hasty_job_snapshot_query": [P, P],
        "hasty_job_snapshot_get": [P, I, P, P],
        "hasty_job_write_outputs_async": [P, ctypes.c_char_p, I],
        "hasty_job_outputs_wait": [P],
        "hasty_debug_intersect": [P, P, SZ, P, P, P, P],
        "hasty_debug_obj_digest": [ctypes.c_char_p, I, P, P, P],
        "hasty_debug_tri_ids": [P, P, P, SZ],
        "hasty_debug_host_trace": [ctypes.c_char_p, I, P, SZ, P, P, P, P, P],
        "hasty_debug_bsdf": [I, P, SZ, P, SZ, P],
        "hasty_debug_wide_emit_check": [I, ctypes.c_char_p, P, P],
        "hasty_batch_render": [P, P, P, SZ, P, P],
        "hasty_pm_render": [P, I],
        "hasty_pm_reset": [P],
        "hasty_pm_read": [P, I, P, SZ, SZ],
        "hasty_pm_read_radii": [P, P, SZ, SZ],
        "hasty_pm_stats_get": [P, P],
        "hasty_debug_pm_map": [P, P, P, P, P, P, P, P],
        "hasty_job_render_pass_static": [P, I, P],
        "hasty_debug_static_scratch": [P, P, P],
        "hasty_debug_pack": [P, P, P, SZ, I64, I64, P, SZ, P],
        "hasty_debug_bounds_status": [P],
        "hasty_server_start": [P, P, P],
        "hasty_server_submit": [P, ctypes.c_char_p, ctypes.c_int32, P, P],
        "hasty_server_poll": [P, P, SZ, P, ctypes.c_int32],
        "hasty_server_read": [P, ctypes.c_int64, I, P, SZ, SZ],
        "hasty_server_read_sums": [P, ctypes.c_int64, I, P, SZ, SZ],
        "hasty_server_release": [P, ctypes.c_int64],
        "hasty_server_stats_get": [P, P],
        "hasty_server_wait_idle": [P, ctypes.c_int32],
        "hasty_server_stop": [P],
    }
    for name, args in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = ctypes.c_int
    _lib = L
    return L


def check(rc: int) -> None:
    if rc != HASTY_OK:
        buf = ctypes.create_string_buffer(2048)
        lib().hasty_last_error(buf, 2048)
        raise HastyError(rc, buf.value.decode(errors="replace"))
