"""Python mirror of the reference's render-job interface over the C ABI.

Names follow the reference: ``RenderJob.loadJSON`` (core/src/RenderJob.cpp:21-28),
``render_passes`` for the renderThread pass loop (core/src/PathTracing.cpp:98-160),
``compute_estimate`` for computeEstimate (apps/ViewerUtils.cpp:95-121),
``write_outputs`` for postProcessAndSaveToDisk without the denoiser
(apps/ViewerUtils.cpp:137-152). Load errors raise ``HastyError`` with code
HASTY_ERR_LOAD, the counterpart of the reference's loader exceptions.
"""
from __future__ import annotations

import ctypes

import numpy as np

from . import native
from .native import AOV_ALBEDO, AOV_COLOR, AOV_NORMAL, HastyError, check

__all__ = ["Context", "RenderJob", "load_jobs", "debug_bsdf", "AOV_COLOR", "AOV_NORMAL", "AOV_ALBEDO", "HastyError"]


class Context:
    """One CUDA device."""

    BINARY_BVH = 1   # HASTY_CTX_BINARY_BVH
    HOST_BVH = 2     # HASTY_CTX_HOST_BVH: build the BVH on the host instead of the GPU
    WAVEFRONT = 4    # HASTY_CTX_WAVEFRONT: never the path kernel
    PATH_KERNEL = 8  # HASTY_CTX_PATH_KERNEL: the path kernel for every scene

    def __init__(self, device: int = 0, flags: int = 0):
        self._h = ctypes.c_void_p()
        check(native.lib().hasty_ctx_create(device, int(flags), ctypes.byref(self._h)))

    def close(self):
        if self._h:
            native.lib().hasty_ctx_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def load_jobs(paths, ctx: Context | None = None, threads: int = 0) -> list:
    """Loads several render jobs at once (hasty_jobs_load: parse, BVH build
    and upload of different jobs overlap on `threads` host threads, 0: all).
    Returns one RenderJob per path, in order; raises on the first failure
    (then no job stays loaded)."""
    ctx = ctx or default_context()
    n = len(paths)
    enc = [p.encode() for p in paths]
    arr = (ctypes.c_char_p * max(n, 1))(*enc)
    handles = (ctypes.c_void_p * max(n, 1))()
    check(native.lib().hasty_jobs_load(ctx._h, arr, n, int(threads), handles))
    jobs = []
    for i in range(n):
        j = RenderJob(None, ctx)
        j._h = ctypes.c_void_p(handles[i])
        jobs.append(j)
    return jobs


class RenderJob:
    """A render job resident on the device (scene, BVH, accumulators)."""

    def __init__(self, path: str | None = None, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self._h = ctypes.c_void_p()
        if path is not None:
            self.loadJSON(path)

    def loadJSON(self, path: str) -> None:
        if self._h:
            self.close()
        check(native.lib().hasty_job_load(self.ctx._h, path.encode(), ctypes.byref(self._h)))

    def close(self) -> None:
        if self._h:
            native.lib().hasty_job_destroy(self._h)
            self._h = ctypes.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def info(self) -> native.JobInfo:
        out = native.JobInfo()
        check(native.lib().hasty_job_info_get(self._h, ctypes.byref(out)))
        return out

    @property
    def width(self) -> int:
        return self.info.width

    @property
    def height(self) -> int:
        return self.info.height

    def set_seed(self, seed: int) -> None:
        check(native.lib().hasty_job_set_seed(self._h, ctypes.c_uint64(seed)))

    def reset(self) -> None:
        check(native.lib().hasty_job_reset(self._h))

    def set_paths_in_flight(self, n: int) -> None:
        check(native.lib().hasty_job_set_paths_in_flight(self._h, ctypes.c_int64(n)))

    def release_paths(self) -> None:
        """Frees the path state (about 336 B per path in flight) until the next render."""
        check(native.lib().hasty_job_release_paths(self._h))

    def render_passes(self, n: int, sync: bool = False) -> None:
        check(native.lib().hasty_job_render_passes(self._h, int(n)))
        if sync:
            self.sync()

    def sync(self) -> None:
        check(native.lib().hasty_job_sync(self._h))

    def stop(self) -> None:
        check(native.lib().hasty_job_stop(self._h))

    def set_stage_timing(self, on: bool = True) -> None:
        check(native.lib().hasty_job_set_stage_timing(self._h, 1 if on else 0))

    def stats(self) -> dict:
        s = native.Stats()
        check(native.lib().hasty_job_stats_get(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in native.Stats._fields_}

    def compute_estimate(self, aov: int = AOV_COLOR) -> np.ndarray:
        i = self.info
        out = np.empty((i.height, i.width, 3), dtype=np.float32)
        n = ctypes.c_int32()
        check(native.lib().hasty_job_read(self._h, aov, out.ctypes.data, i.width, i.height, ctypes.byref(n)))
        return out

    def read_sums(self, aov: int = AOV_COLOR) -> tuple[np.ndarray, int]:
        i = self.info
        out = np.empty((i.height, i.width, 3), dtype=np.float64)
        n = ctypes.c_int32()
        check(native.lib().hasty_job_read_sums(self._h, aov, out.ctypes.data, i.width, i.height, ctypes.byref(n)))
        return out, n.value

    # ---- photon mapping (hasty_pm_*): the reference's second integrator ----
    def pm_render(self, iterations: int = 1) -> None:
        """Renders more stochastic progressive photon-mapping iterations."""
        check(native.lib().hasty_pm_render(self._h, int(iterations)))

    def pm_reset(self) -> None:
        check(native.lib().hasty_pm_reset(self._h))

    def pm_read(self, aov: int = AOV_COLOR) -> np.ndarray:
        """The photon mapper's current image (colour with exposure, normal, albedo)."""
        i = self.info
        out = np.empty((i.height, i.width, 3), dtype=np.float32)
        check(native.lib().hasty_pm_read(self._h, aov, out.ctypes.data, i.width, i.height))
        return out

    def pm_radii(self) -> np.ndarray:
        i = self.info
        out = np.empty((i.height, i.width), dtype=np.float32)
        check(native.lib().hasty_pm_read_radii(self._h, out.ctypes.data, i.width, i.height))
        return out

    def pm_stats(self) -> dict:
        s = native.PmStats()
        check(native.lib().hasty_pm_stats_get(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in native.PmStats._fields_}

    def pm_map(self) -> dict:
        """Photon map of the last iteration (test hook): photons in map order
        and the cell table (x, y, z, first, count)."""
        L = native.lib()
        n_ph, n_c, cell = ctypes.c_int64(), ctypes.c_int64(), ctypes.c_float()
        check(L.hasty_debug_pm_map(self._h, None, None, None, None, ctypes.byref(n_ph), ctypes.byref(n_c),
                                   ctypes.byref(cell)))
        xyz = np.empty((n_ph.value, 3), np.float32)
        em = np.empty(n_ph.value, np.uint32)
        ix = np.empty(n_ph.value, np.uint32)
        cells = np.empty((n_c.value, 5), np.int32)
        check(L.hasty_debug_pm_map(self._h, xyz.ctypes.data, em.ctypes.data, ix.ctypes.data, cells.ctypes.data,
                                   ctypes.byref(n_ph), ctypes.byref(n_c), ctypes.byref(cell)))
        return {"xyz": xyz, "emission": em, "index": ix, "cells": cells, "cell": cell.value}

    def write_outputs(self, out_dir: str, write_pfm: bool = False) -> None:
        check(native.lib().hasty_job_write_outputs(self._h, out_dir.encode(), 1 if write_pfm else 0))

    # ---- progressive read-back (the viewer's display loop) while rendering continues ----
    def snapshot(self, aovs=(AOV_COLOR,)) -> None:
        """Enqueues the estimates of `aovs` behind the passes enqueued so far
        and their copy to host memory; returns without waiting."""
        mask = 0
        for a in aovs:
            mask |= 1 << int(a)
        check(native.lib().hasty_job_snapshot(self._h, mask))

    def snapshot_ready(self) -> bool:
        r = ctypes.c_int()
        check(native.lib().hasty_job_snapshot_query(self._h, ctypes.byref(r)))
        return bool(r.value)

    def snapshot_get(self, aov: int = AOV_COLOR) -> tuple[np.ndarray, int]:
        """Waits for the last snapshot; returns a copy of `aov` and the passes it covers."""
        i = self.info
        p = ctypes.c_void_p()
        n = ctypes.c_int32()
        check(native.lib().hasty_job_snapshot_get(self._h, aov, ctypes.byref(p), ctypes.byref(n)))
        buf = (ctypes.c_float * (i.height * i.width * 3)).from_address(p.value)
        return np.frombuffer(buf, dtype=np.float32).reshape(i.height, i.width, 3).copy(), n.value

    def write_outputs_async(self, out_dir: str, write_pfm: bool = False) -> None:
        """write_outputs of this moment, written by a host thread while rendering continues."""
        check(native.lib().hasty_job_write_outputs_async(self._h, out_dir.encode(), 1 if write_pfm else 0))

    def outputs_wait(self) -> None:
        check(native.lib().hasty_job_outputs_wait(self._h))

    def intersect(self, rays: np.ndarray):
        """Closest hits of rays (n x 6: origin, direction) -> (tri, t, u, v)."""
        r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
        n = r.shape[0]
        tri = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        check(native.lib().hasty_debug_intersect(self._h, r.ctypes.data, n, tri.ctypes.data, t.ctypes.data,
                                                  u.ctypes.data, v.ctypes.data))
        return tri, t, u, v

    def triangle_ids(self):
        """Global triangle index -> (OBJ shape id, face id)."""
        n = self.info.n_triangles
        g = np.empty(n, np.int32)
        p = np.empty(n, np.int32)
        check(native.lib().hasty_debug_tri_ids(self._h, g.ctypes.data, p.ctypes.data, n))
        return g, p


def debug_bsdf(which: int, cases: np.ndarray, replay: np.ndarray) -> np.ndarray:
    """Device BSDF on known inputs: which 0 sample, 1 evaluate, 2 pdf.
    cases: n x 33 float32; replay: n x k uint32 (values served in order)."""
    c = np.ascontiguousarray(cases, dtype=np.float32).reshape(-1, 33)
    r = np.ascontiguousarray(replay, dtype=np.uint32).reshape(c.shape[0], -1)
    out = np.zeros((c.shape[0], 12), np.float32)
    check(native.lib().hasty_debug_bsdf(which, c.ctypes.data, c.shape[0], r.ctypes.data, r.shape[1], out.ctypes.data))
    return out


def host_trace(job_path: str, rays: np.ndarray, kind: int = 1):
    """The device traversal code run on the CPU over a host-built BVH (kind 0
    binary, 1 compressed 8-wide); no GPU needed. Returns (tri, t, u, v, info)."""
    r = np.ascontiguousarray(rays, dtype=np.float32).reshape(-1, 6)
    n = r.shape[0]
    tri = np.empty(n, np.int32)
    t, u, v = (np.empty(n, np.float32) for _ in range(3))
    info = np.zeros(3, np.int64)
    check(native.lib().hasty_debug_host_trace(job_path.encode(), kind, r.ctypes.data, n, tri.ctypes.data, t.ctypes.data,
                                               u.ctypes.data, v.ctypes.data, info.ctypes.data))
    return tri, t, u, v, {"triangles": int(info[0]), "nodes": int(info[1]), "depth": int(info[2])}


BATCH_PACKED = 0   # HASTY_BATCH_PACKED
BATCH_REGEN = 1    # HASTY_BATCH_REGEN


def batch_render(jobs, passes, paths_in_flight: int = 0, regen_fraction: float = 0.0, max_iterations: int = 0,
                 mode: int = BATCH_PACKED, lanes: int = 0, resolve_threads: int = 0, sample_threads: int = 0,
                 trace_blocks_per_sm: int = 0, ctx: Context | None = None) -> dict:
    """Renders passes[i] further passes of jobs[i] in one multi-job run and
    adds the results to each job's accumulators. mode BATCH_PACKED (default):
    the jobs' passes packed into batches of paths_in_flight camera samples on
    `lanes` alternating render lanes (results bit-identical to render_passes);
    BATCH_REGEN: path regeneration over a shared pool in one CUDA-graph
    launch. resolve_threads / sample_threads / trace_blocks_per_sm: block
    shapes of the packed batches' kernels (0: defaults). Returns the batch
    statistics."""
    ctx = ctx or jobs[0].ctx
    n = len(jobs)
    handles = (ctypes.c_void_p * n)(*[j._h.value for j in jobs])
    ps = (ctypes.c_int32 * n)(*[int(p) for p in passes])
    cfg = native.BatchConfig(int(paths_in_flight), float(regen_fraction), int(max_iterations), int(mode), int(lanes),
                             int(resolve_threads), int(sample_threads), int(trace_blocks_per_sm), 0)
    st = native.BatchStats()
    check(native.lib().hasty_batch_render(ctx._h, handles, ps, n, ctypes.byref(cfg), ctypes.byref(st)))
    return {k: getattr(st, k) for k, _ in native.BatchStats._fields_}


SERVE_ROUND_ROBIN = 0     # HASTY_SERVE_ROUND_ROBIN
SERVE_SHORTEST_FIRST = 1  # HASTY_SERVE_SHORTEST_FIRST


class Server:
    """Request loop over packed multi-job batches (hasty_server_* in the C
    ABI): requests are admitted by device-memory footprint, scenes stay
    resident and are shared, and the passes of resident requests are packed
    into batches that keep the render lanes busy; a request arriving while
    others render joins the next batch.

        srv = Server(max_resident_jobs=32, memory_budget=120 << 30)
        rid = srv.submit("job/renderJob.json", passes=64, seed=7)
        for res in srv.poll(wait_ms=1000): img = srv.read(res["id"])
    """

    def __init__(self, ctx: Context | None = None, **cfg):
        self.ctx = ctx or default_context()
        c = native.ServerConfig()
        for k, v in cfg.items():
            if not hasattr(c, k):
                raise TypeError(f"unknown server option {k!r}")
            setattr(c, k, v)
        self._h = ctypes.c_void_p()
        check(native.lib().hasty_server_start(self.ctx._h, ctypes.byref(c), ctypes.byref(self._h)))
        self._sizes = {}

    def submit(self, job_path: str, passes: int = 0, seed: int | None = None) -> int:
        rid = ctypes.c_int64()
        sp = ctypes.byref(ctypes.c_uint64(int(seed))) if seed is not None else None
        check(native.lib().hasty_server_submit(self._h, job_path.encode(), int(passes), sp, ctypes.byref(rid)))
        return rid.value

    def poll(self, max_results: int = 256, wait_ms: int = 0) -> list[dict]:
        buf = (native.ServerResult * max_results)()
        n = ctypes.c_size_t()
        check(native.lib().hasty_server_poll(self._h, buf, max_results, ctypes.byref(n), int(wait_ms)))
        out = []
        for r in buf[: n.value]:
            d = {k: getattr(r, k) for k, _ in native.ServerResult._fields_}
            d["error"] = r.error.decode(errors="replace")
            self._sizes[r.id] = (r.height, r.width)
            out.append(d)
        return out

    def read(self, rid: int, aov: int = AOV_COLOR) -> np.ndarray:
        h, w = self._sizes[rid]
        out = np.empty((h, w, 3), dtype=np.float32)
        check(native.lib().hasty_server_read(self._h, rid, aov, out.ctypes.data, w, h))
        return out

    def read_sums(self, rid: int, aov: int = AOV_COLOR) -> np.ndarray:
        h, w = self._sizes[rid]
        out = np.empty((h, w, 3), dtype=np.float64)
        check(native.lib().hasty_server_read_sums(self._h, rid, aov, out.ctypes.data, w, h))
        return out

    def release(self, rid: int) -> None:
        check(native.lib().hasty_server_release(self._h, rid))
        self._sizes.pop(rid, None)

    def stats(self) -> dict:
        s = native.ServerStats()
        check(native.lib().hasty_server_stats_get(self._h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in native.ServerStats._fields_}

    def wait_idle(self, timeout_ms: int = -1) -> None:
        check(native.lib().hasty_server_wait_idle(self._h, int(timeout_ms)))

    def stop(self) -> None:
        if self._h:
            native.lib().hasty_server_stop(self._h)
            self._h = ctypes.c_void_p()

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.stop()

    def __del__(self):
        try:
            self.stop()
        except Exception:
            pass
