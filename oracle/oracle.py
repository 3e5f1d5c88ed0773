"""Oracle (test infrastructure only): ctypes access to the CPU oracle.

``Oracle`` drives the CPU restatement (oracle/port, built to
oracle/_build/liboracle.so); ``ReferenceBuild`` drives the reference's own
integrator compiled under oracle/_ref (development machine only). Only tests,
__graft_entry__.smoke() and bench.py's CPU-baseline leg use this module.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
PORT_LIB = os.path.join(HERE, "_build", "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "libhasty_ref.so")

_libs: dict[str, ctypes.CDLL] = {}


def _load(path: str, prefix: str) -> ctypes.CDLL:
    if path in _libs:
        return _libs[path]
    if not os.path.exists(path):
        raise RuntimeError(f"oracle library missing: {path} (make -C oracle)")
    L = ctypes.CDLL(path)
    P, I = ctypes.c_void_p, ctypes.c_int
    getattr(L, prefix + "_load").restype = P
    getattr(L, prefix + "_load").argtypes = [ctypes.c_char_p, ctypes.c_char_p, I]
    getattr(L, prefix + "_free").argtypes = [P]
    getattr(L, prefix + "_render").argtypes = [P] + [I] * 7 + [P] * 5
    getattr(L, prefix + "_render_samples").argtypes = [P, I, I, I, I, I, P, P, P]
    getattr(L, prefix + "_kat").argtypes = [I, P, P, I, P]
    if prefix == "hor":
        L.hor_info.argtypes = [P, P]
        L.hor_set_seed.argtypes = [P, ctypes.c_uint64]
        L.hor_set_ulp_nudge.argtypes = [I]
        L.hor_intersect.argtypes = [P, P, ctypes.c_int64, I, P, P, P, P, P]
        L.hor_tri_ids.argtypes = [P, P, P]
        L.hor_rng_stream.argtypes = [ctypes.c_uint64, ctypes.c_uint32, ctypes.c_uint32, I, P]
        L.hor_halton.argtypes = [ctypes.c_uint32, ctypes.c_uint32]
        L.hor_halton.restype = ctypes.c_float
        L.hor_render_rows.argtypes = [P] + [I] * 8 + [P] * 5
    _libs[path] = L
    return L


class _Base:
    prefix = ""
    path = ""

    def __init__(self, job_path: str):
        self.L = _load(self.path, self.prefix)
        err = ctypes.create_string_buffer(1024)
        self.h = getattr(self.L, self.prefix + "_load")(job_path.encode(), err, 1024)
        if not self.h:
            raise RuntimeError("oracle load failed: " + err.value.decode())

    def close(self):
        if self.h:
            getattr(self.L, self.prefix + "_free")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def render(self, pass0: int, npasses: int, x0: int, y0: int, w: int, h: int, nthreads: int = 0) -> dict:
        c = np.zeros((h, w, 3)); c2 = np.zeros_like(c); n = np.zeros_like(c); a = np.zeros_like(c)
        st = np.zeros(6, np.uint64)
        getattr(self.L, self.prefix + "_render")(self.h, pass0, npasses, x0, y0, w, h, nthreads, c.ctypes.data,
                                                 c2.ctypes.data, n.ctypes.data, a.ctypes.data, st.ctypes.data)
        return {"color": c, "color_sq": c2, "normal": n, "albedo": a, "stats": st}

    def render_samples(self, pass_idx: int, x0: int, y0: int, w: int, h: int):
        c = np.zeros((h, w, 3), np.float32); n = np.zeros_like(c); a = np.zeros_like(c)
        getattr(self.L, self.prefix + "_render_samples")(self.h, pass_idx, x0, y0, w, h, c.ctypes.data, n.ctypes.data,
                                                         a.ctypes.data)
        return c, n, a


class Oracle(_Base):
    prefix = "hor"
    path = PORT_LIB

    def info(self) -> dict:
        out = np.zeros(12, np.int64)
        self.L.hor_info(self.h, out.ctypes.data)
        keys = ["width", "height", "num_samples", "max_depth", "n_tris", "n_light_tris", "env_is_texture", "use_mis",
                "roulette_start", "n_shapes", "n_materials", "seed"]
        return dict(zip(keys, out.tolist()))

    def set_seed(self, seed: int) -> None:
        self.L.hor_set_seed(self.h, ctypes.c_uint64(seed))

    def set_ulp_nudge(self, on: bool) -> None:
        """Process-wide: per-sample sin/cos/atan2/acos/pow results moved by one
        ulp (measures how often a last-ulp math difference changes a sample)."""
        self.L.hor_set_ulp_nudge(1 if on else 0)

    def render_rows(self, pass0: int, npasses: int, y0: int, row_stride: int, n_rows: int, nthreads: int = 0) -> dict:
        """Full-width rows y0, y0 + row_stride, ... (n_rows of them) over
        passes [pass0, pass0 + npasses); arrays hold the rendered rows."""
        w = self.info()["width"]
        c = np.zeros((n_rows, w, 3)); c2 = np.zeros_like(c); n = np.zeros_like(c); a = np.zeros_like(c)
        st = np.zeros(6, np.uint64)
        rc = self.L.hor_render_rows(self.h, pass0, npasses, 0, y0, w, n_rows, row_stride, nthreads, c.ctypes.data,
                                    c2.ctypes.data, n.ctypes.data, a.ctypes.data, st.ctypes.data)
        if rc != 0:
            raise RuntimeError("bad row stride")
        return {"color": c, "color_sq": c2, "normal": n, "albedo": a, "stats": st}

    def intersect(self, rays: np.ndarray, fp64: bool = False, brute: bool = False):
        r = np.ascontiguousarray(rays, np.float32).reshape(-1, 6)
        n = r.shape[0]
        tri = np.empty(n, np.int32)
        t, u, v = (np.empty(n, np.float32) for _ in range(3))
        st = np.zeros(2, np.uint64)
        self.L.hor_intersect(self.h, r.ctypes.data, n, 1 if fp64 else (2 if brute else 0), tri.ctypes.data, t.ctypes.data,
                             u.ctypes.data, v.ctypes.data, st.ctypes.data)
        return tri, t, u, v, st

    def triangle_ids(self):
        n = self.info()["n_tris"]
        g = np.empty(n, np.int32); p = np.empty(n, np.int32)
        self.L.hor_tri_ids(self.h, g.ctypes.data, p.ctypes.data)
        return g, p


class ReferenceBuild(_Base):
    prefix = "ref"
    path = REF_LIB

    @staticmethod
    def available() -> bool:
        return os.path.exists(REF_LIB)


class PhotonMapper:
    """Photon mapper of the CPU oracle (oracle/port/oracle_pm.cpp) or of the
    reference build (oracle/ref_pm_harness.cpp): `iterate(n)` runs n more
    progressive iterations and returns the current images (H, W, 3), the
    radii (H, W) and {emitted, stored, iteration} of the last iteration."""

    def __init__(self, job_path: str, reference: bool = False):
        self.reference = reference
        P, I = ctypes.c_void_p, ctypes.c_int
        if reference:
            self.L = _load(REF_LIB, "ref")
            self.L.ref_pm_load.restype = P
            self.L.ref_pm_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, I]
            self.L.ref_pm_free.argtypes = [P]
            self.L.ref_pm_iterate.argtypes = [P, I, P, P, P, P, P]
            err = ctypes.create_string_buffer(1024)
            self.h = self.L.ref_pm_load(job_path.encode(), err, 1024)
            if not self.h:
                raise RuntimeError("reference load failed: " + err.value.decode())
            self.scene = None
        else:
            self.scene = Oracle(job_path)
            self.L = self.scene.L
            self.L.hor_pm_new.restype = P
            self.L.hor_pm_new.argtypes = [P]
            self.L.hor_pm_free.argtypes = [P]
            self.L.hor_pm_iterate.argtypes = [P, P, I, P, P, P, P, P]
            self.h = self.L.hor_pm_new(self.scene.h)
        info = Oracle(job_path).info() if reference else self.scene.info()
        self.W, self.H = info["width"], info["height"]

    def iterate(self, n: int) -> dict:
        c = np.zeros((self.H, self.W, 3), np.float32); nn = np.zeros_like(c); a = np.zeros_like(c)
        r = np.zeros((self.H, self.W), np.float32)
        info = np.zeros(4, np.int64)
        if self.reference:
            rc = self.L.ref_pm_iterate(self.h, n, c.ctypes.data, nn.ctypes.data, a.ctypes.data, r.ctypes.data,
                                       info.ctypes.data)
        else:
            rc = self.L.hor_pm_iterate(self.scene.h, self.h, n, c.ctypes.data, nn.ctypes.data, a.ctypes.data,
                                       r.ctypes.data, info.ctypes.data)
        if rc != 0:
            raise RuntimeError("photon mapper iteration failed")
        return {"color": c, "normal": nn, "albedo": a, "radii": r, "emitted": int(info[0]), "stored": int(info[1]),
                "iteration": int(info[2])}

    def close(self):
        if self.h:
            (self.L.ref_pm_free if self.reference else self.L.hor_pm_free)(self.h)
            self.h = None
        if self.scene is not None:
            self.scene.close()


def kat(which: int, inputs: np.ndarray, replay: np.ndarray, reference: bool = False) -> np.ndarray:
    """Known-answer call of one routine per row of `inputs` with the matching
    row of `replay` as its uniform stream. Output rows have 12 floats."""
    L = _load(REF_LIB, "ref") if reference else _load(PORT_LIB, "hor")
    f = L.ref_kat if reference else L.hor_kat
    x = np.ascontiguousarray(inputs, np.float32)
    r = np.ascontiguousarray(replay, np.uint32)
    out = np.full((x.shape[0], 12), np.nan, np.float32)
    for i in range(x.shape[0]):
        rc = f(which, x[i].ctypes.data, r[i].ctypes.data, r.shape[1], out[i].ctypes.data)
        if rc < 0:
            raise RuntimeError(f"kat {which} case {i} failed ({rc})")
    return out


def rng_stream(seed: int, pixel: int, pass_idx: int, n: int) -> np.ndarray:
    L = _load(PORT_LIB, "hor")
    out = np.empty(n, np.uint32)
    L.hor_rng_stream(ctypes.c_uint64(seed), pixel, pass_idx, n, out.ctypes.data)
    return out


def halton(base: int, k: int) -> float:
    return float(_load(PORT_LIB, "hor").hor_halton(base, k))


def property_test(which: int, n: int, seed: int = 0) -> np.ndarray:
    """The reference's unit tests (apps/Tests.cpp) run as loops in the CPU
    oracle; returns the quantities each test asserts on."""
    L = _load(PORT_LIB, "hor")
    L.hor_property.argtypes = [ctypes.c_int, ctypes.c_int64, ctypes.c_uint64, ctypes.c_void_p]
    out = np.zeros(8, np.float64)
    k = L.hor_property(which, n, ctypes.c_uint64(seed), out.ctypes.data)
    if k < 0:
        raise RuntimeError(f"property test {which} unknown")
    return out[:k]
