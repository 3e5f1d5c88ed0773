"""Builds the native library and CLI in-tree (no CMake, no torch extension).

    python -m hastyrenderer_gb300.build            # library + CLI
    python -m hastyrenderer_gb300.build --oracle   # also the CPU oracle under oracle/
    python -m hastyrenderer_gb300.build --debug-bounds   # the bounds-checked variant, lib/bounds/

CUDA sources are compiled for sm_103a only; `integrator.cu` without FMA
contraction (products and sums round like the reference's scalar C++), and
`bvh_gpu.cu` likewise (its layout writer matches the host writer's bytes), and
`photon.cu` (the photon mapper's shading, like the integrator's).
Outputs: hastyrenderer_gb300/lib/libhasty_gb300.so, lib/hasty_gpu_render.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OBJ = os.path.join(PKG, "lib", "obj")
LIB = os.path.join(PKG, "lib")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off", "-I" + INCLUDE,
               "-I" + CSRC, "--expt-relaxed-constexpr"]
CU_EXTRA = {"integrator.cu": ["--fmad=false"], "bvh_gpu.cu": ["--fmad=false"], "photon.cu": ["--fmad=false"], "photon_build.cu": ["--fmad=false"]}
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-sign-compare"]
CU_SOURCES = ["integrator.cu", "trace.cu", "static_scratch.cu", "bvh_gpu.cu", "photon.cu", "photon_build.cu"]
# Extra nvcc flags for experiments (e.g. HASTY_NVCC_FLAGS="-DHASTY_OUTLINE_MASK=3").
EXTRA_NVCC = os.environ.get("HASTY_NVCC_FLAGS", "").split()
CPP_SOURCES = ["api.cpp", "engine.cpp", "packed.cpp", "server.cpp", "scene_load.cpp", "bvh_build.cpp", "image_out.cpp", "photon_map.cpp"]


def cuda_home() -> str:
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs.append(os.path.join(INCLUDE, "hasty_gpu.h"))
    return sorted(hs)


def _stamp(src: str, cmd: list[str]) -> str:
    h = hashlib.sha256(" ".join(cmd).encode())
    for f in [src] + _headers():
        with open(f, "rb") as fh:
            h.update(fh.read())
    return h.hexdigest()


def _compile(src: str, cmd: list[str], obj: str, verbose: bool) -> str:
    stamp = obj + ".stamp"
    digest = _stamp(src, cmd)
    if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == digest:
        return obj
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as fh:
        fh.write(digest)
    return obj


def build(verbose: bool = False, jobs: int | None = None, debug_bounds: bool = False) -> str:
    """Compile the CUDA/C++ sources; returns the path of libhasty_gb300.so.
    debug_bounds: the bounds-checked variant (HASTY_DEBUG_BOUNDS: device
    index checks that record a status bit and skip the access), written to
    lib/bounds/ beside the regular build."""
    home = cuda_home()
    nvcc = os.path.join(home, "bin", "nvcc")
    cxx = os.environ.get("CXX", "g++")
    lib = os.path.join(LIB, "bounds") if debug_bounds else LIB
    objdir = os.path.join(lib, "obj")
    extra = ["-DHASTY_DEBUG_BOUNDS=1"] if debug_bounds else []
    os.makedirs(objdir, exist_ok=True)
    tasks = []
    for f in CU_SOURCES:
        src = os.path.join(CSRC, f)
        obj = os.path.join(objdir, f + ".o")
        cmd = [nvcc] + ARCH + NVCC_COMMON + CU_EXTRA.get(f, []) + EXTRA_NVCC + extra + ["-c", src, "-o", obj]
        tasks.append((src, cmd, obj))
    for f in CPP_SOURCES + ["cli.cpp"]:
        src = os.path.join(CSRC, f)
        obj = os.path.join(objdir, f + ".o")
        cmd = [cxx] + CXX_FLAGS + extra + ["-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(home, "include"), "-c", src,
                                           "-o", obj]
        tasks.append((src, cmd, obj))
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda t: _compile(t[0], t[1], t[2], verbose), tasks))
    lib_objs = [o for o in objs if not o.endswith("cli.cpp.o")]
    so = os.path.join(lib, "libhasty_gb300.so")
    link = [nvcc] + ARCH + ["-shared", "-o", so] + lib_objs + ["-lpthread"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    exe = os.path.join(lib, "hasty_gpu_render")
    link = [nvcc] + ARCH + ["-o", exe, os.path.join(objdir, "cli.cpp.o"), "-L" + lib, "-lhasty_gb300",
                            "-Xlinker", "-rpath=$ORIGIN"]
    r = subprocess.run(link, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed (cli)\n{r.stdout}\n{r.stderr}")
    return so


def build_oracle(with_reference: bool | None = None, verbose: bool = False) -> None:
    """CPU oracle: oracle/_build/liboracle.so, and the reference build under
    oracle/_ref when HASTY_REFERENCE_DIR names a checkout of the reference
    (its core/src and core/include directories are compiled from there)."""
    odir = os.path.join(ROOT, "oracle")
    targets = ["port"]
    ref = os.environ.get("HASTY_REFERENCE_DIR", "")
    if with_reference is None:
        with_reference = bool(ref) and os.path.isdir(os.path.join(ref, "core", "src"))
    if with_reference:
        if not ref:
            raise RuntimeError("the reference build needs HASTY_REFERENCE_DIR (a checkout of the reference)")
        targets.append("ref")
    cmd = ["make", "-C", odir, f"-j{min(8, os.cpu_count() or 4)}"] + ([f"REF={ref}"] if ref else []) + targets
    r = subprocess.run(cmd, capture_output=not verbose, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"oracle build failed\n{r.stdout}\n{r.stderr}")


if __name__ == "__main__":
    so = build(verbose="-v" in sys.argv, debug_bounds="--debug-bounds" in sys.argv)
    print(so)
    if "--oracle" in sys.argv:
        build_oracle(verbose="-v" in sys.argv)
