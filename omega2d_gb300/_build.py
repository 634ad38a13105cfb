"""Build recipe for libomega2d_gb300.so (sm_103a only).

Every ``csrc/*.cu`` / ``csrc/*.cpp`` translation unit is compiled by nvcc in parallel into
``omega2d_gb300/_build/`` and linked (static cudart) into ``omega2d_gb300/libomega2d_gb300.so``.
An object is rebuilt when its source or any csrc header is newer.
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libomega2d_gb300.so")
INCLUDE = os.path.join(os.path.dirname(PKG), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O3",
                     "-I", INCLUDE, "--expt-relaxed-constexpr"]
# Extra flags, e.g. OBS_NVCC_EXTRA=-DOBS_DEVICE_CHECKS for a bounds-checked debug build
# (build into a separate tree with OBS_BUILD_DIR / OBS_LIB to keep the release library).
NVCC_FLAGS += os.environ.get("OBS_NVCC_EXTRA", "").split()
# per-file flags: clear_inner_layer follows the reference's float arithmetic operation by
# operation, so its products and sums are not fused (the oracle is built the same way)
# (device code: -fmad=false; host code, the cut table: -ffp-contract=off, which matters where the
# host ISA has FMA, e.g. aarch64)
FILE_FLAGS = {"clear_inner.cu": ["-fmad=false", "-Xcompiler", "-ffp-contract=off"]}
BUILD = os.environ.get("OBS_BUILD_DIR", BUILD)
LIB = os.environ.get("OBS_LIB", LIB)


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _sources() -> list[str]:
    return sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))


def _headers() -> list[str]:
    return (glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h"))
            + glob.glob(os.path.join(INCLUDE, "*.h")))


def _compile(src: str, newest_header: float, verbose: bool) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(src), newest_header):
        return obj
    cmd = ([nvcc()] + NVCC_FLAGS + FILE_FLAGS.get(os.path.basename(src), []) + (["-Xptxas", "-v"] if verbose else [])
           + ["-c", src, "-o", obj])
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(r.stdout + r.stderr)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = _sources()
    newest = max([os.path.getmtime(h) for h in _headers()] + [os.path.getmtime(__file__)])
    jobs = jobs or max(1, min(len(srcs), os.cpu_count() or 4))
    with ThreadPoolExecutor(max_workers=jobs) as ex:
        objs = list(ex.map(lambda s: _compile(s, newest, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    tmp = LIB + ".tmp"
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(verbose="-v" in sys.argv))
