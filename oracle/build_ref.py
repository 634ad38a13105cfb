"""Build recipe for oracle/_ref: the reference's own CPU influence code, compiled as a checker.

Test infrastructure only.  For each core-function macro of the reference (src/CoreFunc.h:35-39,
where ``USE_V2_KERNEL`` is hard-wired) this script

* makes a throw-away include directory under the system temp dir holding symlinks to the
  reference's ``src/*`` headers plus a ``CoreFunc.h`` whose active ``#define`` line names the
  wanted core (the quoted include in src/Kernels.h resolves next to the including file, so a
  ``-D`` flag alone cannot switch the core),
* compiles oracle/ref_harness.cpp + src/Body.cpp + lib/tinyexpr/tinyexpr.c (as C) with the
  reference's Release flags (CMakeLists.txt:57: -O3 -march=native, OpenMP),
* writes only ``oracle/_ref/libref_<core>.so`` and removes the temp directory.

Nothing from the reference is copied into the repository.  When the reference tree is absent
(the GPU host) the build is skipped and the tests fall back to the committed golden vectors and
the C restatement in oracle/oracle.c.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
import tempfile
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
# the reference checkout: $OMEGA2D_REFERENCE, else a directory named `reference` beside this
# repository's checkout
REF_ROOT = os.environ.get("OMEGA2D_REFERENCE") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
OUT = os.path.join(HERE, "_ref")

# core id -> macro in src/CoreFunc.h
CORES = {
    "rm": "USE_RM_KERNEL",
    "exp": "USE_EXPONENTIAL_KERNEL",
    "wl": "USE_WL_KERNEL",
    "v2": "USE_V2_KERNEL",
    "v3": "USE_V3_KERNEL",
}


def available() -> bool:
    return os.path.isfile(os.path.join(REF_ROOT, "src", "Influence.h"))


def _make_include_dir(tmp: str, macro: str) -> str:
    src = os.path.join(REF_ROOT, "src")
    inc = os.path.join(tmp, "inc")
    os.makedirs(inc)
    for name in os.listdir(src):
        if name == "CoreFunc.h":
            continue
        os.symlink(os.path.join(src, name), os.path.join(inc, name))
    with open(os.path.join(src, "CoreFunc.h")) as f:
        lines = f.read().split("\n")
    out, switched = [], False
    for ln in lines:
        s = ln.strip()
        if s == "#define USE_V2_KERNEL":
            out.append("#define " + macro)
            switched = True
        else:
            out.append(ln)
    if not switched:
        raise RuntimeError("could not find the core-selection #define in CoreFunc.h")
    with open(os.path.join(inc, "CoreFunc.h"), "w") as f:
        f.write("\n".join(out))
    return inc


def _build_one(core: str, macro: str, force: bool) -> str:
    target = os.path.join(OUT, f"libref_{core}.so")
    harness = os.path.join(HERE, "ref_harness.cpp")
    if (not force and os.path.exists(target)
            and os.path.getmtime(target) > os.path.getmtime(harness)
            and os.path.getmtime(target) > os.path.getmtime(__file__)):
        return target
    tmp = tempfile.mkdtemp(prefix=f"omega_ref_{core}_")
    try:
        inc = _make_include_dir(tmp, macro)
        te_obj = os.path.join(tmp, "tinyexpr.o")
        subprocess.run(["gcc", "-O3", "-fPIC", "-c",
                        os.path.join(REF_ROOT, "lib", "tinyexpr", "tinyexpr.c"), "-o", te_obj],
                       check=True)
        cmd = ["g++", "-std=c++17", "-O3", "-march=native", "-fopenmp", "-fPIC", "-shared",
               "-DVERBOSE=false", "-w",
               "-I", inc, "-I", os.path.join(REF_ROOT, "lib"),
               harness, os.path.join(REF_ROOT, "src", "Body.cpp"), te_obj,
               "-o", target]
        subprocess.run(cmd, check=True)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return target


def build(force: bool = False) -> list[str]:
    """Compile every core variant; returns the library paths ([] when the reference is absent)."""
    if not available():
        return []
    os.makedirs(OUT, exist_ok=True)
    with ThreadPoolExecutor(max_workers=len(CORES)) as ex:
        futs = [ex.submit(_build_one, c, m, force) for c, m in CORES.items()]
        return [f.result() for f in futs]


if __name__ == "__main__":
    print("\n".join(build(force="--force" in sys.argv)))
