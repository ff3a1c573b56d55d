"""Builds the CUDA library libcellflow.so in-tree for sm_103a.

Each translation unit of ``csrc/`` is compiled by nvcc in parallel into
``cellflow_gb300/_build/`` and linked into ``cellflow_gb300/libcellflow.so``.
Host code is compiled with ``-ffp-contract=off`` (the pair tables must round
like the reference's float expressions); device code keeps nvcc's defaults
and pins rounding where it matters with round-to-nearest intrinsics.
"""

from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libcellflow.so"
# the bounds-checked library (-DCF_DEBUG_BOUNDS): out-of-range indices of the
# checked kernels are recorded and skipped (cf_debug_bounds) instead of faulting
BUILD_BOUNDS = PKG / "_build_bounds"
LIB_BOUNDS = PKG / "libcellflow_bounds.so"
INCLUDE = PKG.parent / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["api.cpp", "celllist.cu", "step.cu", "proximity.cu", "init.cu", "peak.cu", "noalloc.cu", "adjoint.cu",
           "preset.cpp"]


def nvcc() -> str:
    cand = os.environ.get("NVCC") or shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return cand


def _flags(src: str, bounds: bool = False) -> list[str]:
    common = ["-std=c++17", "-O3", "-Xcompiler", "-fPIC,-ffp-contract=off", f"-I{INCLUDE}", f"-I{CSRC}"]
    if bounds:
        common.append("-DCF_DEBUG_BOUNDS")
    if src.endswith(".cu"):
        return common + ARCH + ["-lineinfo", "-Xptxas", "-O3"]
    return common


def _compile(src: str, bounds: bool = False) -> Path:
    obj = (BUILD_BOUNDS if bounds else BUILD) / (src + ".o")
    cmd = [nvcc(), *_flags(src, bounds), "-c", str(CSRC / src), "-o", str(obj)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    return obj


def _stale(lib: Path = LIB) -> bool:
    if not lib.exists():
        return True
    t = lib.stat().st_mtime
    deps = list(CSRC.glob("*")) + list(INCLUDE.glob("**/*.h")) + [Path(__file__)]
    return any(p.stat().st_mtime > t for p in deps)


def build(force: bool = False, bounds: bool = False) -> Path:
    """Compile and link libcellflow.so (libcellflow_bounds.so with bounds); returns its path."""
    LIB_OUT = LIB_BOUNDS if bounds else LIB
    if not force and not _stale(LIB_OUT):
        return LIB_OUT
    (BUILD_BOUNDS if bounds else BUILD).mkdir(exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda src: _compile(src, bounds), SOURCES))
    tmp = LIB_OUT.with_suffix(".so.tmp")
    cmd = [nvcc(), "-shared", *ARCH, "-o", str(tmp), *map(str, objs)]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, LIB_OUT)
    return LIB_OUT


if __name__ == "__main__":
    import sys

    print(build(force=True, bounds="--bounds" in sys.argv))
