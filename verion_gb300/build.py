"""Builds the CUDA backend library `verion_gb300/_build/libvgcuda.so` for sm_103a.

The translation units compile in parallel (nvcc for the kernels, g++ for the BVH builder), then
nvcc links them with the static CUDA runtime into one shared library with the C ABI of
`include/vgcuda.h`. Device code is compiled without FMA contraction and with correctly rounded
division and square root, host code with -ffp-contract=off: the kernels then compute exactly the
single-precision operations their source spells out, which is what makes bit-exact comparison
with a CPU restatement possible.
"""
from __future__ import annotations

import fcntl
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = BUILD / "libvgcuda.so"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + [
    "-O3", "-std=c++17", "-lineinfo", "--fmad=false", "-prec-div=true", "-prec-sqrt=true",
    "-Xcompiler", "-fPIC,-ffp-contract=off,-O2", "-I", str(CSRC),
]
CXX_FLAGS = ["-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-I", str(CSRC)]

CU_SOURCES = ["kern_mk.cu", "kern_wf.cu", "kern_wf_restir.cu", "kern_nrc.cu", "kern_batch.cu", "kern_bwave.cu", "vgcuda.cu", "cache.cu", "batch.cu"]
CXX_SOURCES = ["bvh_build.cpp", "exr.cpp"]
DEPS = ["vg_math.h", "host.h", "cdf_guide.h", "tc.cuh", "nrc.cuh", "nrc_device.cuh", "vg_layout.h", "vec3.h", "bvh8.h", "traverse.cuh", "pt_device.cuh", "kernels.cuh",
        "launch.h", "launch_nrc.h", "launch_batch.h", "batch.h", "cache_host.h", "bvh_build.h"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build verion_gb300")
    return cand


def _stale(obj: Path, src: Path) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    deps = [src] + [CSRC / d for d in DEPS] + [PKG.parent / "include" / "vgcuda.h", Path(__file__)]
    return any(d.exists() and d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"build step failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")


def build(force: bool = False, verbose: bool = False, defines=(), build_dir: Path = None) -> Path:
    """Compiles the library if any source is newer than it; returns its path. `defines` adds
    preprocessor definitions (e.g. "VG_SHADE_MIN_BLOCKS=4") for a variant built in `build_dir`.
    Processes that build into the same folder at once take turns (an exclusive lock on
    `<build>/.lock`), so none of them loads a half-written library."""
    BUILD = Path(build_dir) if build_dir else globals()["BUILD"]
    BUILD.mkdir(parents=True, exist_ok=True)
    with open(BUILD / ".lock", "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        try:
            return _build_locked(BUILD, force, verbose, defines)
        finally:
            fcntl.flock(lock, fcntl.LOCK_UN)


def _build_locked(BUILD: Path, force: bool, verbose: bool, defines) -> Path:
    LIB = BUILD / "libvgcuda.so"
    extra = [f"-D{d}" for d in defines]
    nvcc = _nvcc()
    cxx = shutil.which("g++") or "g++"
    jobs = []
    objs = []
    for s in CU_SOURCES:
        o = BUILD / (Path(s).stem + ".o")
        objs.append(o)
        if force or _stale(o, CSRC / s):
            jobs.append([nvcc] + NVCC_FLAGS + extra + ["-c", str(CSRC / s), "-o", str(o)])
    for s in CXX_SOURCES:
        o = BUILD / (Path(s).stem + ".o")
        objs.append(o)
        if force or _stale(o, CSRC / s):
            jobs.append([cxx] + CXX_FLAGS + extra + ["-c", str(CSRC / s), "-o", str(o)])
    if jobs:
        with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
            for cmd in jobs:
                if verbose:
                    print(" ".join(cmd), file=sys.stderr)
            list(ex.map(_run, jobs))
    if force or jobs or not LIB.exists():
        tmp = BUILD / f"libvgcuda.so.{os.getpid()}.tmp"
        _run([nvcc] + ARCH + ["-shared", "-o", str(tmp)] + [str(o) for o in objs])
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
