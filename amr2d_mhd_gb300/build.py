"""Build of the sm_103a library libamr2d_mhd.so and of the host program
amr2d_mhd that drives it (in-tree, amr2d_mhd_gb300/_build/).

Every translation unit compiles in parallel with nvcc for sm_103a only.  Every
translation unit but the FP32 stage kernels (stage_f32_*.cu) is compiled with
-fmad=false and the host code with -ffp-contract=off: that path reproduces the reference's
floating-point operations one by one, so nothing may be fused.  The FP32 stage
kernels (the FP32 bulk path's reconstruction, Riemann fluxes and RK update)
use FMA contraction and the approximate FP32 division and square root
(-prec-div=false -prec-sqrt=false, about 2 ulp): their results are compared
with the FP64 path through a tolerance, and the FP64 parts of that path
(pressure recovery, face field, dt) are compiled elsewhere or stay FP64.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libamr2d_mhd.so")
HOST = os.path.join(HERE, "host")
DRIVER = os.path.join(BUILD, "amr2d_mhd")   # the reference program's main() on the library
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA extension cannot be built")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _flags(src: str):
    common = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
              "-I" + CSRC]
    if src.endswith(".cpp"):
        return ["-x", "cu"] + ARCH + common
    fmad = ["-prec-div=false", "-prec-sqrt=false"] if src.startswith("stage_f32") else ["-fmad=false"]
    return ARCH + common + fmad


def _stamp(d: str = CSRC) -> float:
    """Newest input of the library (d = CSRC) or of the host program (d = HOST)."""
    t = 0.0
    for f in os.listdir(d):
        t = max(t, os.path.getmtime(os.path.join(d, f)))
    t = max(t, os.path.getmtime(os.path.join(HERE, "..", "include", "amr2d_mhd.h")))
    return max(t, os.path.getmtime(__file__))


def _driver_stale() -> bool:
    return not os.path.exists(DRIVER) or os.path.getmtime(DRIVER) < max(_stamp(HOST), os.path.getmtime(LIB))


def build_driver() -> str:
    """amr2d_mhd, the host program that reads input.txt and drives the
    library through its C ABI only (linked with an $ORIGIN run path).  A
    failure is reported on stderr and leaves the library usable."""
    cxx = os.environ.get("CXX") or shutil.which("g++") or "c++"
    src = os.path.join(HOST, "amr2d_main.cpp")
    tmp = DRIVER + ".tmp%d" % os.getpid()
    cmd = [cxx, "-O2", "-std=c++17", "-I" + os.path.join(HERE, "..", "include"), src, "-L" + BUILD,
           "-lamr2d_mhd", "-Wl,-rpath,$ORIGIN", "-o", tmp]
    try:
        r = subprocess.run(cmd, capture_output=True, text=True)
    except OSError as e:
        sys.stderr.write("amr2d_mhd driver not built: %s\n" % e)
        return ""
    if r.returncode != 0:
        sys.stderr.write("amr2d_mhd driver not built:\n%s%s" % (r.stdout, r.stderr))
        return ""
    os.replace(tmp, DRIVER)
    return DRIVER


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= _stamp():
        if _driver_stale():
            build_driver()
        return LIB
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()

    def compile_one(src):
        obj = os.path.join(BUILD, src + ".o")
        cmd = [nvcc, "-c", os.path.join(CSRC, src), "-o", obj] + _flags(src)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    n = jobs or min(len(srcs), max(2, os.cpu_count() or 2))
    with cf.ThreadPoolExecutor(n) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp%d" % os.getpid()
    cmd = [nvcc, "-shared"] + ARCH + ["-o", tmp] + objs + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    build_driver()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
