"""Builds the in-tree shared libraries of porescale_gb300.

* ``porescale_gb300/libporescale_gpu.so`` -- the CUDA library behind the C ABI
  declared in ``include/porescale.h`` (sm_103a only);
* ``oracle/libps_oracle.so`` -- the CPU FP64 restatement used as the parity
  reference by the tests and as the CPU baseline of ``bench.py`` (built, never called,
  by the library itself).

Translation units are compiled in parallel; an output is rebuilt only when a
source or header is newer than it.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "porescale_gb300")
CSRC = os.path.join(PKG, "csrc")
ORACLE = os.path.join(ROOT, "oracle")
BUILD = os.path.join(PKG, "_objs")
LIB = os.path.join(PKG, "libporescale_gpu.so")
DRIVER = os.path.join(PKG, "porescale_run")
DRIVER_SRC = os.path.join(PKG, "driver", "porescale_run.cpp")
ORACLE_LIB = os.path.join(ORACLE, "libps_oracle.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
                      "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]
# per-TU extra flags: the FP64 LBM and gray-lattice kernels must not contract
# a*b+c into FMA (bit-exact against the FP64 oracle)
TU_FLAGS = {
    "lbm_prec_f64.cu": ["--fmad=false"],
    "gray_api.cu": ["--fmad=false"],
}


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build porescale_gb300")


def _newer(target: str, deps: list[str]) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build_gpu(verbose: bool = False, ptxas_info: bool = False) -> str:
    nvcc = _nvcc()
    os.makedirs(BUILD, exist_ok=True)
    sources = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "porescale.h")]
    jobs = []
    objs = []
    for src in sources:
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + ".o")
        objs.append(obj)
        if _newer(obj, [src] + headers) or ptxas_info:
            cmd = [nvcc] + NVCC_COMMON + TU_FLAGS.get(os.path.basename(src), []) + ["-c", src, "-o", obj]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        for cmd in jobs:
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
        list(ex.map(_run, jobs))
    if _newer(LIB, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-cudart=static"])
    return LIB


def build_driver() -> str:
    """porescale_run: the reference driver's LBM loop on the C ABI."""
    lib = build_gpu()
    if _newer(DRIVER, [DRIVER_SRC, lib, os.path.join(ROOT, "include", "porescale.h")]):
        cxx = shutil.which("g++") or "c++"
        _run([cxx, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"), DRIVER_SRC, "-o", DRIVER,
              "-L" + PKG, "-lporescale_gpu", "-Wl,-rpath,$ORIGIN"])
    return DRIVER


def build_oracle() -> str:
    srcs = sorted(glob.glob(os.path.join(ORACLE, "*.c")))
    hdrs = glob.glob(os.path.join(ORACLE, "*.h"))
    if _newer(ORACLE_LIB, srcs + hdrs):
        cc = shutil.which("gcc") or "cc"
        _run([cc, "-O2", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared", "-std=c11", "-o", ORACLE_LIB]
             + srcs + ["-lm"])
    return ORACLE_LIB


def build_all(verbose: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gpu, verbose)
        f2 = ex.submit(build_oracle)
        f1.result()
        f2.result()
    build_driver()


if __name__ == "__main__":
    build_all(verbose="-v" in sys.argv)
    if "--ptxas" in sys.argv:
        build_gpu(verbose=True, ptxas_info=True)
