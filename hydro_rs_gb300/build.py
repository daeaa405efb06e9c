"""Builds the native parts of the library in-tree (no pip install).

* ``_build/libmvmm_gpu.so``  - the CUDA library behind ``include/mvmm_gpu.h``,
  compiled for sm_103a only.  ``step_fp64.cu`` is compiled with ``-fmad=false``
  so the plain form never contracts a*b+c (the Rust reference never does);
  ``step_fp32.cu`` (the FP32-face form, held to an error bound rather than to
  the reference's roundings) keeps FMA contraction and uses the approximate
  FP32 division and square root (``-prec-div=false -prec-sqrt=false``, ~2 ulp).
* ``_build/libmvmm_mesh.so`` - the host Voronoi mesh builder (g++ / OpenMP).

Sources are compiled in parallel; up-to-date objects are reused.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_COMMON = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
                      "--expt-relaxed-constexpr"]

CU_SOURCES = {
    "step_fp64.cu": ["-fmad=false"],
    "step_fp32.cu": ["-fmad=true", "-prec-div=false", "-prec-sqrt=false"],
    "mvmm_api.cu": ["-Xcompiler", "-fopenmp"],
    "noalloc.cu": ["-fmad=false"],
}
HEADERS = ["mvmm_device.cuh", "mvmm_internal.h", "mvmm_cellops.cuh", "bitconv.cuh", "face64.cuh"]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if c and (os.path.sep not in c or os.path.exists(c)):
            return c
    return "nvcc"


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def _run(cmd, log=None):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if log is not None:
        with open(log, "w") as f:
            f.write(" ".join(cmd) + "\n" + r.stdout + r.stderr)
    if r.returncode != 0:
        sys.stderr.write(r.stdout + r.stderr)
        raise RuntimeError("command failed: " + " ".join(cmd))
    return r


def build_gpu(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    nvcc = _nvcc()
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(INCLUDE, "mvmm_gpu.h")]
    jobs = []
    objs = []
    for src, extra in CU_SOURCES.items():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT, src + ".o")
        objs.append(o)
        if _stale(o, [s, __file__] + hdrs):
            cmd = [nvcc] + NVCC_COMMON + extra + ["-Xptxas", "-v", "-c", s, "-o", o]
            jobs.append((cmd, os.path.join(OUT, src + ".ptxas.log")))
    with ThreadPoolExecutor(max_workers=len(jobs) or 1) as ex:
        list(ex.map(lambda j: _run(*j), jobs))
    lib = os.path.join(OUT, "libmvmm_gpu.so")
    if _stale(lib, objs):
        _run([nvcc] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart", "-lgomp"])
    return lib


def build_mesh() -> str:
    os.makedirs(OUT, exist_ok=True)
    src = os.path.join(CSRC, "voronoi.cpp")
    lib = os.path.join(OUT, "libmvmm_mesh.so")
    if _stale(lib, [src, __file__]):
        _run(["g++", "-O2", "-std=c++17", "-fPIC", "-fopenmp", "-shared", "-o", lib, src])
    return lib


def build_all() -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_gpu)
        f2 = ex.submit(build_mesh)
        f1.result()
        f2.result()


if __name__ == "__main__":
    build_all()
