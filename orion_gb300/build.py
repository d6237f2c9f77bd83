"""Build the product's in-tree shared library (no setup.py, no cmake).

``orion_gb300/liborion_gb300.so``: the CUDA kernels for sm_103a (nvcc) and
the host runtime (scene loader, BVH builder, C ABI) compiled with
``-ffp-contract=off`` so host-side float math rounds the same on x86 and Arm
and matches the reference's order of operations. The test oracle is built by
oracle/build.py, apart from the product.

Objects compile in parallel; a rebuild skips objects newer than their inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "orion_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liborion_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _run(cmd: list[str]) -> None:
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(cmd) + "\n" + p.stdout + p.stderr)


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps)


def build_product(verbose_ptxas: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    headers = glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) + \
        [os.path.join(ROOT, "include", "orion_gpu.h")]
    jobs = []
    objs = []
    for cu in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(BUILD, os.path.basename(cu) + ".o")
        objs.append(obj)
        if _stale(obj, [cu] + headers):
            cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-ffp-contract=off",
                   "-c", cu, "-o", obj]
            if verbose_ptxas:
                cmd.insert(1, "-Xptxas=-v")
            jobs.append(cmd)
    for cpp in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(BUILD, os.path.basename(cpp) + ".o")
        objs.append(obj)
        if _stale(obj, [cpp] + headers):
            jobs.append(["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
                         "-I", os.path.join(CUDA_HOME, "include"), "-c", cpp, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        list(ex.map(_run, jobs))
    if _stale(LIB, objs):
        _run([NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fPIC", "-lpthread", "-ldl"])
    return LIB


def sobol_table() -> str:
    """The committed Sobol direction numbers the library loads (data/sobol_matrices.bin)."""
    from orion_gb300 import gen_sobol
    if not os.path.exists(gen_sobol.OUT):
        raise RuntimeError("missing " + gen_sobol.OUT)
    return gen_sobol.OUT


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    sobol_table()
    print(build_product())
