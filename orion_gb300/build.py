"""Build the in-tree shared libraries (no setup.py, no cmake).

* ``orion_gb300/liborion_gb300.so`` -- the product: CUDA kernels for sm_103a
  (nvcc) and the host runtime (scene loader, BVH builder, C ABI) compiled
  with ``-ffp-contract=off`` so host-side float math rounds the same on x86
  and Arm and matches the reference's order of operations.
* ``oracle/_build/liborion_port.so`` -- the CPU restatement used as the
  test oracle and CPU baseline (test infrastructure, never loaded by the
  product).
* ``oracle/_ref/liborion_ref.so`` -- the reference's own renderer, only when
  the reference tree is present (``ORION_REFERENCE`` or /root/reference).

Objects compile in parallel; a rebuild skips objects newer than their inputs.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "orion_gb300")
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "liborion_gb300.so")
ORACLE = os.path.join(ROOT, "oracle")
PORT_LIB = os.path.join(ORACLE, "_build", "liborion_port.so")
REF_LIB = os.path.join(ORACLE, "_ref", "liborion_ref.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def reference_root() -> str | None:
    r = os.environ.get("ORION_REFERENCE", "/root/reference")
    return r if os.path.isfile(os.path.join(r, "src", "integrator", "path.cpp")) else None


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


def build_port() -> str:
    srcs = sorted(glob.glob(os.path.join(ORACLE, "port", "*.cpp")))
    deps = srcs + glob.glob(os.path.join(ORACLE, "port", "*.h")) + [os.path.join(ORACLE, "cpu_bvh.h"),
                                                                     os.path.join(ROOT, "include", "orion_gpu.h")]
    if not srcs:
        return ""
    os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
    if _stale(PORT_LIB, deps):
        _run(["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-Wall",
              "-o", PORT_LIB, *srcs])
    return PORT_LIB


def build_reference() -> str | None:
    ref = reference_root()
    if ref is None or shutil.which("make") is None:
        return None
    _run(["make", "-s", "-C", os.path.join(ORACLE, "ref"), f"REF={ref}", f"-j{os.cpu_count() or 4}"])
    return REF_LIB


def sobol_table() -> str:
    from orion_gb300 import gen_sobol
    ref = reference_root()
    if ref is not None:
        vals = gen_sobol.extract(os.path.join(ref, "src", "sampler", "sobol.cpp"))
        out = gen_sobol.OUT
        if not os.path.exists(out) or open(out, "rb").read() != __import__("struct").pack("<%dI" % len(vals), *vals):
            gen_sobol.write(vals)
    if not os.path.exists(gen_sobol.OUT):
        raise RuntimeError("missing " + gen_sobol.OUT)
    return gen_sobol.OUT


def build_all(with_reference: bool = True) -> dict:
    out = {"sobol": sobol_table()}
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f_prod = ex.submit(build_product)
        f_port = ex.submit(build_port)
        out["product"] = f_prod.result()
        out["port"] = f_port.result()
    if with_reference:
        out["reference"] = build_reference()
    return out


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build_all())
