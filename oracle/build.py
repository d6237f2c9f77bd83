"""Build the test oracle (test infrastructure only; the product never loads it).

* ``oracle/_build/liborion_port.so`` -- the CPU restatement of the
  reference's path-tracing code (oracle/port/port.cpp): the checker of the
  GPU tests and the timed CPU baseline.
* ``oracle/_ref/liborion_ref.so`` -- the reference renderer itself, compiled
  from its sources in place by oracle/ref/Makefile, only where the reference
  tree is present: ``$ORION_REFERENCE``, else a directory named ``reference``
  beside the repository.

Both use -O3 without -march (the same flags on x86 and Arm) and
-ffp-contract=off, so the restatement rounds as the reference does.

    python -m oracle.build
"""
from __future__ import annotations

import glob
import os
import shutil
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ORACLE = os.path.join(ROOT, "oracle")
PORT_LIB = os.path.join(ORACLE, "_build", "liborion_port.so")
REF_LIB = os.path.join(ORACLE, "_ref", "liborion_ref.so")
CXXFLAGS = ["-std=c++17", "-O3", "-fPIC", "-fopenmp", "-ffp-contract=off", "-Wall"]


def reference_root() -> str | None:
    """The reference source tree, or None where it is absent."""
    r = os.environ.get("ORION_REFERENCE") or os.path.join(os.path.dirname(ROOT), "reference")
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


def build_port() -> str:
    srcs = sorted(glob.glob(os.path.join(ORACLE, "port", "*.cpp")))
    deps = srcs + glob.glob(os.path.join(ORACLE, "port", "*.h")) + [os.path.join(ORACLE, "cpu_bvh.h"),
                                                                     os.path.join(ROOT, "include", "orion_gpu.h"),
                                                                     os.path.abspath(__file__)]
    if not srcs:
        return ""
    os.makedirs(os.path.dirname(PORT_LIB), exist_ok=True)
    if _stale(PORT_LIB, deps):
        _run(["g++", *CXXFLAGS, "-shared", "-o", PORT_LIB, *srcs])
    return PORT_LIB


def build_reference() -> str | None:
    """The reference renderer and its adapter test, where the reference tree is present."""
    ref = reference_root()
    if ref is None or shutil.which("make") is None:
        return None
    _run(["make", "-s", "-C", os.path.join(ORACLE, "ref"), f"REF={ref}", f"-j{os.cpu_count() or 4}"])
    return REF_LIB


def build_all(with_reference: bool = True) -> dict:
    out = {"port": build_port()}
    if with_reference:
        out["reference"] = build_reference()
    return out


if __name__ == "__main__":
    sys.path.insert(0, ROOT)
    print(build_all())
