"""Test oracle for the GPU path tracer (test infrastructure, never shipped).

* ``oracle.port``  -- ctypes wrapper of oracle/port/port.cpp, the CPU
  restatement of the reference's path-tracing code (built into
  oracle/_build/liborion_port.so by orion_gb300.build).
* oracle/ref       -- recipe that compiles the reference renderer itself into
  oracle/_ref/liborion_ref.so where its sources exist; used to pin the
  restatement and to generate tests/golden.
* oracle/cpu_bvh.h -- the CPU closest-hit kernel both use in Embree's place.

Only tests/, the smoke check and bench.py's CPU-baseline leg import this.
"""
