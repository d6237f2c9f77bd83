"""Extract the Sobol generator matrices into orion_gb300/data/sobol_matrices.bin.

The sampler must be bit-exact with the reference's ``sobol::sample``
(src/sampler/sobol.h:28-43), which XORs the 1024 x 52 table of 32-bit
direction numbers in src/sampler/sobol.cpp (S. Joe and F. Y. Kuo,
"Constructing Sobol sequences with better two-dimensional projections",
SIAM J. Sci. Comput. 30, 2635-2654, 2008; direction numbers
new-joe-kuo-6.21201). The numbers are data, not code: this script reads them
from the reference tree and writes them as little-endian uint32, dimension
major, 52 per dimension.

    python -m orion_gb300.gen_sobol /path/to/orion/src/sampler/sobol.cpp
"""
from __future__ import annotations

import os
import re
import struct
import sys

DIMS, BITS = 1024, 52
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "data", "sobol_matrices.bin")


def extract(sobol_cpp: str) -> list[int]:
    text = open(sobol_cpp).read()
    start = text.index("matrices[Matrices::num_dimensions * Matrices::size]")
    body = text[start:text.index("};", start)]
    vals = [int(h, 16) for h in re.findall(r"0x([0-9a-fA-F]+)U", body)]
    if len(vals) != DIMS * BITS:
        raise ValueError(f"expected {DIMS * BITS} direction numbers, found {len(vals)}")
    return vals


def write(vals: list[int], out: str = OUT) -> str:
    os.makedirs(os.path.dirname(out), exist_ok=True)
    with open(out, "wb") as f:
        f.write(struct.pack("<%dI" % len(vals), *vals))
    return out


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python -m orion_gb300.gen_sobol /path/to/orion/src/sampler/sobol.cpp")
    print(write(extract(sys.argv[1])))
