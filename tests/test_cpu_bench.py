"""The benchmark's reference arm (`bench.py --impl reference`): the CPU oracle
timed on the host cores, printing the same JSON line as the GPU arm. It needs
no GPU, so its contract is checked here on a small workload."""
from __future__ import annotations

import json
import subprocess
import sys

import helpers


def test_reference_arm_prints_one_contract_line(built):
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--workload", "cornell",
           "--steps", "2", "--warmup", "1", "--cpu-seconds", "1"]
    out = subprocess.run(cmd, cwd=helpers.ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "Mpaths/s" and d["higher_is_better"] is True
    assert d["steps"] == 2 and d["warmup"] == 1 and d["value"] > 0
    cfg = d["config"]
    assert (cfg["width"], cfg["height"], cfg["spp"], cfg["max_depth"]) == (256, 256, 16, 5)
    assert cfg["rr_depth"] >= cfg["max_depth"]  # the Cornell workload renders without Russian roulette
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and "rows" in cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
