"""Benchmark: the plain GPU path tracer on the large displaced-mesh workload.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload NAME]

One step = one Integrator::render() of the workload: 1024x1024 pixels x 64
samples (67.1M camera paths) of a 1,310,720-triangle displaced icosphere on a
ground quad, GGX conductor, spotlight + constant environment, depth 8,
Russian roulette after bounce 3.

* value  -- Mpaths/s with the scene resident in HBM, device time of the
  render's kernels (CUDA events on the library's stream).
* e2e    -- the same step through the C ABI from host buffers: scene arrays
  copied host->device, render, film copied device->host, per step.
* roofline -- the kernel with the largest share of device time, its
  algorithmic bytes per launch over its measured time, against the measured
  HBM copy bandwidth.
* cpu_baseline -- the CPU oracle (the reference's algorithm restated in C++,
  one path per OpenMP thread, project CPU BVH in Embree's place) timed on a
  bounded sample of the same workload on this machine's host cores.

N > 1: one process per GPU (torchrun), independent replicas rendering
disjoint sample passes of the same image; value = all paths / max time.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Mpaths/s and served req/s with p50/p99 latency vs plain path, at matched RMSE"
CACHE = os.path.join(tempfile.gettempdir(), "orion_gb300_scenes")

WORKLOADS = {
    # name: (scenegen function, kwargs, description)
    "displaced": ("displaced", {}, "displaced icosphere subdiv 8 (1,310,720 tris) + ground quad, GGX conductor, "
                                   "spot + constant env, 1024x1024, 64 spp, max depth 8, RR after bounce 3"),
    "cornell": ("cornell", {}, "Cornell box (10,252 tris), 256x256, 16 spp, max depth 5"),
    "mixed": ("mixed", {}, "8 displaced icospheres (1.27M tris), 5 materials, thin lens, 1920x1080, 128 spp, depth 16"),
}


def scene_path(workload: str, **override) -> str:
    from orion_gb300 import scenegen
    fn, kw, _ = WORKLOADS[workload]
    kw = {**kw, **{k: v for k, v in override.items() if v is not None}}
    tag = "_".join(f"{k}{v}" for k, v in sorted(kw.items()))
    d = os.path.join(CACHE, workload + ("_" + tag if tag else ""))
    marker = os.path.join(d, "done")
    if not os.path.exists(marker):
        s = getattr(scenegen, fn)(**kw)
        path = scenegen.write_ori(s, d)
        with open(marker, "w") as f:
            f.write(path)
    return open(marker).read().strip()


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


# Algorithmic bytes per unit of work (one ray or one path), independent of
# BVH quality: what the stage must read and write at minimum.
ALG_BYTES = {
    "trace_ext": 32 + 16,      # ray in (o, d), hit out (t, u, v, prim)
    "trace_shadow": 32 + 4,    # ray in, occlusion flag out
    "trace_mis": 32 + 16,
    "shade": 16 + 96 + 2 * 64,  # hit in, shading record in, path state read + write
    "resolve": 4 * 16 + 16,
    "camera": 64,
    "film": 16 + 16,
}


def cpu_baseline(workload: str, threads: int, seconds: float = 15.0) -> dict | None:
    """Time the CPU oracle on a bounded sample of the workload (rows of the image at its spp)."""
    try:
        from oracle import port
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": f"unavailable: {e}"}
    return port.time_sample(scene_path(workload), threads=threads, seconds=seconds)


def scale_kw(args) -> dict:
    return {"res": getattr(args, "res", None), "spp": getattr(args, "spp", None)}


def run_ours(args) -> dict:
    import orion_gb300 as og
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist
        torch.cuda.set_device(local)
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))

    path = scene_path(args.workload, **scale_kw(args))
    host = og.HostScene.load(path)
    d = host.desc()
    W, H, spp, depth = d.camera.width, d.camera.height, d.spp, d.max_depth
    ctx = og.Context(local)
    t0 = time.time()
    sid = ctx.upload(host)
    build_s = time.time() - t0
    scene_bytes = ctx.scene_bytes(sid)
    paths_per_step = W * H * spp

    def barrier():
        if dist is not None:
            import torch
            torch.cuda.synchronize()
            dist.barrier()

    first = rank * spp  # replicas render disjoint sample passes
    for _ in range(args.warmup):
        ctx.render(sid, W, H, spp=spp, first_pass=first)

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    dev_ms, launches, rays = [], 0, 0
    t_wall = time.time()
    for _ in range(args.steps):
        ctx.render(sid, W, H, spp=spp, first_pass=first)
        st = ctx.last_stats()
        dev_ms.append(st["device_ms"])
        launches += st["kernel_launches"]
        rays += st["rays"]
    wall = time.time() - t_wall
    clk = clocks.stop()
    barrier()
    total_ms = float(np.sum(dev_ms))
    if dist is not None:
        import torch
        t = torch.tensor([total_ms], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    ms_per_step = total_ms / args.steps
    value = paths_per_step * world / (ms_per_step * 1e-3) / 1e6

    # End to end through the C ABI: upload scene arrays, render, read the film back.
    e2e_ms = []
    film_bytes = W * H * (3 * 4 + 4)
    for i in range(0 if args.quick else max(1, min(args.steps, 5))):
        t = time.time()
        sid2 = ctx.upload(host)
        img, cnt = ctx.render(sid2, W, H, spp=spp, first_pass=first)
        ctx.release(sid2)
        e2e_ms.append((time.time() - t) * 1e3)
    e2e_step = float(np.median(e2e_ms)) if e2e_ms else float("nan")

    if args.quick:
        ctx.close()
        return {"metric": METRIC, "value": round(value, 3), "unit": "Mpaths/s", "ms_per_step": ms_per_step,
                "config": {"workload": args.workload, "scale": scale_kw(args)}} if rank == 0 else None
    # Roofline: one profiled render, per-stage device times.
    ctx.set_profiling(True)
    ctx.render(sid, W, H, spp=spp, first_pass=first)
    stages = ctx.stage_times()
    st = ctx.last_stats()
    ctx.set_profiling(False)
    units = {"trace_ext": st["ext_rays"], "trace_shadow": st["shadow_rays"], "trace_mis": st["mis_rays"],
             "shade": st["ext_rays"], "resolve": st["shadow_rays"], "camera": st["paths"], "film": st["paths"]}
    top = max((k for k in stages if k in ALG_BYTES), key=lambda k: stages[k]["ms"])
    peaks = measured_peaks()
    alg_bytes = ALG_BYTES[top] * units[top]
    achieved = alg_bytes / (stages[top]["ms"] * 1e-3) / 1e9
    traffic = None
    prof_json = os.path.join(ROOT, "profiles", f"{top}_{args.workload}.json")
    if os.path.exists(prof_json):
        traffic = json.load(open(prof_json)).get("dram_bytes_per_launch")
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 5), "traffic": traffic,
                "peak_source": peaks["source"],
                "alg_bytes_per_unit": ALG_BYTES[top], "units": int(units[top]),
                "launches": stages[top]["launches"], "stage_ms": round(stages[top]["ms"], 3)}

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded procedural scene generated in-process",
        "config": {"workload": WORKLOADS[args.workload][2], "paths_per_step": paths_per_step,
                   "triangles": int(d.num_prims), "l2": "inputs larger than L2 (scene "
                   f"{scene_bytes / 1e6:.0f} MB + path state per wave)", "parallelism": f"replicas x{world}"},
        "mrays_per_s": round(rays / (total_ms * 1e-3) / 1e6 * world, 2) if total_ms else None,
        "e2e": {"value": round(paths_per_step / (e2e_step * 1e-3) / 1e6, 3), "unit": "Mpaths/s",
                "ms_per_step": round(e2e_step, 2), "h2d_bytes_per_step": int(scene_bytes),
                "d2h_bytes_per_step": int(film_bytes)},
        "roofline": roofline,
        "stages_ms": {k: round(v["ms"], 3) for k, v in stages.items()},
        "clocks": clk,
        "gpu_launches": int(launches),
        "host_build_s": round(build_s, 3),
        "wall_s": round(wall, 3),
    }
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args.workload, threads=os.cpu_count() or 1, seconds=args.cpu_seconds)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return out if rank == 0 else None


def run_reference(args) -> dict | None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    try:
        from oracle import port
    except Exception as e:  # noqa: BLE001
        return {"impl": "reference", "unavailable": f"CPU oracle library not built: {e}"}
    path = scene_path(args.workload)
    for _ in range(args.warmup):
        port.time_sample(path, threads=threads, seconds=1.0)
    vals = []
    t = time.time()
    for _ in range(args.steps):
        r = port.time_sample(path, threads=threads, seconds=args.cpu_seconds)
        vals.append(r["value"])
    wall = time.time() - t
    v = float(np.median(vals))
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mpaths/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOADS[args.workload][2]},
            "cpu_baseline": {"value": v, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": r["sample"]},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="displaced", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--res", type=int, help="scale the workload down: square image side (profiling runs)")
    ap.add_argument("--spp", type=int, help="scale the workload down: samples per pixel (profiling runs)")
    ap.add_argument("--quick", action="store_true", help="timed steps only: no e2e, roofline or CPU legs")
    args = ap.parse_args()
    from orion_gb300 import build
    build.build_product()
    build.build_port()
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
