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
  bounded sample of the same workload (image rows spread over the whole
  image) on this machine's host cores.
* rmse_vs_oracle -- every result set against the oracle: the GPU film on the
  oracle's sample rows (the same Sobol samples, path for path: relative RMSE
  and the fraction of identical pixels), and a 1024-spp FP64 GPU render
  against the reference's own 65,536-spp FP64 pixel means (tests/golden
  fixtures): fraction of pixels within 3 sigma and relative RMSE.

* batched -- 64 seeded jobs (1-6 displaced icospheres, 1k-500k triangles,
  128^2..1024^2, 4/16/64 spp, depth 4-12): one render call per image against
  one batched graph launch tuned by the batch autotuner; requests/s of each,
  both arms reading FP32 film sums back.
* served -- an open-loop Poisson request stream of 2,000 requests (125
  resident scenes x 16 views) through the serving loop, swept over arrival
  rates of 5-200 req/s: requests/s, Mpaths/s and p50/p95/p99 latency, beside
  the plain per-image path with the scene resident and with the scene built
  and uploaded per image.

N > 1: one process per GPU (launched by torchrun, which sets WORLD_SIZE = N),
independent replicas rendering disjoint sample passes of the same image;
value = all paths / max time. `--gpus N` without N torchrun ranks is an error.

--impl reference: the CPU oracle alone on all host cores, on the same
workload built from the scene generator's arrays in Python (the GPU library
is never loaded in that process).
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
GOLDEN = os.path.join(ROOT, "tests", "golden")
RR_DEFAULT = 3  # the reference's hard-coded `bounces > 3` (src/integrator/path.cpp:91)

WORKLOADS = {
    # name: (scenegen function, kwargs, description, Russian-roulette depth)
    "displaced": ("displaced", {}, "displaced icosphere subdiv 8 (1,310,720 tris) + ground quad, GGX conductor, "
                                   "spot + constant env, 1024x1024, 64 spp, max depth 8, RR after bounce 3",
                  RR_DEFAULT),
    # "No Russian roulette": a path is rouletted only after bounce rr_depth, and
    # with rr_depth = max depth (5) that never happens.
    "cornell": ("cornell", {}, "Cornell box (10,252 tris), 256x256, 16 spp, max depth 5, no Russian roulette", 5),
    "mixed": ("mixed", {}, "8 displaced icospheres (1.27M tris), 5 materials, thin lens, 1920x1080, 128 spp, "
                           "depth 16, RR after bounce 3", RR_DEFAULT),
}
# High-spp FP64 pixel statistics per workload (tests/golden): from the reference renderer itself, except
# for the eight-sphere scene, whose Beckmann plastic the reference cannot render (it has GGX only): that
# fixture comes from the oracle restatement (its "renderer" field says which).
CONVERGED = {"displaced": "fullsize_displaced.npz", "mixed": "fullsize_mixed_beckmann.npz",
             "cornell": "fullsize_cornell.npz"}


def scene_path(workload: str, **override) -> str:
    from orion_gb300 import scenegen
    fn, kw, _, _ = WORKLOADS[workload]
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


def workload_config(workload: str, width: int, height: int, spp: int, max_depth: int, triangles: int) -> dict:
    """The `config` of both arms' JSON lines: the workload alone (no arm- or rank-specific keys)."""
    return {"workload": WORKLOADS[workload][2], "width": width, "height": height, "spp": spp, "max_depth": max_depth,
            "rr_depth": WORKLOADS[workload][3], "paths_per_step": width * height * spp, "triangles": int(triangles),
            "l2": "inputs larger than L2: scene arrays and per-wave path state exceed the 129 MB L2"}


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
NODE_BYTES, TRI_BYTES = 80, 48  # one 8-wide BVH node; one Woop triangle
ALG_BYTES = {
    "trace_ext": 32 + 16,      # ray in (o, d), hit out (t, u, v, prim)
    "trace_shadow": 32 + 4,    # ray in, occlusion flag out
    "trace_mis": 32 + 16,
    "shade": 16 + 96 + 2 * 64,  # hit in, shading record in, path state read + write
    "resolve": 4 * 16 + 16,
    "camera": 64,
    "film": 16 + 16,
}


# ------------------------------------------------------------- parity checks

def _rel_rmse(a: np.ndarray, b: np.ndarray) -> float:
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / max(float(np.sqrt(np.mean(b ** 2))), 1e-30))


def same_sample_parity(gpu_sums: np.ndarray, oracle_sums: np.ndarray) -> dict:
    """GPU film sums against the CPU oracle's on the same pixels and Sobol samples (path for path)."""
    g, c = np.asarray(gpu_sums, np.float64), np.asarray(oracle_sums, np.float64)
    close = (np.abs(g - c) <= 1e-4 * np.abs(c) + 1e-5).all(-1)
    return {"pixels": int(close.size), "pixels_identical": round(float(close.mean()), 6),
            "rel_rmse": _rel_rmse(g, c)}


def converged_parity(ctx, sid: int, workload: str, width: int, height: int, spp: int, host=None,
                     check_spp: int = 1024) -> dict | None:
    """The GPU against the high-spp FP64 per-pixel means of the workload's fixture (1024 seeded pixels;
    65,536 spp):

    matched_rmse: the GPU image at the workload's `spp` and the CPU oracle's image at the same spp (the
      same samples, the same Russian-roulette depth; the oracle is the reference's algorithm pinned bit
      for bit to it), each as relative RMSE against those means; `ratio` = GPU / oracle.
    converged: a `check_spp`-sample FP64 GPU render on sample passes disjoint from the fixture's: the
      fraction of pixels within 3 sigma of the combined Monte Carlo error, and its relative RMSE beside
      the RMSE Monte Carlo noise alone gives."""
    fx = os.path.join(GOLDEN, CONVERGED.get(workload, ""))
    if workload not in CONVERGED or not os.path.exists(fx):
        return None
    g = np.load(fx)
    rr = WORKLOADS[workload][3]
    ref_spp = int(g["spp"])
    pix = g["pix"]
    rmean = g["sum"] / ref_spp
    norm = float(np.sqrt(np.mean(rmean ** 2)))
    out = {"pixels": int(len(pix)), "reference_spp": ref_spp,
           "reference": bytes(g["renderer"]).decode() if "renderer" in g else "reference"}
    s, _ = ctx.render(sid, width, height, spp=spp, rr_depth=rr, fp64=True)
    gpu = s[pix[:, 1], pix[:, 0]] / spp
    e_gpu = float(np.sqrt(np.mean((gpu - rmean) ** 2)) / norm)
    out["matched_rmse"] = {"spp": spp, "gpu_rel_rmse": round(e_gpu, 6)}
    if host is not None:
        try:
            from oracle import port
            o, _ = port.Scene(host).render_pixels(pix, spp, rr_depth=rr)
            e_cpu = float(np.sqrt(np.mean((o / spp - rmean) ** 2)) / norm)
            out["matched_rmse"].update({"oracle_rel_rmse": round(e_cpu, 6), "ratio": round(e_gpu / e_cpu, 5),
                                        "within_1pct": bool(abs(e_gpu / e_cpu - 1) <= 0.01)})
        except OSError as e:  # the oracle library is not built on this machine
            out["matched_rmse"]["oracle"] = f"unavailable: {e}"
    s, q = ctx.render(sid, width, height, spp=check_spp, first_pass=ref_spp, rr_depth=rr, fp64=True)
    s, q = s[pix[:, 1], pix[:, 0]], q[pix[:, 1], pix[:, 0]]
    mean = s / check_spp
    var = np.maximum(q / check_spp - mean ** 2, 0)
    rvar = np.maximum(g["sumsq"] / ref_spp - rmean ** 2, 0)
    sigma2 = var / check_spp + rvar / ref_spp
    z = np.abs(mean - rmean) / (np.sqrt(sigma2) + 1e-7)
    out["converged"] = {"gpu_spp": check_spp, "within_3_sigma": round(float((z <= 3).all(1).mean()), 4),
                        "rel_rmse": round(float(np.sqrt(np.mean((mean - rmean) ** 2)) / norm), 5),
                        "rel_rmse_expected_from_noise": round(float(np.sqrt(np.mean(sigma2)) / norm), 5)}
    return out


# ------------------------------------------------------------------ our arm

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

    rr = WORKLOADS[args.workload][3]
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

    from orion_gb300 import replicas
    first, _ = replicas.pass_range(rank, world, spp)  # replicas render disjoint sample passes
    kw = dict(spp=spp, first_pass=first, rr_depth=rr)
    for _ in range(args.warmup):
        ctx.render(sid, W, H, **kw)

    clocks = ClockSampler(local)
    barrier()
    clocks.start()
    dev_ms, launches, rays = [], 0, 0
    t_wall = time.time()
    film = None
    for _ in range(args.steps):
        film, _cnt = ctx.render(sid, W, H, **kw)
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
    config = workload_config(args.workload, W, H, spp, depth, d.num_prims)

    # End to end through the C ABI: upload scene arrays, render, read the film back (into the
    # caller's film buffers, allocated once as a caller rendering repeatedly would).
    e2e_ms, e2e_parts = [], []
    film_bytes = W * H * (3 * 4 + 4)
    e2e_out = (np.zeros((H, W, 3), np.float32), np.zeros((H, W), np.uint32))
    for i in range(0 if args.quick else max(1, min(args.steps, 7))):
        t = time.time()
        sid2 = ctx.upload(host)
        t1 = time.time()
        ctx.render(sid2, W, H, out=e2e_out, **kw)
        t2 = time.time()
        ctx.release(sid2)
        e2e_ms.append((time.time() - t) * 1e3)
        e2e_parts.append([(t1 - t) * 1e3, (t2 - t1) * 1e3, ctx.last_stats()["device_ms"]])
    e2e_step = float(np.median(e2e_ms)) if e2e_ms else float("nan")
    e2e_split = np.median(np.array(e2e_parts), 0) if e2e_parts else [float("nan")] * 3

    if args.quick:
        ctx.close()
        return {"metric": METRIC, "value": round(value, 3), "unit": "Mpaths/s", "ms_per_step": ms_per_step,
                "config": config} if rank == 0 else None
    # Roofline: one profiled render, per-stage device times.
    ctx.set_profiling(True)
    ctx.render(sid, W, H, **kw)
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
    if os.path.exists(prof_json):  # ncu DRAM bytes per unit, scaled to this run's average launch
        bpu = json.load(open(prof_json)).get("dram_bytes_per_unit")
        if bpu and stages[top]["launches"]:
            traffic = int(bpu * units[top] / stages[top]["launches"])
    roofline = {"bound": "hbm", "kernel": top, "achieved": round(achieved, 2), "peak": peaks["hbm_gbs"],
                "unit": "GB/s", "frac": round(achieved / peaks["hbm_gbs"], 5), "traffic": traffic,
                "peak_source": peaks["source"],
                "alg_bytes_per_unit": ALG_BYTES[top], "units": int(units[top]),
                "launches": stages[top]["launches"], "stage_ms": round(stages[top]["ms"], 3),
                "timing": "one profiled render on one stream, CUDA events around each stage; the trace grids "
                          "keep the production size (6 blocks of 128 threads per SM, leaving the rest of each "
                          "SM to the other waves' shading), which a one-stream render leaves idle"}
    # Model bytes: BVH nodes (80 B) and triangles (48 B) the trace kernels
    # fetch, counted on the device over the workload's first sample pass
    # (1/spp of its paths, every bounce); per ray, then scaled to the timed
    # render's rays of the top kernel's kind.
    kind = {"trace_ext": "ext", "trace_shadow": "shadow", "trace_mis": "mis"}.get(top)
    ctx.set_profiling(og.PROFILE_TRAVERSAL)
    ctx.render(sid, W, H, spp=1, first_pass=first, rr_depth=rr)
    work = ctx.traversal_work()
    ctx.set_profiling(False)
    per_ray = {k: {"nodes": round(w["nodes"] / w["rays"], 2), "triangles": round(w["triangles"] / w["rays"], 2)}
               for k, w in work.items() if w["rays"]}
    model = {"sample": f"1 of {spp} sample passes ({work['ext']['rays']} extension rays), counted on the device",
             "per_ray": per_ray, "node_bytes": NODE_BYTES, "triangle_bytes": TRI_BYTES}
    if kind in per_ray:
        mb = (NODE_BYTES * per_ray[kind]["nodes"] + TRI_BYTES * per_ray[kind]["triangles"]) * units[top]
        model.update({"kernel": top, "bytes_per_launch": int(mb / max(stages[top]["launches"], 1)),
                      "achieved_gbs": round(mb / (stages[top]["ms"] * 1e-3) / 1e9, 1)})
    roofline["model"] = model

    out = {
        "metric": METRIC, "value": round(value, 3), "unit": "Mpaths/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(ms_per_step, 3), "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic: seeded procedural scene generated in-process",
        "config": config, "parallelism": f"replicas x{world}", "scene_bytes": int(scene_bytes),
        "mrays_per_s": round(rays / (total_ms * 1e-3) / 1e6 * world, 2) if total_ms else None,
        "rays_per_path": round(rays / (paths_per_step * args.steps), 4),
        "e2e": {"value": round(paths_per_step / (e2e_step * 1e-3) / 1e6, 3), "unit": "Mpaths/s",
                "ms_per_step": round(e2e_step, 2), "h2d_bytes_per_step": int(scene_bytes),
                "d2h_bytes_per_step": int(film_bytes), "steps": len(e2e_ms),
                "median_split_ms": {"upload": round(float(e2e_split[0]), 2), "render_and_readback": round(float(e2e_split[1]), 2),
                                    "render_device": round(float(e2e_split[2]), 2)}},
        "roofline": roofline,
        "stages_ms": {k: round(v["ms"], 3) for k, v in stages.items()},
        "clocks": clk,
        "gpu_launches": int(launches),
        "host_build_s": round(build_s, 3),
        "wall_s": round(wall, 3),
    }
    if rank == 0:
        out["rmse_vs_oracle"] = converged_parity(ctx, sid, args.workload, W, H, spp,
                                                 host=None if args.no_cpu_baseline else host) or {}
    ctx.release(sid)
    if rank == 0 and not args.no_cpu_baseline:
        cb = cpu_baseline(path, threads=os.cpu_count() or 1, seconds=args.cpu_seconds, rr_depth=rr, keep_film=True)
        if cb.get("film") is not None and first == 0:
            rows = cb.pop("rows")
            out["rmse_vs_oracle"]["same_samples"] = {"rows": int(len(rows)),
                                                     **same_sample_parity(film[rows], cb.pop("film")[rows])}
        cb.pop("film", None)
        cb.pop("rows", None)
        out["cpu_baseline"] = cb
    if rank == 0 and args.batch_jobs > 0:
        out["batched"] = run_batched(ctx, args.batch_jobs, steps=max(1, min(args.steps, 3)), tune_ms=args.tune_ms,
                                     oracle_jobs=0 if args.no_cpu_baseline else 4)
    if rank == 0 and args.serve_scenes > 0:
        out["served"] = run_served(ctx, args.serve_scenes, args.serve_views, args.serve_rates, args.serve_requests,
                                   budget_gb=150.0, spp_chunk=args.spp_chunk, plain_n=args.plain_requests,
                                   oracle_requests=0 if args.no_cpu_baseline else 2)
    if rank == 0 and not args.quick:
        out["other_configs"] = run_other_configs(ctx, cpu_seconds=0.0 if args.no_cpu_baseline else 6.0)
    if rank == 0 and args.sppm_res > 0:
        out["sppm"] = run_sppm(ctx, args.sppm_res, args.sppm_iterations, steps=max(1, min(args.steps, 3)),
                               cpu_iterations=0 if args.no_cpu_baseline else 4)
    ctx.close()
    if dist is not None:
        dist.destroy_process_group()
    return out if rank == 0 else None


def scale_kw(args) -> dict:
    return {"res": getattr(args, "res", None), "spp": getattr(args, "spp", None)}


def cpu_baseline(source, threads: int, seconds: float = 15.0, rr_depth: int = RR_DEFAULT,
                 keep_film: bool = False) -> dict:
    """Time the CPU oracle on a bounded sample of the workload (image rows spread over the image, at its spp)."""
    try:
        from oracle import port
    except Exception as e:  # noqa: BLE001
        return {"value": None, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": f"unavailable: {e}"}
    return port.time_sample(source, threads=threads, seconds=seconds, rr_depth=rr_depth, keep_film=keep_film)


def make_jobs(first_seed: int, n: int) -> list:
    """(scene, host scene) for `n` seeded jobs of the batched/served distribution."""
    from orion_gb300 import scenegen
    out = []
    for i in range(n):
        s = scenegen.job(first_seed + i)
        out.append((s, scenegen.to_host_scene(s)))
    return out


def oracle_film(scene, camera=None, threads: int = 0) -> np.ndarray:
    """The CPU oracle's FP32 film sums of a generated scene (optionally from another camera)."""
    import orion_gb300 as og
    from oracle import port
    from orion_gb300 import scenegen
    kw = scenegen.scene_arrays(scene)
    if camera is not None:
        kw["camera"] = camera
    sc = port.Scene(desc=og.desc_from_arrays(**kw))
    film, _ = sc.render(threads=threads)
    return film


def run_batched(ctx, n_jobs: int, steps: int, tune_ms: float, oracle_jobs: int = 4) -> dict:
    """64 independent jobs: one render call per image (plain) against one batched graph launch.

    Both arms render the same sample indices of the same jobs and read FP32
    film sums back (the batched films are rounded on the device), so their
    images agree to float rounding (matched RMSE by construction;
    rmse_batched_vs_plain checks it on the first jobs, rmse_vs_oracle checks
    `oracle_jobs` small jobs against the CPU oracle). Scenes are resident in
    both arms.
    """
    t0 = time.time()
    jobs = make_jobs(0, n_jobs)
    gen_s = time.time() - t0
    t0 = time.time()
    sids = [ctx.upload(h) for _, h in jobs]
    upload_s = time.time() - t0
    specs = [dict(sid=sid, width=s.width, height=s.height, spp=s.spp) for sid, (s, _) in zip(sids, jobs)]
    paths = sum(s.width * s.height * s.spp for s, _ in jobs)
    tris = [int(h.desc().num_prims) for _, h in jobs]

    # Both arms write every film into host buffers allocated once and reused, so the timed passes
    # compare the renders and their FP32 read-backs, not first-touch page faults of fresh arrays.
    plain_out = [(np.zeros((j["height"], j["width"], 3), np.float32), np.zeros((j["height"], j["width"]), np.uint32))
                 for j in specs]

    def plain_pass():
        t, dev = time.perf_counter(), 0.0
        for j, out in zip(specs, plain_out):
            ctx.render(j["sid"], j["width"], j["height"], spp=j["spp"], out=out)
            dev += ctx.last_stats()["device_ms"]
        return (time.perf_counter() - t) * 1e3, dev

    batch_out = None

    def batch_pass():
        nonlocal batch_out
        t = time.perf_counter()
        batch_out, st = ctx.render_batch(specs, sumsq=False, fp32=True, outs=batch_out)
        return (time.perf_counter() - t) * 1e3, st["device_ms"], st

    plain_pass()  # warm-up
    plain = [plain_pass() for _ in range(steps)]
    plain_cfg = ctx.get_config()
    tuned, tuned_mp = ctx.autotune_batch(specs, spp_cap=4, budget_ms=tune_ms)
    batch_pass()  # warm-up (graph instantiation at the tuned configuration; the output buffers)
    batched = [batch_pass() for _ in range(steps)]
    ctx.set_config(**plain_cfg)  # the legs after this one run at the context's defaults
    p_wall = float(np.median([p[0] for p in plain]))
    b_wall = float(np.median([b[0] for b in batched]))
    p_dev = float(np.median([p[1] for p in plain]))
    b_dev = float(np.median([b[1] for b in batched]))
    # The buffers hold the last pass of each arm.
    rmse = max(_rel_rmse(b, p) for (b, _, _), (p, _) in zip(batch_out[:8], plain_out[:8]))
    oracle = None
    if oracle_jobs > 0:
        order = sorted(range(n_jobs), key=lambda i: jobs[i][0].width * jobs[i][0].height * jobs[i][0].spp
                       + jobs[i][0].num_tris / 10)[:oracle_jobs]
        per = []
        for i in order:
            ref = oracle_film(jobs[i][0], threads=os.cpu_count() or 1)
            per.append({"job": i, **same_sample_parity(batch_out[i][0], ref)})
        oracle = {"jobs": per, "max_rel_rmse": max(p["rel_rmse"] for p in per),
                  "min_pixels_identical": min(p["pixels_identical"] for p in per)}
    # Per-stage device time of each arm (profiling: events around every kernel).
    ctx.set_profiling(True)
    ctx.render_batch(specs, sumsq=False, fp32=True)
    b_stages = {k: round(v["ms"], 2) for k, v in ctx.stage_times().items()}
    p_stages = dict.fromkeys(b_stages, 0.0)
    for j in specs:
        ctx.render(j["sid"], j["width"], j["height"], spp=j["spp"])
        for k, v in ctx.stage_times().items():
            p_stages[k] = round(p_stages[k] + v["ms"], 2)
    ctx.set_profiling(False)
    for sid in sids:
        ctx.release(sid)
    pixels = sum(s.width * s.height for s, _ in jobs)
    return {
        "jobs": n_jobs, "seeds": [0, n_jobs - 1], "paths_per_step": int(paths), "triangles_total": int(sum(tris)),
        "film_readback": f"FP32 sums into reused host buffers, {pixels * 12} bytes per step in both arms "
                         f"(+ {pixels * 4} bytes of counts in the plain arm; the batched arm fills counts on the host)",
        "plain": {"req_s": round(n_jobs / (p_wall * 1e-3), 2), "mpaths_s": round(paths / (p_wall * 1e-3) / 1e6, 2),
                  "wall_ms": round(p_wall, 2), "device_ms": round(p_dev, 2),
                  "device_busy": round(p_dev / p_wall, 3), "launch_calls": n_jobs, "stages_ms": p_stages},
        "batched": {"req_s": round(n_jobs / (b_wall * 1e-3), 2), "mpaths_s": round(paths / (b_wall * 1e-3) / 1e6, 2),
                    "wall_ms": round(b_wall, 2), "device_ms": round(b_dev, 2),
                    "device_busy": round(b_dev / b_wall, 3), "launch_calls": 1,
                    "loop_iterations": int(batched[-1][2]["iterations"]), "slots": int(batched[-1][2]["capacity"]),
                    "stages_ms": b_stages},
        "req_s_ratio": round(p_wall / b_wall, 3),
        # With the plain arm's device busy for device_busy of its wall time, removing every
        # per-image launch and host gap can make it at most 1 / device_busy faster.
        "ratio_bound_from_plain_idle": round(p_wall / p_dev, 3),
        "rmse_batched_vs_plain": rmse,
        "rmse_vs_oracle": oracle,
        "autotuned": {**tuned, "tuning_mpaths_s": round(tuned_mp, 2), "budget_ms": tune_ms, "spp_cap": 4},
        "scene_gen_s": round(gen_s, 2), "upload_build_s": round(upload_s, 2),
    }


def rate_plan(rates: list, total: int) -> list:
    """Requests per arrival rate: `total` split in proportion to the rates, so each rate runs about as long."""
    w = np.asarray(rates, np.float64)
    n = np.maximum(1, np.round(total * w / w.sum())).astype(int)
    n[-1] += total - int(n.sum())
    return [int(x) for x in n]


def run_served(ctx, n_scenes: int, views: int, rates: list, n_requests: int, budget_gb: float, spp_chunk: int,
               plain_n: int, oracle_requests: int = 2) -> dict:
    """Open-loop Poisson request stream through the serving loop, against the plain per-image path.

    Requests are the (scene, view) pairs of `n_scenes` seeded jobs x `views`
    orbit cameras, shuffled with a fixed seed; `n_requests` of them are split
    over the arrival rates in proportion to the rate. A warm-up request per
    scene makes every scene resident first. Latency = completion - submission
    on the server's clock. The plain arms render the first `plain_n` requests
    one orion_gpu_render call each: `plain_resident` with every view's scene
    already uploaded, `plain_cold` uploading (BVH build + copy) per image.
    """
    import orion_gb300 as og
    from orion_gb300 import scenegen
    rng = np.random.default_rng(2024)
    t0 = time.time()
    jobs = make_jobs(1000, n_scenes)
    gen_s = time.time() - t0
    cams = [scenegen.job_views(s, views) for s, _ in jobs]
    reqs = [(i, v) for i in range(n_scenes) for v in range(views)]
    rng.shuffle(reqs)
    srv = og.Server(ctx, memory_budget=int(budget_gb * 1e9), spp_chunk=spp_chunk)
    t0 = time.time()
    warm = [srv.submit(h, spp=s.spp, camera=cams[i][0]) for i, (s, h) in enumerate(jobs)]
    for t in warm:
        srv.wait(t, timeout=900)
        srv.release(t)
    warm_s = time.time() - t0
    sweeps = []
    k = 0
    checked = []
    for rate, count in zip(rates, rate_plan(rates, n_requests)):
        sel = [reqs[(k + j) % len(reqs)] for j in range(count)]
        k += count
        gaps = rng.exponential(1.0 / rate, size=len(sel))
        t0 = time.perf_counter()
        arrive = t0 + np.cumsum(gaps)
        tickets = []
        for (i, v), ta in zip(sel, arrive):
            dt = ta - time.perf_counter()
            if dt > 0:
                time.sleep(dt)
            s, h = jobs[i]
            tickets.append(srv.submit(h, spp=s.spp, camera=cams[i][v]))
        for t in tickets:
            srv.wait(t, timeout=900)
        st = [srv.status(t) for t in tickets]
        if len(checked) < oracle_requests:  # results kept for the oracle check: the smallest requests
            for t, (i, v) in sorted(zip(tickets, sel), key=lambda x: jobs[x[1][0]][0].num_tris)[:oracle_requests]:
                checked.append(((i, v), srv.result(t)[0]))
        for t in tickets:
            srv.release(t)
        lat = np.array([x["t_done"] - x["t_submit"] for x in st]) * 1e3
        span = max(x["t_done"] for x in st) - min(x["t_submit"] for x in st)
        paths = sum(jobs[i][0].width * jobs[i][0].height * jobs[i][0].spp for i, _ in sel)
        sweeps.append({"rate_req_s": rate, "requests": len(sel), "req_s": round(len(sel) / span, 2),
                       "mpaths_s": round(paths / span / 1e6, 2), "p50_ms": round(float(np.percentile(lat, 50)), 1),
                       "p95_ms": round(float(np.percentile(lat, 95)), 1),
                       "p99_ms": round(float(np.percentile(lat, 99)), 1)})
    stats = srv.stats()
    srv.close()
    oracle = None
    if checked:
        per = []
        for (i, v), s in checked[:oracle_requests]:
            ref = oracle_film(jobs[i][0], camera=cams[i][v], threads=os.cpu_count() or 1)
            per.append({"scene": 1000 + i, "view": v, **same_sample_parity(s, ref)})
        oracle = {"requests": per, "max_rel_rmse": max(p["rel_rmse"] for p in per)}

    # Plain per-image path on the first plain_n requests.
    sel = reqs[:plain_n]
    arrays = {i: jobs[i][1].arrays() for i in {i for i, _ in sel}}

    def view_host(i, v):  # the job's scene seen from view v, as a scene of its own
        a = arrays[i]
        return og.HostScene.from_arrays(a["positions"], a["normals"], a["material_of_prim"], a["materials"],
                                        a["lights"], cams[i][v], a["spp"], a["max_depth"],
                                        light_of_prim=a["light_of_prim"])

    def render(sid, i, v):
        ctx.render(sid, cams[i][v].width, cams[i][v].height)

    paths = sum(jobs[i][0].width * jobs[i][0].height * jobs[i][0].spp for i, _ in sel)
    sids = {k: ctx.upload(view_host(*k)) for k in sel}
    for k in sel[:2]:
        render(sids[k], *k)  # warm-up
    t = time.perf_counter()
    for k in sel:
        render(sids[k], *k)
    resident_s = time.perf_counter() - t
    for s in sids.values():
        ctx.release(s)
    cold = {k: view_host(*k) for k in sel}  # no BVH built yet
    t = time.perf_counter()
    for k in sel:
        sid = ctx.upload(cold[k])
        render(sid, *k)
        ctx.release(sid)
    cold_s = time.perf_counter() - t
    best = max(x["req_s"] for x in sweeps)
    plain_resident = len(sel) / resident_s
    plain_cold = len(sel) / cold_s
    return {
        "scenes": n_scenes, "views_per_scene": views, "scene_seeds": [1000, 1000 + n_scenes - 1],
        "requests": n_requests, "budget_gb": budget_gb, "spp_chunk": spp_chunk, "arrivals": "Poisson, seed 2024",
        "sweep": sweeps,
        "plain_resident": {"requests": len(sel), "req_s": round(plain_resident, 2),
                           "mpaths_s": round(paths / resident_s / 1e6, 2)},
        "plain_cold": {"requests": len(sel), "req_s": round(plain_cold, 2),
                       "mpaths_s": round(paths / cold_s / 1e6, 2), "includes": "BVH build + upload per image"},
        # The >=3x target is judged against plain_resident (the scene already on the device); plain_cold
        # also builds and uploads the scene per image, as a one-image-per-run renderer would.
        "target_vs": "plain_resident",
        "served_over_plain_resident": round(best / plain_resident, 3),
        "served_over_plain_cold": round(best / plain_cold, 3),
        "rmse_vs_oracle": oracle,
        "server": {"launches": int(stats["launches"]), "paths": int(stats["paths"]),
                   "device_ms": round(stats["device_ms"], 1), "resident_scenes": int(stats["resident_scenes"])},
        "scene_gen_s": round(gen_s, 2), "warm_s": round(warm_s, 2),
    }


def run_other_configs(ctx, names=("cornell", "mixed"), steps: int = 3, cpu_seconds: float = 0.0) -> dict:
    """The other single-image configurations at their full sizes (C1: Cornell box 256x256, 16 spp, depth 5,
    no Russian roulette; C3: eight displaced icospheres, 5 materials, thin lens, 1920x1080, 128 spp, depth 16):
    device time of a plain render, median of `steps` after one warm-up, with the oracle checks."""
    import orion_gb300 as og
    out = {}
    for name in names:
        rr = WORKLOADS[name][3]
        path = scene_path(name)
        host = og.HostScene.load(path)
        d = host.desc()
        W, H, spp = d.camera.width, d.camera.height, d.spp
        sid = ctx.upload(host)
        ctx.render(sid, W, H, rr_depth=rr)
        ms, rays, film = [], 0, None
        for _ in range(steps):
            film, _ = ctx.render(sid, W, H, rr_depth=rr)
            st = ctx.last_stats()
            ms.append(st["device_ms"])
            rays = st["rays"]
        t = float(np.median(ms))
        out[name] = {"workload": WORKLOADS[name][2], "paths": W * H * spp, "ms": round(t, 2),
                     "mpaths_s": round(W * H * spp / (t * 1e-3) / 1e6, 2), "mrays_s": round(rays / (t * 1e-3) / 1e6, 2),
                     "rays_per_path": round(rays / (W * H * spp), 4), "triangles": int(d.num_prims),
                     "rmse_vs_oracle": converged_parity(ctx, sid, name, W, H, spp,
                                                        host=host if cpu_seconds > 0 else None) or {}}
        ctx.release(sid)
        if cpu_seconds > 0:
            cb = cpu_baseline(path, threads=os.cpu_count() or 1, seconds=cpu_seconds, rr_depth=rr, keep_film=True)
            if cb.get("film") is not None:
                rows = cb.pop("rows")
                out[name]["rmse_vs_oracle"]["same_samples"] = {"rows": int(len(rows)),
                                                               **same_sample_parity(film[rows], cb.pop("film")[rows])}
            out[name]["cpu_baseline"] = cb
    return out


def run_sppm(ctx, res: int, iterations: int, steps: int, cpu_iterations: int) -> dict:
    """SPPM leg: the caustics box (every light type, smooth and rough glass) rendered by
    orion_gpu_render_sppm, against the CPU oracle's restatement of SPPM::render on all host
    threads (atomic photon sums, as the reference runs it) over `cpu_iterations` iterations of
    the same configuration; the GPU renders those iterations too for rmse_vs_oracle."""
    import orion_gb300 as og
    from orion_gb300 import scenegen
    kw = dict(res=res, iterations=iterations, photons=res * res, radius=0.05, max_depth=5, subdiv=5)
    d = os.path.join(tempfile.gettempdir(), "orion_bench_sppm")
    path = scenegen.write_ori(scenegen.caustics(**kw), d)
    host = og.HostScene.load(path)
    sid = ctx.upload(host)
    ctx.render_sppm(sid, res, res, iterations=2)  # warm-up
    ms, rays = [], 0
    for _ in range(steps):
        film, cnt = ctx.render_sppm(sid, res, res)
        st = ctx.last_stats()
        ms.append(st["device_ms"])
        rays = st["rays"]
    short = ctx.render_sppm(sid, res, res, iterations=cpu_iterations)[0] if cpu_iterations > 0 else None
    ctx.release(sid)
    units = iterations * 2 * res * res  # camera paths + photons
    gpu_ms = float(np.median(ms))
    out = {"config": {"workload": f"caustics box SPPM {res}x{res}, {iterations} iterations x {res * res} photons, "
                                  f"radius 0.05, depth 5", "triangles": int(host.desc().num_prims)},
           "gpu": {"ms": round(gpu_ms, 2), "mpaths_s": round(units / (gpu_ms * 1e-3) / 1e6, 2),
                   "mrays_s": round(rays / (gpu_ms * 1e-3) / 1e6, 2), "launches": st["kernel_launches"]},
           "unit": "Mpaths/s (camera paths + photons)", "finite": bool(np.isfinite(film).all())}
    if cpu_iterations <= 0:
        return out
    try:
        from oracle import port
        sc = port.Scene(host)
        cores = os.cpu_count() or 1
        t = time.time()
        cfilm, _ = sc.render_sppm(iterations=cpu_iterations, threads=cores)
        cpu_s = time.time() - t
        cu = cpu_iterations * 2 * res * res
        out["cpu_baseline"] = {"value": round(cu / cpu_s / 1e6, 4), "cores": cores, "kind": "port",
                               "sample": f"{cpu_iterations} of the {iterations} iterations on {cores} threads "
                                         f"(atomic photon sums, as the reference), {cpu_s:.2f} s"}
        out["gpu_vs_cpu"] = round(out["gpu"]["mpaths_s"] / out["cpu_baseline"]["value"], 1)
        out["rmse_vs_oracle"] = {"iterations": cpu_iterations, **same_sample_parity(short, cfilm)}
    except Exception as e:  # the oracle is optional on a machine without its build
        out["cpu_baseline"] = {"unavailable": str(e)[:200]}
    return out


# ------------------------------------------------------------ reference arm

def run_reference(args) -> dict | None:
    """The CPU oracle alone on all host cores (rank 0 only). The workload is built from the scene
    generator's arrays in Python, so this process never loads the GPU library."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return None
    threads = os.cpu_count() or 1
    try:
        from oracle import port
        port.lib()
    except Exception as e:  # noqa: BLE001
        return {"impl": "reference", "unavailable": f"CPU oracle library not built: {e}"}
    from orion_gb300 import scenegen
    fn, kw, _, rr = WORKLOADS[args.workload]
    scene = getattr(scenegen, fn)(**kw)
    t0 = time.time()
    sc = port.Scene.from_generated(scene)
    build_s = time.time() - t0
    config = workload_config(args.workload, scene.width, scene.height, scene.spp, scene.max_depth, scene.num_tris)
    # Size one step's sample (rows spread over the image) to about `step_s` on all cores; each
    # sample pass runs its rows in parallel (PathTracing::render's loop), so at least 4 rows a thread.
    n, step_s = min(sc.height, 4 * threads), max(0.5, args.cpu_seconds / 5)
    while True:
        rows = port.spread_rows(n, sc.height)
        t = time.time()
        sc.render(rows=rows, threads=threads, rr_depth=rr)
        dt = time.time() - t
        want = min(sc.height, int(n * step_s / max(dt, 1e-3)))
        if dt >= 0.7 * step_s or len(rows) >= sc.height or want <= n:
            break
        n = want
    for _ in range(max(0, args.warmup - 1)):
        sc.render(rows=rows, threads=threads, rr_depth=rr)
    vals, rays = [], 0
    t_all = time.time()
    for _ in range(args.steps):
        t = time.time()
        _, rays = sc.render(rows=rows, threads=threads, rr_depth=rr)
        vals.append(len(rows) * sc.width * sc.spp / (time.time() - t) / 1e6)
    wall = time.time() - t_all
    v = round(float(np.median(vals)), 4)
    paths = len(rows) * sc.width * sc.spp
    sample = (f"{len(rows)} image rows spread over all {sc.height} x {sc.width} px x {sc.spp} spp = {paths} paths "
              f"per step, median of {args.steps} steps, {rays} rays per step")
    return {"impl": "reference", "metric": METRIC, "value": v, "unit": "Mpaths/s", "n_gpus": 0, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(wall / args.steps * 1e3, 1), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic: seeded procedural scene generated in-process", "config": config,
            "rays_per_path": round(rays / paths, 4), "scene_build_s": round(build_s, 2),
            "cpu_baseline": {"value": v, "unit": "Mpaths/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="displaced", choices=sorted(WORKLOADS))
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true", help="skip every CPU oracle leg and check")
    ap.add_argument("--res", type=int, help="scale the workload down: square image side (profiling runs)")
    ap.add_argument("--spp", type=int, help="scale the workload down: samples per pixel (profiling runs)")
    ap.add_argument("--quick", action="store_true", help="timed steps only: no e2e, roofline or CPU legs")
    ap.add_argument("--batch-jobs", type=int, default=64, help="batched leg: jobs per launch (0 = skip)")
    ap.add_argument("--tune-ms", type=float, default=6000.0, help="batched leg: autotuner budget (device ms)")
    ap.add_argument("--serve-scenes", type=int, default=125, help="served leg: resident scenes (0 = skip)")
    ap.add_argument("--serve-views", type=int, default=16)
    ap.add_argument("--serve-rates", type=float, nargs="+", default=[5.0, 20.0, 50.0, 100.0, 200.0])
    ap.add_argument("--serve-requests", type=int, default=2000, help="served leg: requests over all arrival rates")
    # 16: 146 req/s saturated and p50 8.5 ms at 50 req/s, against 137 req/s and 16.4 ms with chunks of 4
    ap.add_argument("--spp-chunk", type=int, default=16, help="served leg: progressive spp per pass")
    ap.add_argument("--plain-requests", type=int, default=32, help="served leg: requests timed on the plain path")
    ap.add_argument("--batch-only", action="store_true", help="run the batched leg alone (profiling)")
    ap.add_argument("--sppm-res", type=int, default=512, help="SPPM leg: image side (0 = skip)")
    ap.add_argument("--sppm-iterations", type=int, default=16)
    ap.add_argument("--sppm-only", action="store_true", help="run the SPPM leg alone (profiling)")
    args = ap.parse_args()
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.gpus != world:
        sys.exit(f"bench.py: --gpus {args.gpus} but {world} process(es): launch N > 1 as "
                 f"`python -m torch.distributed.run --nproc-per-node {args.gpus} --master-addr 127.0.0.1 bench.py "
                 f"--gpus {args.gpus}` (one replica per GPU)")
    if args.quick:
        args.batch_jobs = args.serve_scenes = args.sppm_res = 0
    from oracle import build as oracle_build
    from orion_gb300 import build
    oracle_build.build_port()  # the CPU baseline and the parity checks
    if args.impl == "reference":
        out = run_reference(args)
        if out is not None:
            print(json.dumps(out), flush=True)
        return
    build.build_product()
    if args.sppm_only:  # profiling runs of the SPPM leg alone
        import orion_gb300 as og
        ctx = og.Context(0)
        print(json.dumps(run_sppm(ctx, args.sppm_res or 512, args.sppm_iterations, steps=max(1, args.steps),
                                  cpu_iterations=0)))
        ctx.close()
        return
    if args.batch_only:  # profiling runs of the batched engine alone
        import orion_gb300 as og
        ctx = og.Context(0)
        print(json.dumps(run_batched(ctx, args.batch_jobs or 64, steps=max(1, args.steps), tune_ms=args.tune_ms,
                                     oracle_jobs=0)))
        ctx.close()
        return
    out = run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
