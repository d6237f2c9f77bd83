"""Batched rendering (many jobs, one graph launch) against the plain path.

Each path runs the plain render's device functions on the same samples; the
batched and plain shading kernels are compiled separately, so the compiler
may contract different multiply-adds, and a path's FP32 radiance can differ
in its last bits. Per-pixel FP64 sums must agree with the plain FP64 render
to 1e-5 relative (FP32 rounding), counts exactly. Within the batched engine
(same kernels), the same job must give the same result to 1e-12 alone and in
a mix of other jobs, and with a pool of slots far smaller than its path
count (heavy slot regeneration).
"""
from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

SCENES = [("cornell", dict(res=48, spp=8)), ("zoo", dict(res=40, spp=4, beckmann=True)),
          ("mixed", dict(width=64, height=36, spp=4, subdivs=(2, 2, 2, 2, 2, 2, 2, 2))),
          ("displaced", dict(res=32, spp=6, subdiv=4)), ("textured", dict(res=32, spp=4, subdiv=2))]


@pytest.fixture(scope="module")
def scenes(ctx, tmp_path_factory):
    import orion_gb300 as og
    d = tmp_path_factory.mktemp("batch")
    out = []
    for name, kw in SCENES:
        host = og.HostScene.load(helpers.write_scene(name, str(d / name), **kw))
        desc = host.desc()
        out.append(dict(name=name, host=host, sid=ctx.upload(host), width=desc.camera.width,
                        height=desc.camera.height, spp=desc.spp))
    yield out
    for s in out:
        ctx.release(s["sid"])


@pytest.fixture(params=["pooled", "waves"])
def mode(ctx, request):
    """Both batch modes: a refilled pool of path slots, and waves over the jobs' work list."""
    import orion_gb300 as og
    m = og.BATCH_POOLED if request.param == "pooled" else og.BATCH_WAVES
    ctx.set_batch_mode(m)
    yield request.param
    ctx.set_batch_mode(og.BATCH_WAVES)


def _job(s, **kw):
    return dict(sid=s["sid"], width=s["width"], height=s["height"], **kw)


def _close(a, b, rtol=1e-12):
    return np.all(np.abs(a - b) <= rtol * np.abs(b) + 1e-12)


def test_batch_matches_plain_fp64(ctx, scenes, mode):
    outs, st = ctx.render_batch([_job(s) for s in scenes])
    assert st["paths"] == sum(s["width"] * s["height"] * s["spp"] for s in scenes)
    for s, (sm, sq, cnt) in zip(scenes, outs):
        ps, pq = ctx.render(s["sid"], s["width"], s["height"], fp64=True)
        assert (cnt == s["spp"]).all(), s["name"]
        assert np.allclose(sm, ps, rtol=1e-5, atol=1e-7), f"{s['name']}: max diff {np.abs(sm - ps).max()}"
        assert np.allclose(sq, pq, rtol=1e-5, atol=1e-7), s["name"]
    print(f"{mode} batch of {len(scenes)} jobs: {st['iterations']} loop iterations, {st['paths']} paths, "
          f"{st['device_ms']:.2f} ms")


def test_job_alone_equals_job_in_mix(ctx, scenes, mode):
    alone, _ = ctx.render_batch([_job(scenes[1])])
    mix, _ = ctx.render_batch([_job(scenes[0]), _job(scenes[1]), _job(scenes[2]), _job(scenes[1], first_pass=4)])
    assert _close(mix[1][0], alone[0][0]) and np.array_equal(mix[1][2], alone[0][2])
    # the same scene with other sample passes is a different estimate of the same image
    assert not np.array_equal(mix[3][0], mix[1][0])


def test_small_pool_forces_regeneration(ctx, scenes, mode):
    cfg = ctx.get_config()
    try:
        ctx.set_config(batch_slots=2048)
        outs, st = ctx.render_batch([_job(s) for s in scenes])
        assert st["capacity"] <= 1 << 22
    finally:
        ctx.set_config(**cfg)
    ref, _ = ctx.render_batch([_job(s) for s in scenes])
    for (a, _, c1), (b, _, c2) in zip(outs, ref):
        assert np.array_equal(c1, c2)
        assert _close(a, b)


def test_config_limits_and_large_stacks(ctx, scenes):
    import orion_gb300 as og
    cfg = ctx.get_config()
    with pytest.raises(og.OrionError, match="shared memory|trace_block"):
        ctx.set_config(trace_block=1024, smem_stack=32)  # 256 KB of stack per block (or too many threads)
    with pytest.raises(og.OrionError, match="trace_block"):
        ctx.set_config(trace_block=100)
    assert ctx.get_config() == cfg
    ref, _ = ctx.render_batch([_job(s) for s in scenes])
    try:
        ctx.set_config(trace_block=256, smem_stack=32)  # 64 KB: above the 48 KB default, allowed by opt-in
        outs, _ = ctx.render_batch([_job(s) for s in scenes])
        img, cnt = ctx.render(scenes[0]["sid"], scenes[0]["width"], scenes[0]["height"])
    finally:
        ctx.set_config(**cfg)
    ref_img, ref_cnt = ctx.render(scenes[0]["sid"], scenes[0]["width"], scenes[0]["height"])
    assert np.array_equal(cnt, ref_cnt) and np.allclose(img, ref_img, rtol=1e-5, atol=1e-6)
    for (a, _, c1), (b, _, c2) in zip(outs, ref):
        assert np.array_equal(c1, c2)
        assert np.allclose(a, b, rtol=1e-5, atol=1e-9)


def test_batch_autotuner(ctx, scenes):
    cfg = ctx.get_config()
    try:
        best, mpaths = ctx.autotune_batch([_job(s) for s in scenes], spp_cap=2, budget_ms=300.0)
        assert mpaths > 0 and best["batch_slots"] >= 1024
        assert ctx.get_config()["trace_block"] == best["trace_block"]
        outs, _ = ctx.render_batch([_job(s) for s in scenes])
    finally:
        ctx.set_config(**cfg)
    ref, _ = ctx.render_batch([_job(s) for s in scenes])
    for (a, _, c1), (b, _, c2) in zip(outs, ref):
        assert np.array_equal(c1, c2)
        assert np.allclose(a, b, rtol=1e-5, atol=1e-9)
    print(f"batch autotuner: {best}, {mpaths:.1f} Mpaths/s")


def test_profiled_batch_matches_graph_batch(ctx, scenes, mode):
    ref, _ = ctx.render_batch([_job(s) for s in scenes])
    ctx.set_profiling(True)
    try:
        outs, st = ctx.render_batch([_job(s) for s in scenes])
        stages = ctx.stage_times()
    finally:
        ctx.set_profiling(False)
    for (a, q1, c1), (b, q2, c2) in zip(outs, ref):
        assert np.array_equal(c1, c2)
        assert _close(a, b) and _close(q1, q2)
    assert stages["shade"]["launches"] >= st["iterations"] and stages["trace_ext"]["ms"] > 0


def test_modes_give_the_same_films(ctx, scenes):
    """Both modes trace every path with the same samples; only the FP64 film's order of additions differs."""
    import orion_gb300 as og
    try:
        ctx.set_batch_mode(og.BATCH_POOLED)
        pooled, _ = ctx.render_batch([_job(s) for s in scenes])
        ctx.set_batch_mode(og.BATCH_WAVES)
        cfg = ctx.get_config()
        ctx.set_config(batch_slots=4096)  # many waves
        waves, st = ctx.render_batch([_job(s) for s in scenes])
    finally:
        ctx.set_config(**cfg)
        ctx.set_batch_mode(og.BATCH_WAVES)
    for (a, q1, c1), (b, q2, c2) in zip(pooled, waves):
        assert np.array_equal(c1, c2)
        assert _close(a, b) and _close(q1, q2)


def test_batch_iteration_cap_is_reported(ctx, scenes, mode):
    """A batch loop stopped by its iteration bound returns ORION_ERR_DEVICE (no hang, no partial result
    reported as success), and the next batch on the same context renders normally."""
    import orion_gb300 as og
    jobs = [_job(s) for s in scenes]
    before, _ = ctx.render_batch(jobs)
    try:
        ctx.set_test_limits(batch_iterations=2)
        with pytest.raises(og.OrionError, match="iteration cap") as e:
            ctx.render_batch(jobs)
        assert e.value.code == -7
    finally:
        ctx.set_test_limits()
    after, _ = ctx.render_batch(jobs)
    for (a, _, ca), (b, _, cb) in zip(before, after):
        assert _close(a, b) and np.array_equal(ca, cb)


def test_batch_fp32_readback(ctx, scenes, mode):
    """orion_job.sum32: the FP64 sums rounded to FP32 on the device (FP64 atomics add in any order, so
    two batches' sums agree to FP64 rounding and their FP32 roundings to one FP32 step)."""
    jobs = [_job(s) for s in scenes]
    f64, _ = ctx.render_batch(jobs, sumsq=False)
    f32, _ = ctx.render_batch(jobs, fp32=True)
    for (a, _, ca), (b, q, cb) in zip(f64, f32):
        assert b.dtype == np.float32 and q is None
        assert np.all(np.abs(a - b) <= 2.0 ** -23 * np.abs(a) + 1e-30) and np.array_equal(ca, cb)
