"""Wave scheduling: a render is split into waves of path slots, and consecutive
waves run on two streams. Every pixel's film sum is taken in sample order
(RenderTarget::acumulate, src/texture/rendertarget.cpp:22-27), so the film
must be bit-identical whatever the wave size, whether waves overlap on two
streams or run on one (profiled renders), and from run to run."""
from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scene(ctx, tmp_path_factory):
    import orion_gb300 as og
    path = helpers.write_scene("zoo", str(tmp_path_factory.mktemp("waves") / "zoo"), res=48, spp=12)
    host = og.HostScene.load(path)
    sid = ctx.upload(host)
    yield sid
    ctx.release(sid)


def test_film_independent_of_waves_and_streams(ctx, scene):
    total = 48 * 48 * 12
    ref, cnt = ctx.render(scene, 48, 48, wave_paths=total)  # one wave, one stream
    assert (cnt == 12).all()
    cfg = ctx.get_config()
    try:
        for streams in (1, 2, 3, 4):
            ctx.set_config(streams=streams)
            for wave in (4096, 3001, 48 * 48):
                img, c = ctx.render(scene, 48, 48, wave_paths=wave)  # several waves on `streams` streams
                assert np.array_equal(c, cnt)
                assert np.array_equal(img.view(np.uint32), ref.view(np.uint32)), f"wave {wave}, {streams} streams"
    finally:
        ctx.set_config(**cfg)
    # FP64 sums of squares are grouped by wave (rounding depends on the wave size), so the FP64
    # film is compared at one wave size: two streams against one.
    s1, q1 = ctx.render(scene, 48, 48, wave_paths=5000, fp64=True)
    ctx.set_profiling(True)
    try:
        img, _ = ctx.render(scene, 48, 48, wave_paths=4096)  # profiled: one stream
        s2, q2 = ctx.render(scene, 48, 48, wave_paths=5000, fp64=True)
    finally:
        ctx.set_profiling(False)
    assert np.array_equal(s1, s2) and np.array_equal(q1, q2)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    ctx.render(scene, 48, 48, wave_paths=4096)
    st = ctx.last_stats()
    again, _ = ctx.render(scene, 48, 48, wave_paths=4096)
    assert np.array_equal(again.view(np.uint32), ref.view(np.uint32))
    assert ctx.last_stats()["rays"] == st["rays"]


def test_traversal_work_counts(ctx, scene):
    """A counting render traces the same rays into the same film and reports
    per-kind BVH work: every ray visits the root node at least."""
    import orion_gb300 as og
    ref, _ = ctx.render(scene, 48, 48, wave_paths=4096)
    assert all(v == 0 for k in ctx.traversal_work().values() for v in k.values())
    ctx.set_profiling(og.PROFILE_TRAVERSAL)
    try:
        img, _ = ctx.render(scene, 48, 48, wave_paths=4096)
        st = ctx.last_stats()
        work = ctx.traversal_work()
        ctx.set_profiling(og.PROFILE_STAGES | og.PROFILE_TRAVERSAL)
        both, _ = ctx.render(scene, 48, 48, wave_paths=4096)
        assert ctx.stage_times()["trace_ext"]["launches"] > 0
        assert ctx.traversal_work()["ext"]["rays"] == work["ext"]["rays"]
    finally:
        ctx.set_profiling(False)
    assert np.array_equal(img.view(np.uint32), ref.view(np.uint32))
    assert np.array_equal(both.view(np.uint32), ref.view(np.uint32))
    assert work["ext"]["rays"] == st["ext_rays"]
    assert work["shadow"]["rays"] == st["shadow_rays"]
    assert work["mis"]["rays"] == st["mis_rays"]
    for kind, w in work.items():
        if w["rays"]:
            assert w["nodes"] >= w["rays"], kind
            assert w["triangles"] > 0, kind
            assert w["nodes"] < 10_000 * w["rays"], kind
    ctx.render(scene, 48, 48, wave_paths=4096)
    assert ctx.traversal_work()["ext"]["nodes"] == 0
