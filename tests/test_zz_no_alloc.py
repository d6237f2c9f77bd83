"""orion_gpu_trace_noalloc (fixed static device scratch) against orion_gpu_trace.

Collected last so that it runs both after every other test and, alone, in a
fresh process. Both calls go through the C ABI. Tolerance: the same as the
1M-ray parity test (same primitive except ties, t within 1e-5 relative).
"""
import ctypes

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def _bounds(host):
    p = host.arrays()["positions"].reshape(-1, 3)
    return p.min(0), p.max(0)


def _agree(a, b, n):
    t, u, v, prim = a
    rt, ru, rv, rprim = b
    hit = rprim >= 0
    assert np.count_nonzero((prim >= 0) != hit) <= n * 1e-5
    both = hit & (prim >= 0)
    t_ok = np.abs(t - rt) <= 1e-5 * np.abs(rt) + 1e-7
    assert ((prim == rprim) | t_ok)[both].all(), "a different primitive at a different distance"
    assert t_ok[both].mean() > 0.99999
    return both.mean(), float(np.max(np.abs(t - rt)[both] / np.maximum(np.abs(rt[both]), 1e-30), initial=0.0))


@pytest.mark.parametrize("name,kw", [("cornell", {}), ("displaced", dict(res=64, spp=4, subdiv=6))])
def test_noalloc_trace_matches_trace(ctx, tmp_path, name, kw):
    import orion_gb300 as og
    host = og.HostScene.load(helpers.write_scene(name, str(tmp_path / name), **kw))
    lo, hi = _bounds(host)
    sid = ctx.upload(host)
    try:
        # two calls in a row: the full scratch, then a smaller call over other rays
        for call, (n, seed) in enumerate([(og.NOALLOC_MAX_RAYS, 31), (40000, 37)]):
            rays = helpers.random_rays(n, lo, hi, seed=seed)
            rays[: n // 8, 7] = (helpers.splitmix_uniform(n // 8, seed + 5) * float(np.max(hi - lo))).astype(np.float32)
            for any_hit in (False, True):
                got = ctx.trace_noalloc(sid, rays, any_hit=any_hit)
                want = ctx.trace(sid, rays, any_hit=any_hit)
                frac, err = _agree(got, want, n)
                print(f"{name} call {call + 1}: {n} rays, any_hit={any_hit}, {frac:.3f} hit, max rel t error {err:.1e}")
    finally:
        ctx.release(sid)


def test_noalloc_trace_limits(ctx, tmp_path):
    import orion_gb300 as og
    host = og.HostScene.load(helpers.write_scene("cornell", str(tmp_path / "c")))
    sid = ctx.upload(host)
    try:
        lib = og.library()
        n = og.NOALLOC_MAX_RAYS + 1
        rays = np.zeros((n, 8), np.float32)
        out = [np.zeros(n, np.float32) for _ in range(3)] + [np.zeros(n, np.int32)]
        ptr = lambda a: a.ctypes.data_as(ctypes.c_void_p)
        rc = lib.orion_gpu_trace_noalloc(ctx._h, sid, n, ptr(rays), 0, *(ptr(a) for a in out))
        assert rc == -1  # ORION_ERR_INVALID
        assert "ORION_NOALLOC_MAX_RAYS" in lib.orion_last_error().decode()
        rc = lib.orion_gpu_trace_noalloc(ctx._h, sid, 0, None, 0, None, None, None, None)
        assert rc == 0
    finally:
        ctx.release(sid)
