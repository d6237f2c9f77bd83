"""orion_gpu_trace_noalloc (fixed static device scratch) against orion_gpu_trace and the oracle.

Collected last so that it runs both after every other test and, alone, in a
fresh process. All calls go through the C ABI.

* against orion_gpu_trace: the same kernel (k_trace_rays) at the same launch
  configuration on the same rays, so t, u, v and prim must be bit-identical;
  a scratch layout or offset fault would show here;
* against the CPU oracle: the tolerance of the 1M-ray parity test (same
  primitive except ties, t within helpers.t_tolerance, hit/miss differing on
  at most 10 rays per million);
* it allocates nothing: the device's free memory (cudaMemGetInfo) is the same
  before and after a call made once the entry point has been set up.
"""
import ctypes

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def _bounds(host):
    p = host.arrays()["positions"].reshape(-1, 3)
    return p.min(0), p.max(0)


def _agree_with_oracle(got, want, rays, positions, any_hit):
    t, u, v, prim = got
    rt, ru, rv, rprim = want
    n = len(rays)
    hit = rprim >= 0
    assert np.count_nonzero((prim >= 0) != hit) <= n * 1e-5
    if any_hit:
        return hit.mean()
    both = hit & (prim >= 0)
    tol = helpers.t_tolerance(rays, rt, rprim, positions)
    assert (np.abs(t.astype(np.float64) - rt) <= tol)[both].all(), "t outside the rounding bound"
    return both.mean()


@pytest.mark.parametrize("name,kw", [("cornell", {}), ("displaced", dict(res=64, spp=4, subdiv=6))])
def test_noalloc_trace_matches_trace(ctx, built, tmp_path, name, kw):
    import orion_gb300 as og
    from oracle import port
    host = og.HostScene.load(helpers.write_scene(name, str(tmp_path / name), **kw))
    lo, hi = _bounds(host)
    positions = host.arrays()["positions"]
    oracle = port.Scene(host)
    sid = ctx.upload(host)
    try:
        # two calls in a row: the full scratch, then a smaller call over other rays
        for call, (n, seed) in enumerate([(og.NOALLOC_MAX_RAYS, 31), (40000, 37)]):
            rays = helpers.random_rays(n, lo, hi, seed=seed)
            rays[: n // 8, 7] = (helpers.splitmix_uniform(n // 8, seed + 5) * float(np.max(hi - lo))).astype(np.float32)
            want_cpu = oracle.trace(rays)
            for any_hit in (False, True):
                got = ctx.trace_noalloc(sid, rays, any_hit=any_hit)
                want = ctx.trace(sid, rays, any_hit=any_hit)
                for a, b in zip(got, want):
                    assert np.array_equal(a.view(np.uint32), b.view(np.uint32)), "differs from orion_gpu_trace"
                frac = _agree_with_oracle(got, want_cpu, rays, positions, any_hit)
                print(f"{name} call {call + 1}: {n} rays, any_hit={any_hit}, {frac:.3f} hit, bit-identical to "
                      f"orion_gpu_trace, within the oracle tolerance")
        # no device allocation: the set-up is done, so a further call leaves free memory unchanged
        rays = helpers.random_rays(4096, lo, hi, seed=41)
        ctx.trace_noalloc(sid, rays)
        free0, _ = ctx.mem_info()
        ctx.trace_noalloc(sid, rays)
        free1, _ = ctx.mem_info()
        assert free1 == free0, f"free device memory changed by {free0 - free1} bytes during the call"
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
