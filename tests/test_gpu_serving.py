"""Serving: requests admitted by memory, progressive chunks, continuous batching.

A request's film is the sum over its own sample passes. Served requests run
the batched engine's kernels, compiled apart from the plain path's (the
compiler may contract different multiply-adds), so against the plain FP64
render of the same view a film agrees to FP32 rounding (1e-5 relative); among
served results, alone or overlapped with other requests and whatever the
chunk size, films agree to 1e-12.
"""
from __future__ import annotations

import threading
import time

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def hosts(tmp_path_factory):
    import orion_gb300 as og
    d = tmp_path_factory.mktemp("serve")
    return {name: og.HostScene.load(helpers.write_scene(name, str(d / name), **kw)) for name, kw in [
        ("cornell", dict(res=48, spp=8)), ("zoo", dict(res=40, spp=8)), ("displaced", dict(res=32, spp=8, subdiv=4))]}


def _plain(ctx, host, **kw):
    sid = ctx.upload(host)
    d = host.desc()
    s, q = ctx.render(sid, d.camera.width, d.camera.height, fp64=True, **kw)
    ctx.release(sid)
    return s


def _close(a, b):
    return np.all(np.abs(a - b) <= 1e-12 * np.abs(b) + 1e-12)


def _near(a, b):
    return np.allclose(a, b, rtol=1e-5, atol=1e-7)


def test_request_same_alone_and_in_mix(ctx, hosts):
    import orion_gb300 as og
    ref = {k: _plain(ctx, h) for k, h in hosts.items()}
    srv = og.Server(ctx, spp_chunk=2)
    try:
        t = srv.submit(hosts["zoo"])
        assert srv.wait(t, 60)
        alone, _, cnt = srv.result(t)
        srv.release(t)
        assert (cnt == 8).all() and _near(alone, ref["zoo"])
        ref["zoo"] = alone
        # Concurrent arrivals from another thread while the server is busy.
        tickets = {}

        def submitter():
            for k in ["cornell", "zoo", "displaced", "zoo", "cornell"]:
                tickets.setdefault(k, []).append(srv.submit(hosts[k]))
                time.sleep(0.002)
        th = threading.Thread(target=submitter)
        th.start()
        th.join()
        for k, ts in tickets.items():
            for t in ts:
                assert srv.wait(t, 120)
                s, _, c = srv.result(t)
                assert (c == 8).all()
                assert (_close if k == "zoo" else _near)(s, ref[k]), k
                st = srv.status(t)
                assert st["t_done"] >= st["t_admit"] >= st["t_submit"]
                srv.release(t)
        stats = srv.stats()
        assert stats["completed"] == 6 and stats["launches"] >= 4
    finally:
        srv.close()


def test_tight_budget_queues_and_evicts(ctx, hosts):
    import orion_gb300 as og
    ref = _plain(ctx, hosts["cornell"])
    srv = og.Server(ctx, memory_budget=1, spp_chunk=4)   # nothing fits: request fails cleanly
    try:
        t = srv.submit(hosts["cornell"])
        with pytest.raises(og.OrionError):
            srv.wait(t, 30)
        assert srv.status(t)["state"] == og.REQ_FAILED
        srv.release(t)
    finally:
        srv.close()
    srv = og.Server(ctx, spp_chunk=4)
    try:
        t = srv.submit(hosts["cornell"], camera=None)
        assert srv.wait(t, 60)
        s, _, _ = srv.result(t)
        assert _near(s, ref)
        srv.release(t)
    finally:
        srv.close()


def test_other_views_of_a_resident_scene(ctx, hosts):
    import orion_gb300 as og
    srv = og.Server(ctx, spp_chunk=3)
    try:
        cams = [og.look_at_camera((x, 0.2, 3.5), (0, 0, 0), (0, 1, 0), 40.0, 32, 24) for x in (-0.5, 0.0, 0.5)]
        ts = [srv.submit(hosts["cornell"], spp=5, camera=c) for c in cams]
        outs = []
        for t in ts:
            assert srv.wait(t, 60)
            s, _, c = srv.result(t)
            assert s.shape == (24, 32, 3) and (c == 5).all()
            outs.append(s)
            srv.release(t)
        assert srv.stats()["resident_scenes"] == 1
        assert not np.allclose(outs[0], outs[2])  # different views
        # the same view submitted again gives the same film
        t = srv.submit(hosts["cornell"], spp=5, camera=cams[1])
        assert srv.wait(t, 60)
        s, _, _ = srv.result(t)
        assert _close(s, outs[1])
        srv.release(t)
    finally:
        srv.close()


def test_cancel(ctx, hosts):
    import orion_gb300 as og
    srv = og.Server(ctx, spp_chunk=1)
    try:
        t = srv.submit(hosts["displaced"], spp=64)
        srv.cancel(t)
        with pytest.raises(og.OrionError):
            srv.wait(t, 30)
        for _ in range(100):
            try:
                srv.release(t)
                break
            except og.OrionError:
                time.sleep(0.05)
        assert srv.stats()["submitted"] == 1
    finally:
        srv.close()


def test_preview_is_the_bmp_of_the_averaged_film(ctx, hosts, tmp_path):
    """orion_server_preview: the device-side 8-bit preview equals the pixels orion_film_write_bmp writes
    for the averaged film (saveAsBmp, src/core/texture.cpp:77-136), top-down and bottom-up."""
    import orion_gb300 as og
    srv = og.Server(ctx, spp_chunk=2)
    try:
        t = srv.submit(hosts["cornell"])
        assert srv.wait(t, 60)
        s, _, c = srv.result(t)
        top = srv.preview(t)
        bottom = srv.preview(t, bottom_up=True)
        srv.release(t)
    finally:
        srv.close()
    avg = (s / c[..., None]).astype(np.float32)
    bmp = tmp_path / "film.bmp"
    og.saveAsBmp(avg, str(bmp))
    data = np.frombuffer(open(bmp, "rb").read()[54:], np.uint8).reshape(avg.shape[0], avg.shape[1], 4)
    assert np.array_equal(bottom, data)
    assert np.array_equal(top, data[::-1])
    assert (top[..., 3] == 255).all() and top[..., :3].any()
