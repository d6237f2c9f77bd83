"""GPU path vs the reference, through the C ABI, on the committed golden vectors.

Tolerances (FP32 path math; integer work is bit-exact):
  * Sobol samples: bit-exact.
  * BSDF f / pdf / sampled f, wi, pdf: |gpu - ref| <= 1e-5 * |ref| + 1e-6 * scale
    for at least 99.5% of entries; the rest (sampled-lobe flips at
    u == F, grazing cancellations) are listed in the failure message.
  * camera rays: 1e-5 relative.
  * closest hits: same primitive except ties, t within 1e-5 relative.
  * images: same Sobol samples per path, so per-pixel sums agree to FP32
    rounding except where a path takes a different branch.
"""
from __future__ import annotations

import os
import tempfile

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu


def test_sobol_bit_exact(ctx):
    g = helpers.golden("sobol.npz")
    out = ctx.sobol(g["index"], g["dim"])
    assert out.dtype == np.float32
    bad = np.flatnonzero(out.view(np.uint32) != g["value"].view(np.uint32))
    assert bad.size == 0, f"{bad.size} mismatches, first index={g['index'][bad[:5]]} dim={g['dim'][bad[:5]]}"


def _close(a, b, rtol=1e-5, atol_scale=1e-6):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    scale = max(1.0, float(np.nanmax(np.abs(b))) if b.size else 1.0)
    ok = np.abs(a - b) <= rtol * np.abs(b) + atol_scale * scale
    ok |= (a == b)  # infinities
    ok |= np.isnan(a) & np.isnan(b)
    return ok


@pytest.mark.parametrize("case", [c[0] for c in helpers.BSDF_CASES])
@pytest.mark.parametrize("type_mask", [31, 15])
def test_bsdf_matches_reference(ctx, case, type_mask):
    g = helpers.golden("bsdf.npz")
    fields = dict(helpers.BSDF_CASES)[case]
    mat = helpers.make_material(fields)
    frame, wo, wi, rnd = (g[f"{case}/{k}"] for k in ("frame", "wo", "wi", "rnd"))
    out = ctx.bsdf_eval(mat, frame, wo, wi, rnd, type_mask)
    ref = {k: g[f"{case}/{type_mask}/{k}"] for k in ("f", "pdf", "sf", "swi", "spdf", "stype", "nbxdf")}
    assert np.array_equal(out["nbxdf"], ref["nbxdf"])
    # Evaluation at given directions.
    ok_f = _close(out["f"], ref["f"]).all(1) & _close(out["pdf"], ref["pdf"])
    assert ok_f.mean() >= 0.995, f"f/pdf mismatch rows {np.flatnonzero(~ok_f)[:10]}"
    # Sampling: compare where both chose the same lobe outcome.
    same_type = out["stype"] == ref["stype"]
    assert same_type.mean() >= 0.99, f"sampled type differs in {np.flatnonzero(~same_type)[:10]}"
    valid = same_type & (ref["spdf"] > 0)
    ok_s = (_close(out["sf"], ref["sf"]).all(1) & _close(out["spdf"], ref["spdf"]) &
            _close(out["swi"], ref["swi"], atol_scale=1e-5).all(1))
    assert ok_s[valid].mean() >= 0.995 if valid.any() else True, \
        f"sample mismatch rows {np.flatnonzero(valid & ~ok_s)[:10]}"


def _scene(tmp, name, **kw):
    path = helpers.write_scene(name, os.path.join(tmp, name), **kw)
    return path


def test_camera_rays_match_reference(ctx):
    import orion_gb300 as og
    g = helpers.golden("camera.npz")
    with tempfile.TemporaryDirectory() as tmp:
        for name, kw in [("cornell", dict(res=64, spp=4)),
                         ("mixed", dict(width=96, height=54, spp=4, subdivs=(1, 1, 1, 1, 1, 1, 1, 1)))]:
            path = _scene(tmp, name, **kw)
            assert helpers.scene_hash(path) == bytes(g[f"{name}/hash"]).decode(), "scene generator drifted"
            hs = og.HostScene.load(path)
            sid = ctx.upload(hs)
            rays = ctx.camera_rays(sid, g[f"{name}/index"])
            ctx.release(sid)
            ok = _close(rays, g[f"{name}/rays"], rtol=1e-5, atol_scale=1e-6).all(1)
            assert ok.all(), f"{name}: rows {np.flatnonzero(~ok)[:10]}"


def test_closest_hit_matches_reference(ctx):
    import orion_gb300 as og
    g = helpers.golden("trace.npz")
    with tempfile.TemporaryDirectory() as tmp:
        path = _scene(tmp, "cornell")
        assert helpers.scene_hash(path) == bytes(g["hash"]).decode(), "scene generator drifted"
        hs = og.HostScene.load(path)
        sid = ctx.upload(hs)
        t, u, v, prim = ctx.trace(sid, g["rays"])
        _, _, _, occ = ctx.trace(sid, g["rays"], any_hit=True)
        ctx.release(sid)
    hit_ref = g["prim"] >= 0
    assert np.array_equal(prim >= 0, hit_ref), f"hit/miss differs on {np.count_nonzero((prim >= 0) != hit_ref)} rays"
    assert np.array_equal(occ >= 0, hit_ref), "occlusion query disagrees with closest hit"
    same = prim == g["prim"]
    # Ties: the other primitive is hit at the same distance (shared edges, coplanar walls).
    t_ok = np.abs(t - g["t"]) <= 1e-5 * np.abs(g["t"]) + 1e-7
    assert (same | t_ok).all(), f"different primitive at a different t on rays {np.flatnonzero(~(same | t_ok))[:10]}"
    assert same.mean() > 0.999, f"primitive differs on {np.count_nonzero(~same)} rays"
    assert t_ok[hit_ref].all(), f"t differs on rays {np.flatnonzero(hit_ref & ~t_ok)[:10]}"


@pytest.mark.parametrize("name,kw", [("cornell", dict(res=64, spp=16)), ("zoo", dict(res=48, spp=16))])
def test_image_matches_reference_render(ctx, name, kw):
    import orion_gb300 as og
    g = helpers.golden(f"image_{name}.npz")
    with tempfile.TemporaryDirectory() as tmp:
        path = _scene(tmp, name, **kw)
        assert helpers.scene_hash(path) == bytes(g["hash"]).decode(), "scene generator drifted"
        ro = og.Parser(path, ctx).getRenderOption()
        ro.integrator.render(ro.scene)
        film = ro.camera.getFilm()
        ctx.release(ro.scene.sid)
    ref = g["film"].astype(np.float64)
    gpu = film.data.astype(np.float64)
    assert (film.counter == kw["spp"]).all()
    diff = np.abs(gpu - ref)
    close = diff <= 1e-4 * np.abs(ref) + 1e-5
    frac = close.all(2).mean()
    rmse = float(np.sqrt(np.mean((gpu - ref) ** 2)) / max(np.sqrt(np.mean(ref ** 2)), 1e-12))
    print(f"{name}: pixels matching the reference path-for-path {frac:.4f}, relative RMSE {rmse:.2e}")
    assert frac >= 0.97, f"only {frac:.3f} of pixels match"
    assert rmse < 0.02
