"""The GPU renderer against the reference and the oracle at the full sizes of the
single-image workloads: the 256x256 x 16 spp Cornell box, the 1024x1024 x 64 spp
displaced sphere (1,310,722 triangles, GGX conductor, spot + environment light,
depth 8) and the 1920x1080 x 128 spp eight-sphere scene (1.27M triangles, five
materials, thin lens, depth 16). Fixtures: tests/golden/fullsize_*.npz, 1024
seeded pixels each.

* path for path: the GPU traces the same Sobol samples as the reference
  (src/integrator/path.cpp:15-37 over src/integrator/path.cpp:50-99), so a
  pixel's sum over the workload's samples is the reference's except where FP32
  rounding (device transcendentals, contraction) sends one of its paths down
  another branch. Checked on the reference's own sums and on the oracle's FP32
  film rows spread over the image: the fraction of identical pixels.
* matched RMSE: the GPU image at the workload's spp and the reference's image at
  the same spp, each against the reference's 65,536-spp FP64 means: their
  relative RMSEs agree within 1% (2% against the oracle's Beckmann extension).
* statistics: a 1024-spp FP64 GPU render (sample passes disjoint from the
  reference's) against the 65,536-spp means: within 3 sigma of the combined
  Monte Carlo error.

The relative RMSE of the path-for-path difference itself is printed, not
bounded: it is the few divergent paths, and one of them landing on a spot-light
highlight in the glossy conductor (a path of radiance in the thousands) sets it.

The reference has one microfacet distribution (GGX); the eight-sphere scene's
plastic is Beckmann as specified only against the oracle restatement
(fullsize_mixed_beckmann.npz), and GGX against the reference
(fullsize_mixed.npz).
"""
from __future__ import annotations

import numpy as np
import pytest

import helpers

pytestmark = pytest.mark.gpu

IDENTICAL = 0.97       # fraction of pixels whose sums agree to 1e-4 relative (+1e-5); measured 0.980-0.993
# |RMSE(GPU) / RMSE(reference) - 1| at the workload's spp, both against the 65,536-spp means: within 1% of the
# reference's (measured 0.0000-0.0015). Against the oracle's Beckmann extension 2% (measured 0.0145): there the
# GPU's device transcendentals and the C library's round the Beckmann sampling differently more often, and the
# ratio moves by the few divergent paths that reach a light's highlight (|ratio - 1| is at most the difference
# image's relative RMSE, 5e-3 of the image here, over the image's relative RMSE, 0.043).
MATCHED_RMSE = {"reference": 0.01, "oracle": 0.02}
WITHIN_3_SIGMA = 0.95  # measured 0.99-1.00
FIXTURES = ["fullsize_cornell.npz", "fullsize_displaced.npz", "fullsize_mixed.npz", "fullsize_mixed_beckmann.npz"]


@pytest.fixture(scope="module")
def port(built):
    from oracle import port as p
    p.lib()
    return p


@pytest.fixture(scope="module")
def scenes(ctx):
    """fixture name -> (host scene, scene id, fixture arrays), uploaded once for the module."""
    import orion_gb300 as og
    out = {}
    for fixture, (name, kw) in helpers.FULLSIZE.items():
        g = helpers.golden(fixture)
        path = helpers.fullsize_scene(name, **kw)
        assert helpers.scene_hash(path) == bytes(g["hash"]).decode(), "scene generator output differs from the fixture"
        host = og.HostScene.load(path)
        out[fixture] = (path, host, ctx.upload(host), g)
    yield out
    for _, _, sid, _ in out.values():
        ctx.release(sid)


def _identical(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float((np.abs(a - b) <= 1e-4 * np.abs(b) + 1e-5).all(-1).mean())


def _rel_rmse(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.sqrt(np.mean((a - b) ** 2)) / np.sqrt(np.mean(b ** 2)))


def _who(g):
    return bytes(g["renderer"]).decode()


@pytest.mark.parametrize("fixture", FIXTURES)
def test_fullsize_pixels_match_path_for_path(ctx, scenes, fixture):
    _, host, sid, g = scenes[fixture]
    W, H, spp = int(g["width"]), int(g["height"]), int(g["band_spp"])
    s, _ = ctx.render(sid, W, H, spp=spp, fp64=True)
    pix = g["band_pix"]
    gpu = s[pix[:, 1], pix[:, 0]]
    close = _identical(gpu, g["band_sum"])
    conv = g["sum"] / float(g["spp"])
    e_gpu, e_ref = _rel_rmse(gpu / spp, conv), _rel_rmse(g["band_sum"] / spp, conv)
    print(f"{fixture}: {close:.4f} of {len(pix)} pixels identical to the {_who(g)}'s sums path for path "
          f"(difference: relative RMSE {_rel_rmse(gpu, g['band_sum']):.2e}); RMSE against the converged means at "
          f"{spp} spp: GPU {e_gpu:.5f}, {_who(g)} {e_ref:.5f} (ratio {e_gpu / e_ref:.5f})")
    assert close >= IDENTICAL
    assert abs(e_gpu / e_ref - 1) <= MATCHED_RMSE[_who(g)]


@pytest.mark.parametrize("fixture", ["fullsize_cornell.npz", "fullsize_displaced.npz", "fullsize_mixed_beckmann.npz"])
def test_fullsize_rows_match_oracle(ctx, port, scenes, fixture):
    """The FP32 film (sums in sample order) on 16 rows spread over the image against the oracle's."""
    path, host, sid, g = scenes[fixture]
    W, H = int(g["width"]), int(g["height"])
    film, cnt = ctx.render(sid, W, H)
    rows = port.spread_rows(16, H)
    ref, _ = port.Scene(host).render(rows=rows)
    assert (cnt == int(g["band_spp"])).all()
    close = _identical(film[rows], ref[rows])
    print(f"{fixture}: {close:.4f} of {len(rows) * W} pixels identical to the oracle path for path "
          f"(difference: relative RMSE {_rel_rmse(film[rows], ref[rows]):.2e})")
    assert close >= IDENTICAL


@pytest.mark.parametrize("fixture", FIXTURES)
def test_fullsize_statistics_within_3_sigma(ctx, scenes, fixture):
    _, host, sid, g = scenes[fixture]
    W, H = int(g["width"]), int(g["height"])
    n, ref_spp = 1024, int(g["spp"])
    s, q = ctx.render(sid, W, H, spp=n, first_pass=ref_spp, fp64=True)
    pix = g["pix"]
    s, q = s[pix[:, 1], pix[:, 0]], q[pix[:, 1], pix[:, 0]]
    mean, rmean = s / n, g["sum"] / ref_spp
    var = np.maximum(q / n - mean ** 2, 0)
    rvar = np.maximum(g["sumsq"] / ref_spp - rmean ** 2, 0)
    sigma = np.sqrt(var / n + rvar / ref_spp) + 1e-7
    frac = float((np.abs(mean - rmean) / sigma <= 3).all(1).mean())
    rmse = _rel_rmse(mean, rmean)
    noise = float(np.sqrt(np.mean(sigma ** 2)) / np.sqrt(np.mean(rmean ** 2)))
    print(f"{fixture}: {len(pix)} pixels, {frac:.3f} within 3 sigma, relative RMSE {rmse:.4f} "
          f"(Monte Carlo noise alone {noise:.4f}) vs the {ref_spp}-spp {_who(g)}")
    assert frac >= WITHIN_3_SIGMA
