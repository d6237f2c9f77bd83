"""Generate the golden fixtures in tests/golden/ from the reference renderer.

Runs only where the reference sources exist: it builds oracle/_ref (the
reference's own integrator, BSDFs, lights, camera, Sobol sampler and film,
compiled from its sources; Embree replaced by the project CPU BVH) and
records its outputs on fixed inputs:

  sobol.npz    sobol::sample on an (index, dim) grid      (src/sampler/sobol.h:28-43)
  bsdf.npz     BSDF f/pdf/sample_f per material            (src/core/bsdf.cpp, src/bsdf/*)
  camera.npz   Pinhole::generateRay, pinhole + thin lens    (src/camera/pinhole.cpp:8-33)
  trace.npz    Scene::intersect hits on the Cornell box     (project CPU kernel in Embree's place)
  image_*.npz  PathTracing::render film sums                (src/integrator/path.cpp:15-37);
               image_envlit lit by an image environment map (src/light/envmap.cpp),
               image_textured with image textures on every material input (src/core/texture.cpp)
  image_*_sppm.npz  SPPM::render film sums (src/integrator/sppm.cpp:58-322), one thread:
               caustics (every light type), envlit (image environment map), textured
  stats_*.npz  FP64 per-pixel mean and variance at high spp (for 3-sigma checks)
  fullsize_*.npz  the 1024x1024 displaced-sphere and the 1920x1080 eight-sphere
               workloads at their full sizes: per-pixel FP64 sums at the
               workload's own spp on seeded pixels (path-for-path parity) and
               at 65,536 spp on the same pixels (3-sigma and RMSE checks); the
               eight-sphere scene with its Beckmann plastic (no Beckmann in the
               reference) comes from the oracle restatement instead
  geometry.npz loader output digests

    python tests/golden/make_golden.py [--quick] [--only fullsize]
"""
from __future__ import annotations

import argparse
import ctypes as C
import os
import sys
import tempfile
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import helpers  # noqa: E402
from oracle import build  # noqa: E402
from orion_gb300 import Material  # noqa: E402


def vp(a):
    return C.c_void_p(a.ctypes.data)


class Ref:
    def __init__(self):
        lib = build.build_reference()
        if lib is None:
            raise SystemExit("reference tree not found; set ORION_REFERENCE")
        self.lib = C.CDLL(lib)
        self.lib.ref_scene_load.restype = C.c_void_p
        self.lib.ref_scene_load.argtypes = [C.c_char_p]

    def load(self, path):
        h = C.c_void_p(self.lib.ref_scene_load(path.encode()))
        info = np.zeros(5, np.int32)
        self.lib.ref_scene_info(h, vp(info))
        return h, info

    def load_in_scene_dir(self, path):
        """load() from the scene's directory: the reference opens image-texture file names
        relative to the working directory (src/util/parser.cpp:438-443)."""
        cwd = os.getcwd()
        os.chdir(os.path.dirname(os.path.abspath(path)))
        try:
            return self.load(os.path.abspath(path))
        finally:
            os.chdir(cwd)

    def sobol(self, idx, dim):
        out = np.zeros(len(idx), np.float32)
        self.lib.ref_sobol(vp(idx), vp(dim), C.c_int64(len(idx)), vp(out))
        return out

    def bsdf(self, mat, frame, wo, wi, rnd, type_mask):
        n = len(frame)
        out = {k: np.zeros(s, dt) for k, s, dt in [("f", (n, 3), np.float32), ("pdf", n, np.float32),
                                                  ("sf", (n, 3), np.float32), ("swi", (n, 3), np.float32),
                                                  ("spdf", n, np.float32), ("stype", n, np.int32),
                                                  ("nbxdf", n, np.int32)]}
        self.lib.ref_bsdf_eval(C.byref(mat), C.c_int64(n), vp(frame), vp(wo), vp(wi), vp(rnd), C.c_int32(type_mask),
                               *(vp(out[k]) for k in ("f", "pdf", "sf", "swi", "spdf", "stype", "nbxdf")))
        return out


def sobol_grid():
    idx = [0, 1, 2, 3, 4, 5, 7, 8, 255, 256, 257, 65535, 65536, 65537]
    for k in range(1, 52):
        idx += [(1 << k) - 1, 1 << k, (1 << k) + 1]
    u = helpers.splitmix_uniform(400, 11)
    idx += [int(x * (1 << 28)) for x in u[:200]]          # sample indices of a 1080p x 128 spp render
    idx += [int(x * (1 << 52)) for x in u[200:]]
    dims = list(range(0, 160)) + [255, 256, 511, 512, 1000, 1023]
    I, D = np.meshgrid(np.array(idx, np.uint64), np.array(dims, np.uint32), indexing="ij")
    I, D = I.ravel(), D.ravel()
    keep = helpers.splitmix_uniform(len(I), 12) < 0.25
    keep[:len(dims) * 20] = True
    return I[keep].copy(), D[keep].copy()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true")
    ap.add_argument("--only", choices=["fullsize"], help="regenerate one group of fixtures only")
    args = ap.parse_args()
    ref = Ref()
    t0 = time.time()
    if args.only == "fullsize":
        fullsize(ref, args.quick)
        return

    # Sobol
    idx, dim = sobol_grid()
    val = ref.sobol(idx, dim)
    np.savez_compressed(os.path.join(HERE, "sobol.npz"), index=idx, dim=dim, value=val)
    print("sobol", len(idx), time.time() - t0)

    # BSDFs
    n = 512
    out = {}
    for ci, (name, fields) in enumerate(helpers.BSDF_CASES):
        mat = helpers.make_material(fields)
        frame, wo, wi, rnd = helpers.bsdf_inputs(n, 1000 + ci)
        out[f"{name}/frame"], out[f"{name}/wo"], out[f"{name}/wi"], out[f"{name}/rnd"] = frame, wo, wi, rnd
        for tm in (31, 15):
            r = ref.bsdf(mat, frame, wo, wi, rnd, tm)
            for k, v in r.items():
                out[f"{name}/{tm}/{k}"] = v
    np.savez_compressed(os.path.join(HERE, "bsdf.npz"), **out)
    print("bsdf", time.time() - t0)

    with tempfile.TemporaryDirectory() as tmp:
        # Camera rays: pinhole (cornell) and thin lens (mixed, reduced)
        cam = {}
        for name, kw in [("cornell", dict(res=64, spp=4)),
                         ("mixed", dict(width=96, height=54, spp=4, subdivs=(1, 1, 1, 1, 1, 1, 1, 1)))]:
            path = helpers.write_scene(name, os.path.join(tmp, name), **kw)
            h, info = ref.load(path)
            W, H = int(info[0]), int(info[1])
            si = (helpers.splitmix_uniform(1024, 21) * W * H * 4).astype(np.int64)
            si[:4] = [0, 1, W * H - 1, W * H]
            rays = np.zeros((len(si), 6), np.float32)
            ref.lib.ref_scene_camera_rays(h, C.c_int64(len(si)), vp(si), vp(rays))
            cam[f"{name}/index"], cam[f"{name}/rays"] = si, rays
            cam[f"{name}/hash"] = np.frombuffer(helpers.scene_hash(path).encode(), np.uint8)
            ref.lib.ref_scene_free(h)
        np.savez_compressed(os.path.join(HERE, "camera.npz"), **cam)
        print("camera", time.time() - t0)

        # Trace: Cornell box, C1 geometry
        path = helpers.write_scene("cornell", os.path.join(tmp, "cornell256"))
        h, info = ref.load(path)
        n = 16384
        rays = helpers.random_rays(n, (-1, -1, -1), (1, 1, 1), seed=5)
        rays[: n // 4, 7] = (helpers.splitmix_uniform(n // 4, 6) * 3.0).astype(np.float32)  # finite tfar
        t = np.zeros(n, np.float32)
        prim = np.zeros(n, np.int32)
        p, ng, ns = (np.zeros((n, 3), np.float32) for _ in range(3))
        ref.lib.ref_scene_trace(h, C.c_int64(n), vp(rays), vp(t), vp(prim), vp(p), vp(ng), vp(ns))
        np.savez_compressed(os.path.join(HERE, "trace.npz"), rays=rays, t=t, prim=prim, p=p, ng=ng, ns=ns,
                            hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8))
        # Loader digest for the same file
        T = int(info[2])
        P, N, UV = np.zeros((T, 9), np.float32), np.zeros((T, 9), np.float32), np.zeros((T, 6), np.float32)
        lop, pw = np.zeros(T, np.int32), np.zeros(int(info[3]), np.float32)
        ref.lib.ref_scene_geometry(h, vp(P), vp(N), vp(UV), vp(lop), vp(pw))
        geo = {"cornell/positions_sha": np.frombuffer(__import__("hashlib").sha256(P.tobytes()).hexdigest().encode(), np.uint8),
               "cornell/normals_sha": np.frombuffer(__import__("hashlib").sha256(N.tobytes()).hexdigest().encode(), np.uint8),
               "cornell/light_of_prim": lop, "cornell/light_power": pw}
        ref.lib.ref_scene_free(h)
        print("trace", time.time() - t0)

        # Images through the reference's own PathTracing::render
        for name, kw in [("cornell", dict(res=64, spp=16)), ("zoo", dict(res=48, spp=16)),
                         ("envlit", dict(res=48, spp=16)), ("textured", dict(res=48, spp=16))]:
            path = helpers.write_scene(name, os.path.join(tmp, "img_" + name), **kw)
            h, info = ref.load_in_scene_dir(path)
            W, H = int(info[0]), int(info[1])
            img = np.zeros((H, W, 3), np.float32)
            ref.lib.ref_scene_render(h, vp(img))
            np.savez_compressed(os.path.join(HERE, f"image_{name}.npz"), film=img, width=W, height=H,
                                spp=kw["spp"], hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8))
            if name == "zoo":
                T = int(info[2])
                P, N, UV = np.zeros((T, 9), np.float32), np.zeros((T, 9), np.float32), np.zeros((T, 6), np.float32)
                lop, pw = np.zeros(T, np.int32), np.zeros(int(info[3]), np.float32)
                ref.lib.ref_scene_geometry(h, vp(P), vp(N), vp(UV), vp(lop), vp(pw))
                geo["zoo/light_power"] = pw
                geo["zoo/positions_sha"] = np.frombuffer(__import__("hashlib").sha256(P.tobytes()).hexdigest().encode(), np.uint8)
            ref.lib.ref_scene_free(h)
            print("image", name, time.time() - t0)
        np.savez_compressed(os.path.join(HERE, "geometry.npz"), **geo)

        # SPPM through the reference's own SPPM::render, one OpenMP thread so that the photon
        # sums and the grid's cell lists have one order.
        sppm_kw = dict(res=48, iterations=8, photons=20000, radius=0.08, max_depth=5)
        path = helpers.write_scene("caustics", os.path.join(tmp, "sppm"), **sppm_kw)
        h, info = ref.load(path)
        W, H = int(info[0]), int(info[1])
        img = np.zeros((H, W, 3), np.float32)
        ref.lib.ref_set_threads(1)
        ref.lib.ref_scene_render(h, vp(img))
        ref.lib.ref_set_threads(0)
        np.savez_compressed(os.path.join(HERE, "image_caustics_sppm.npz"), film=img, width=W, height=H,
                            hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8), **sppm_kw)
        ref.lib.ref_scene_free(h)
        # SPPM with photons from an image environment map, and with image textures
        for name in ("envlit_sppm", "textured_sppm"):
            kw = dict(res=32, iterations=4, photons=10000, radius=0.08)
            path = helpers.write_scene(name, os.path.join(tmp, name), **kw)
            h, info = ref.load_in_scene_dir(path)
            W, H = int(info[0]), int(info[1])
            img = np.zeros((H, W, 3), np.float32)
            ref.lib.ref_set_threads(1)
            ref.lib.ref_scene_render(h, vp(img))
            ref.lib.ref_set_threads(0)
            np.savez_compressed(os.path.join(HERE, f"image_{name}.npz"), film=img, width=W, height=H,
                                hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8), **kw)
            ref.lib.ref_scene_free(h)
        print("sppm", time.time() - t0)

        # FP64 statistics: Cornell at the full C1 resolution, a seeded pixel subset at high spp.
        spp_hi = 4096 if args.quick else 65536
        path = helpers.write_scene("cornell", os.path.join(tmp, "stats"))
        h, info = ref.load(path)
        W, H = int(info[0]), int(info[1])
        npix = 64 if args.quick else 256
        u = helpers.splitmix_uniform(2 * npix, 31).reshape(npix, 2)
        pix = np.stack([(u[:, 0] * W).astype(np.int32), (u[:, 1] * H).astype(np.int32)], 1).astype(np.int32)
        s = np.zeros((npix, 3), np.float64)
        q = np.zeros((npix, 3), np.float64)
        ref.lib.ref_scene_render_pixels(h, C.c_int64(npix), vp(pix), C.c_int32(0), C.c_int32(spp_hi), vp(s), vp(q),
                                        C.c_int32(0))
        np.savez_compressed(os.path.join(HERE, "stats_cornell.npz"), pix=pix, spp=spp_hi, sum=s, sumsq=q,
                            hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8))
        ref.lib.ref_scene_free(h)
        print("stats", time.time() - t0)
    fullsize(ref, args.quick)


# Full-size workloads: (scenegen function, its arguments, fixture name, seed of the pixel choice, renderer).
# The reference has one microfacet distribution (GGX) and renders the eight-sphere scene's Beckmann plastic
# as GGX, so its fixture is of the scene with a GGX plastic; the scene as specified (Beckmann) gets a
# fixture from the oracle restatement, which implements Beckmann as an extension.
FULLSIZE = [("cornell", {}, "fullsize_cornell.npz", 37, "reference"),
            ("displaced", {}, "fullsize_displaced.npz", 41, "reference"),
            ("mixed", {"plastic_distribution": "ggx"}, "fullsize_mixed.npz", 43, "reference"),
            ("mixed", {}, "fullsize_mixed_beckmann.npz", 47, "oracle")]


def seeded_pixels(n: int, W: int, H: int, seed: int) -> np.ndarray:
    """n (x, y) pixels from SplitMix64, uniform over the image (tests recompute nothing: the fixture stores them)."""
    u = helpers.splitmix_uniform(2 * n, seed).reshape(n, 2)
    return np.stack([(u[:, 0] * W).astype(np.int32), (u[:, 1] * H).astype(np.int32)], 1).astype(np.int32)


def fullsize(ref: Ref, quick: bool) -> None:
    """Per-pixel FP64 sums of the reference's PathTracing::Li on the full-size workloads.

    On 1024 seeded pixels (band_pix = pix):
    band_*: the workload's own spp, sample passes [0, spp): the same Sobol samples the GPU
    renderer and the oracle trace, so sums agree path for path, and the Monte Carlo error of
    an image at the workload's spp (matched-RMSE checks);
    sum/sumsq: 65,536 spp, passes [0, 65536): the converged per-pixel means and their
    Monte Carlo variance (3-sigma checks, the reference image of the RMSE checks)."""
    spp_hi = 4096 if quick else 65536
    for name, kw, fixture, seed, renderer in FULLSIZE:
        t0 = time.time()
        with tempfile.TemporaryDirectory() as tmp:
            path = helpers.write_scene(name, os.path.join(tmp, name), **kw)
            spp = scene_spp(path)
            if renderer == "reference":
                h, info = ref.load(path)
                W, H = int(info[0]), int(info[1])

                def pixels(pix, first, n):
                    s, q = np.zeros((len(pix), 3)), np.zeros((len(pix), 3))
                    ref.lib.ref_scene_render_pixels(h, C.c_int64(len(pix)), vp(pix), C.c_int32(first), C.c_int32(n),
                                                    vp(s), vp(q), C.c_int32(0))
                    return s, q
            else:
                from oracle import port
                sc = port.Scene.load(path)
                W, H = sc.width, sc.height

                def pixels(pix, first, n):
                    return sc.render_pixels(pix, n, first_pass=first)
            pix = band = seeded_pixels(1024, W, H, seed)
            bs, bq = pixels(band, 0, spp)
            s, q = pixels(pix, 0, spp_hi)
            np.savez_compressed(os.path.join(HERE, fixture), band_pix=band, band_spp=spp, band_sum=bs, band_sumsq=bq,
                                pix=pix, spp=spp_hi, sum=s, sumsq=q, width=W, height=H,
                                renderer=np.frombuffer(renderer.encode(), np.uint8),
                                hash=np.frombuffer(helpers.scene_hash(path).encode(), np.uint8))
            if renderer == "reference":
                ref.lib.ref_scene_free(h)
        print(fixture, f"{time.time() - t0:.1f} s")


def scene_spp(ori_path: str) -> int:
    """The samples per pixel the scene file's integrator asks for (<Param nSamplesPerPixel=...>)."""
    import re
    m = re.search(r'nSamplesPerPixel="(\d+)"', open(ori_path).read())
    if not m:
        raise RuntimeError("no spp in " + ori_path)
    return int(m.group(1))


if __name__ == "__main__":
    main()
