"""ctypes wrapper of the CPU oracle (oracle/port/port.cpp). Test infrastructure only."""
from __future__ import annotations

import ctypes as C
import os
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB = os.path.join(HERE, "_build", "liborion_port.so")
SOBOL = os.path.join(ROOT, "orion_gb300", "data", "sobol_matrices.bin")

_lib = None


def lib() -> C.CDLL:
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            raise OSError(f"{LIB} missing: build with oracle.build.build_port()")
        l = C.CDLL(LIB)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        for name, res, args in [
            ("port_load_sobol", i32, [C.c_char_p]),
            ("port_sobol", i32, [vp, vp, i64, vp]),
            ("port_bsdf_eval", i32, [vp, i64, vp, vp, vp, vp, i32, vp, vp, vp, vp, vp, vp, vp]),
            ("port_scene_create", vp, [vp]),
            ("port_scene_free", None, [vp]),
            ("port_trace", i32, [vp, i64, vp, i32, vp, vp, vp, vp]),
            ("port_camera_rays", i32, [vp, i64, vp, vp]),
            ("port_render", i64, [vp, i32, i64, i32, i32, i32, i32, vp, i32]),
            ("port_render_rows", i64, [vp, i32, i64, i32, i32, i32, vp, vp, i32]),
            ("port_render_pixels", i32, [vp, i64, vp, i64, i32, i32, i32, vp, vp, i32]),
            ("port_scene_info", i32, [vp, vp]),
            ("port_render_sppm", i64, [vp, i32, i32, C.c_float, i32, vp, i32]),
        ]:
            f = getattr(l, name)
            f.restype, f.argtypes = res, args
        if l.port_load_sobol(SOBOL.encode()) != 0:
            raise OSError(f"cannot read {SOBOL}")
        _lib = l
    return _lib


def _p(a):
    return C.c_void_p(a.ctypes.data)


def sobol(index, dim) -> np.ndarray:
    index = np.ascontiguousarray(index, np.uint64)
    dim = np.ascontiguousarray(dim, np.uint32)
    out = np.zeros(len(index), np.float32)
    lib().port_sobol(_p(index), _p(dim), len(index), _p(out))
    return out


def bsdf_eval(mat, frame, wo, wi, rnd, type_mask=31) -> dict:
    from orion_gb300 import _bsdf_call
    return _bsdf_call(lambda m, *a: lib().port_bsdf_eval(C.cast(m, C.c_void_p), *a), mat, frame, wo, wi, rnd,
                      type_mask)


class Scene:
    """The oracle's copy of a scene, built from the same flat record (orion_scene_desc) the GPU path receives."""

    def __init__(self, host_scene=None, desc=None):
        """From a parsed orion_gb300.HostScene, or from a desc built in Python (`desc` = (desc, keep-alive)),
        which leaves the product library unloaded."""
        if host_scene is not None:
            self._host = host_scene
            d = host_scene.desc()
        else:
            d, self._host = desc
        self._h = C.c_void_p(lib().port_scene_create(C.byref(d)))
        info = np.zeros(5, np.int32)
        lib().port_scene_info(self._h, _p(info))
        self.width, self.height, self.spp, self.max_depth, self.num_lights = (int(x) for x in info)
        self.integrator = int(d.integrator)
        self.sppm = (int(d.sppm.iterations), int(d.sppm.photons_per_iter), float(d.sppm.initial_radius),
                     int(d.sppm.max_depth))

    @classmethod
    def load(cls, path: str) -> "Scene":
        """The scene file parsed by the product's loader (orion_scene_load_ori)."""
        import orion_gb300 as og
        return cls(og.HostScene.load(path))

    @classmethod
    def from_generated(cls, scene) -> "Scene":
        """A generated scene (orion_gb300.scenegen.Scene) from its arrays, without loading the product
        library: the same geometry as its scene file to float rounding of the written text."""
        from orion_gb300 import scenegen
        return cls(desc=scenegen.scene_desc(scene))

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.port_scene_free(self._h)

    def trace(self, rays, brute_force=False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        prim = np.zeros(n, np.int32)
        lib().port_trace(self._h, n, _p(rays), int(brute_force), _p(t), _p(u), _p(v), _p(prim))
        return t, u, v, prim

    def camera_rays(self, index):
        idx = np.ascontiguousarray(index, np.int64)
        out = np.zeros((len(idx), 6), np.float32)
        lib().port_camera_rays(self._h, len(idx), _p(idx), _p(out))
        return out

    def render(self, spp=None, first_pass=0, max_depth=None, rr_depth=3, rows=None, threads=0):
        """FP32 film sums (H, W, 3) of PathTracing::render; `rows` = (row0, row1) band or a list of rows
        (the other rows stay zero)."""
        film = np.zeros((self.height, self.width, 3), np.float32)
        if rows is None:
            rows = (0, self.height)
        rl = np.ascontiguousarray(np.arange(*rows) if isinstance(rows, tuple) else rows, np.int32)
        rays = lib().port_render_rows(self._h, spp or self.spp, first_pass,
                                      self.max_depth if max_depth is None else max_depth, rr_depth, len(rl), _p(rl),
                                      _p(film), threads)
        if rays < 0:
            raise ValueError("row outside the image")
        return film, int(rays)

    def render_sppm(self, iterations=None, photons=None, radius=None, max_depth=None, threads=1):
        """FP32 film sums (H, W, 3) of SPPM::render: one estimate per iteration added to the film.
        Defaults: the scene's sppm parameters (photons < 0: W x H). threads=1: the reference's
        single-thread order (parity); 0: all cores with atomic photon sums (timing)."""
        it0, ph0, r0, md0 = self.sppm
        it = it0 if iterations is None else iterations
        ph = ph0 if photons is None else photons
        if ph < 0:
            ph = self.width * self.height
        film = np.zeros((self.height, self.width, 3), np.float32)
        rays = lib().port_render_sppm(self._h, it, ph, r0 if radius is None else radius,
                                      md0 if max_depth is None else max_depth, _p(film), threads)
        return film, int(rays)

    def render_pixels(self, pix, spp, first_pass=0, max_depth=None, rr_depth=3, threads=0):
        pix = np.ascontiguousarray(pix, np.int32).reshape(-1, 2)
        s = np.zeros((len(pix), 3), np.float64)
        q = np.zeros((len(pix), 3), np.float64)
        lib().port_render_pixels(self._h, len(pix), _p(pix), first_pass, spp,
                                 self.max_depth if max_depth is None else max_depth, rr_depth, _p(s), _p(q), threads)
        return s, q


def spread_rows(n: int, height: int) -> np.ndarray:
    """n image rows spread evenly over the whole image (the centre row of each of n equal bands)."""
    n = max(1, min(n, height))
    return np.unique(((np.arange(n) + 0.5) * height / n).astype(np.int32))


def time_sample(source, threads: int, seconds: float = 15.0, runs: int = 3, rr_depth: int = 3,
                keep_film: bool = False) -> dict:
    """Mpaths/s of the CPU oracle on a sample of image rows spread over the whole image, at the scene's spp.

    `source` is a scene file (parsed by the product's loader) or a generated scene
    (orion_gb300.scenegen.Scene, built in Python: the product library stays unloaded).
    The number of rows grows until one render takes about `seconds` / (runs + 2);
    that sample is then rendered `runs` more times and the median time is reported.
    keep_film: also return the film sums and rows ("film", "rows") for a parity check.
    """
    sc = Scene.load(source) if isinstance(source, str) else Scene.from_generated(source)
    # Each sample pass runs its rows in parallel (PathTracing::render's loop), so
    # start with several rows per thread.
    n = min(sc.height, 4 * max(1, threads or os.cpu_count() or 1))
    target = seconds / (runs + 2)
    while True:
        rows = spread_rows(n, sc.height)
        t = time.time()
        sc.render(rows=rows, threads=threads, rr_depth=rr_depth)
        dt = time.time() - t
        if dt > target or len(rows) >= sc.height:
            break
        n = min(sc.height, max(n * 2, int(n * target / max(dt, 1e-3))))
    times = []
    for _ in range(max(1, runs)):
        t = time.time()
        film, rays = sc.render(rows=rows, threads=threads, rr_depth=rr_depth)
        times.append(time.time() - t)
    dt = sorted(times)[len(times) // 2]
    paths = len(rows) * sc.width * sc.spp
    out = {"value": round(paths / dt / 1e6, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
           "sample": f"{len(rows)} image rows spread over all {sc.height} x {sc.width} px x {sc.spp} spp = {paths} "
                     f"paths, median of {len(times)} runs {dt:.2f} s, {rays} rays",
           "mrays_per_s": round(rays / dt / 1e6, 3), "rays_per_path": round(rays / paths, 4)}
    if keep_film:
        out["film"], out["rows"] = film, rows
    return out
