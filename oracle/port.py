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
            raise OSError(f"{LIB} missing: build with orion_gb300.build.build_port()")
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
    """The oracle's copy of a scene, built from the same flat record the GPU path receives."""

    def __init__(self, host_scene):
        import orion_gb300 as og
        self._host = host_scene
        d = host_scene.desc()
        self._h = C.c_void_p(lib().port_scene_create(C.byref(d)))
        info = np.zeros(5, np.int32)
        lib().port_scene_info(self._h, _p(info))
        self.width, self.height, self.spp, self.max_depth, self.num_lights = (int(x) for x in info)
        self.integrator = int(d.integrator)
        self.sppm = (int(d.sppm.iterations), int(d.sppm.photons_per_iter), float(d.sppm.initial_radius),
                     int(d.sppm.max_depth))
        self._og = og

    @classmethod
    def load(cls, path: str) -> "Scene":
        import orion_gb300 as og
        return cls(og.HostScene.load(path))

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
        """FP32 film sums (H, W, 3) of PathTracing::render; `rows` = (row0, row1) band."""
        film = np.zeros((self.height, self.width, 3), np.float32)
        r0, r1 = rows if rows is not None else (0, self.height)
        rays = lib().port_render(self._h, spp or self.spp, first_pass,
                                 self.max_depth if max_depth is None else max_depth, rr_depth, r0, r1, _p(film),
                                 threads)
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


def time_sample(path: str, threads: int, seconds: float = 15.0, runs: int = 3) -> dict:
    """Mpaths/s of the CPU oracle on a band of image rows at the scene's spp.

    The band grows until one render takes about `seconds` / (runs + 2); the
    measured band is then rendered `runs` more times and the median time is
    reported.
    """
    sc = Scene.load(path)
    rows = 1
    target = seconds / (runs + 2)

    def band(n):  # n rows from the middle of the image, moved up to stay inside it
        r0 = max(0, min(sc.height // 2, sc.height - n))
        return (r0, r0 + n)

    while True:
        t = time.time()
        sc.render(rows=band(rows), threads=threads)
        dt = time.time() - t
        if dt > target or rows >= sc.height:
            break
        rows = min(sc.height, max(rows * 2, int(rows * target / max(dt, 1e-3))))
    times = []
    for _ in range(max(1, runs)):
        t = time.time()
        _, rays = sc.render(rows=band(rows), threads=threads)
        times.append(time.time() - t)
    dt = sorted(times)[len(times) // 2]
    paths = rows * sc.width * sc.spp
    return {"value": round(paths / dt / 1e6, 4), "unit": "Mpaths/s", "cores": threads, "kind": "port",
            "sample": f"{rows} image rows x {sc.width} px x {sc.spp} spp = {paths} paths, median of "
                      f"{len(times)} runs {dt:.2f} s, {rays} rays", "mrays_per_s": round(rays / dt / 1e6, 3)}
