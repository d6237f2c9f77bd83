"""GB300 wavefront path tracer behind orion's scene-file / Integrator surface.

Host mirror of the reference's API for the path-tracing hot path, over the
C ABI in include/orion_gpu.h (liborion_gb300.so, built in-tree):

    reference (C++)                              here
    Parser(path).getRenderOption()               Parser(path, ctx).getRenderOption()
      src/util/parser.cpp:463-471
    integrator->render(*scene)                   ro.integrator.render(ro.scene)
      src/core/integrator.h:26
    camera->getFilm()->getAveraged()             ro.camera.getFilm().getAveraged()
      src/texture/rendertarget.cpp:28-37

Loading the library never falls back to anything else: if the shared
library or a CUDA device is missing, the call raises.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "liborion_gb300.so")

ORION_OK = 0
ERRORS = {-1: "invalid", -2: "io", -3: "parse", -4: "cuda", -5: "nomem", -6: "unsupported", -7: "device",
          -8: "not_ready", -9: "cancelled"}

MAT_MATTE, MAT_METAL, MAT_MIRROR, MAT_GLASS, MAT_PLASTIC, MAT_UBER = range(6)
INTEGRATOR_PATH, INTEGRATOR_SPPM = 0, 1
BATCH_POOLED, BATCH_WAVES = 0, 1
PROFILE_STAGES, PROFILE_TRAVERSAL = 1, 2
DIST_GGX, DIST_BECKMANN = 0, 1
LIGHT_AREA, LIGHT_POINT, LIGHT_SPOT, LIGHT_DISTANT, LIGHT_ENV = range(5)
NOALLOC_MAX_RAYS = 65536  # ORION_NOALLOC_MAX_RAYS
BXDF_ALL = 31
BXDF_NONSPECULAR = 31 & ~16


class OrionError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Material(C.Structure):
    _fields_ = [("type", C.c_int32), ("distribution", C.c_int32), ("has_sigma", C.c_int32), ("reserved", C.c_int32),
                ("Kd", C.c_float * 3), ("Ks", C.c_float * 3), ("Kr", C.c_float * 3), ("Kt", C.c_float * 3),
                ("opacity", C.c_float * 3), ("eta_rgb", C.c_float * 3), ("k", C.c_float * 3),
                ("sigma", C.c_float), ("roughness", C.c_float), ("eta", C.c_float),
                ("tex", C.c_int32 * 8)]  # per ORION_TEX_* input: 0 = constant, k = image k - 1


class Light(C.Structure):
    _fields_ = [("type", C.c_int32), ("prim", C.c_int32), ("L", C.c_float * 3), ("p", C.c_float * 3),
                ("dir", C.c_float * 3), ("l2w", C.c_float * 12), ("w2l", C.c_float * 12),
                ("cos_total", C.c_float), ("cos_falloff", C.c_float), ("image", C.c_int32), ("reserved", C.c_int32)]


class SppmParams(C.Structure):
    _fields_ = [("iterations", C.c_int32), ("photons_per_iter", C.c_int32), ("initial_radius", C.c_float),
                ("max_depth", C.c_int32)]


class Image(C.Structure):
    _fields_ = [("width", C.c_int32), ("height", C.c_int32), ("rgb", C.c_void_p)]


class Camera(C.Structure):
    _fields_ = [("c2w", C.c_float * 16), ("fov", C.c_float), ("lens_radius", C.c_float),
                ("focal_distance", C.c_float), ("width", C.c_int32), ("height", C.c_int32)]


class SceneDesc(C.Structure):
    _fields_ = [("num_prims", C.c_int64), ("positions", C.c_void_p), ("normals", C.c_void_p), ("uvs", C.c_void_p),
                ("material_of_prim", C.c_void_p), ("light_of_prim", C.c_void_p), ("num_materials", C.c_int32),
                ("num_lights", C.c_int32), ("materials", C.c_void_p), ("lights", C.c_void_p), ("camera", Camera),
                ("spp", C.c_int32), ("max_depth", C.c_int32), ("num_images", C.c_int32), ("reserved", C.c_int32),
                ("images", C.c_void_p), ("integrator", C.c_int32), ("reserved2", C.c_int32),
                ("sppm", SppmParams)]


class GpuOpts(C.Structure):
    _fields_ = [("device", C.c_int32), ("reserved", C.c_int32), ("memory_budget", C.c_int64),
                ("sobol_path", C.c_char_p)]


class RenderParams(C.Structure):
    _fields_ = [("spp", C.c_int32), ("max_depth", C.c_int32), ("rr_depth", C.c_int32), ("flags", C.c_int32),
                ("first_pass", C.c_int64), ("wave_paths", C.c_int32), ("reserved", C.c_int32)]


class RenderStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("rays", C.c_int64), ("ext_rays", C.c_int64), ("shadow_rays", C.c_int64),
                ("mis_rays", C.c_int64), ("kernel_launches", C.c_int64), ("device_ms", C.c_double)]


class StageTimes(C.Structure):
    _fields_ = [("ms", C.c_double * 8), ("launches", C.c_int64 * 8)]


class TraversalWork(C.Structure):
    _fields_ = [("rays", C.c_int64 * 3), ("nodes", C.c_int64 * 3), ("triangles", C.c_int64 * 3)]


STAGES = ("camera", "trace_ext", "shade", "trace_shadow", "trace_mis", "resolve", "film", "other")


class Job(C.Structure):
    _fields_ = [("scene", C.c_int32), ("reserved", C.c_int32), ("params", RenderParams), ("camera", C.c_void_p),
                ("sum", C.c_void_p), ("sumsq", C.c_void_p), ("count", C.c_void_p), ("sum32", C.c_void_p)]


class BatchStats(C.Structure):
    _fields_ = [("paths", C.c_int64), ("rays", C.c_int64), ("iterations", C.c_int64), ("capacity", C.c_int64),
                ("device_ms", C.c_double)]


class LaunchConfig(C.Structure):
    _fields_ = [("trace_block", C.c_int32), ("shade_block", C.c_int32), ("smem_stack", C.c_int32),
                ("blocks_per_sm", C.c_int32), ("wave_paths", C.c_int32), ("batch_slots", C.c_int32),
                ("refill_below", C.c_int32), ("streams", C.c_int32)]

class ServerOpts(C.Structure):
    _fields_ = [("memory_budget", C.c_int64), ("spp_chunk", C.c_int32), ("max_jobs", C.c_int32)]


class RequestStatus(C.Structure):
    _fields_ = [("state", C.c_int32), ("spp_done", C.c_int32), ("spp_total", C.c_int32), ("width", C.c_int32),
                ("height", C.c_int32), ("reserved", C.c_int32), ("t_submit", C.c_double), ("t_admit", C.c_double),
                ("t_done", C.c_double)]


class ServerStats(C.Structure):
    _fields_ = [("submitted", C.c_int64), ("completed", C.c_int64), ("launches", C.c_int64), ("paths", C.c_int64),
                ("resident_scenes", C.c_int64), ("bytes_in_use", C.c_int64), ("device_ms", C.c_double)]


REQ_QUEUED, REQ_RUNNING, REQ_DONE, REQ_CANCELLED, REQ_FAILED = range(5)

_lib = None


def library() -> C.CDLL:
    """The product library; raises if it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: run __graft_entry__.build() first")
        lib = C.CDLL(LIB_PATH)
        vp, i32, i64 = C.c_void_p, C.c_int32, C.c_int64
        sigs = {
            "orion_last_error": (C.c_char_p, []),
            "orion_scene_load_ori": (i32, [C.c_char_p, C.POINTER(vp)]),
            "orion_scene_from_desc": (i32, [C.POINTER(SceneDesc), C.POINTER(vp)]),
            "orion_scene_get_desc": (i32, [vp, C.POINTER(SceneDesc)]),
            "orion_scene_free": (None, [vp]),
            "orion_gpu_create": (i32, [C.POINTER(GpuOpts), C.POINTER(vp)]),
            "orion_gpu_destroy": (i32, [vp]),
            "orion_gpu_scene_upload": (i32, [vp, vp, C.POINTER(i32)]),
            "orion_gpu_scene_release": (i32, [vp, i32]),
            "orion_gpu_scene_bytes": (i32, [vp, i32, C.POINTER(i64)]),
            "orion_gpu_render": (i32, [vp, i32, C.POINTER(RenderParams), vp, vp]),
            "orion_gpu_render_fp64": (i32, [vp, i32, C.POINTER(RenderParams), vp, vp]),
            "orion_gpu_render_sppm": (i32, [vp, i32, C.POINTER(SppmParams), vp, vp]),
            "orion_gpu_set_batch_mode": (i32, [vp, i32]),
            "orion_gpu_last_stats": (i32, [vp, C.POINTER(RenderStats)]),
            "orion_gpu_set_profiling": (i32, [vp, i32]),
            "orion_gpu_stage_times": (i32, [vp, C.POINTER(StageTimes)]),
            "orion_gpu_traversal_work": (i32, [vp, C.POINTER(TraversalWork)]),
            "orion_film_write_bmp": (i32, [C.c_char_p, i32, i32, vp]),
            "orion_gpu_render_batch": (i32, [vp, i32, vp, C.POINTER(BatchStats)]),
            "orion_gpu_get_config": (i32, [vp, C.POINTER(LaunchConfig)]),
            "orion_gpu_set_config": (i32, [vp, C.POINTER(LaunchConfig)]),
            "orion_gpu_autotune": (i32, [vp, i32, i32, C.c_double, C.POINTER(LaunchConfig), C.POINTER(C.c_double)]),
            "orion_gpu_autotune_batch": (i32, [vp, i32, vp, i32, C.c_double, C.POINTER(LaunchConfig),
                                               C.POINTER(C.c_double)]),
            "orion_server_create": (i32, [vp, C.POINTER(ServerOpts), C.POINTER(vp)]),
            "orion_server_submit": (i32, [vp, vp, C.POINTER(RenderParams), vp, C.POINTER(i64)]),
            "orion_server_status": (i32, [vp, i64, C.POINTER(RequestStatus)]),
            "orion_server_wait": (i32, [vp, i64, C.c_double]),
            "orion_server_result": (i32, [vp, i64, vp, vp, vp]),
            "orion_server_preview": (i32, [vp, i64, vp, i32]),
            "orion_server_cancel": (i32, [vp, i64]),
            "orion_server_release": (i32, [vp, i64]),
            "orion_server_stats_get": (i32, [vp, C.POINTER(ServerStats)]),
            "orion_server_destroy": (i32, [vp]),
            "orion_gpu_sobol": (i32, [vp, i64, vp, vp, vp]),
            "orion_gpu_trace": (i32, [vp, i32, i64, vp, i32, vp, vp, vp, vp]),
            "orion_gpu_trace_noalloc": (i32, [vp, i32, i64, vp, i32, vp, vp, vp, vp]),
            "orion_gpu_trace_wave": (i32, [vp, i32, i64, vp, i32, vp, vp, vp, vp]),
            "orion_gpu_set_test_limits": (i32, [vp, i32, i32]),
            "orion_gpu_mem_info": (i32, [vp, vp, vp]),
            "orion_gpu_camera_rays": (i32, [vp, i32, i64, vp, vp]),
            "orion_gpu_bsdf_eval": (i32, [vp, C.POINTER(Material), i64, vp, vp, vp, vp, i32, vp, vp, vp, vp, vp,
                                          vp, vp]),
        }
        for name, (res, args) in sigs.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def _check(rc: int) -> None:
    if rc != ORION_OK:
        raise OrionError(rc, library().orion_last_error().decode())


def _ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


# ------------------------------------------------------------------ scenes


def desc_from_arrays(positions, normals, material_of_prim, materials, lights, camera: Camera, spp: int,
                     max_depth: int, light_of_prim=None, uvs=None, images=None, sppm=None):
    """An orion_scene_desc over the given arrays, built without the library: (desc, keep), where
    `keep` holds the arrays the desc points into and must outlive every use of the desc.
    Arguments as HostScene.from_arrays."""
    pos = np.ascontiguousarray(positions, dtype=np.float32).reshape(-1, 9)
    nrm = np.ascontiguousarray(normals, dtype=np.float32).reshape(-1, 9)
    mop = np.ascontiguousarray(material_of_prim, dtype=np.int32)
    lop = np.ascontiguousarray(light_of_prim if light_of_prim is not None else np.full(len(pos), -1), np.int32)
    mats = (Material * len(materials))(*materials)
    lts = (Light * max(1, len(lights)))(*lights)
    d = SceneDesc()
    d.num_prims = len(pos)
    d.positions, d.normals = pos.ctypes.data, nrm.ctypes.data
    uva = np.ascontiguousarray(uvs, np.float32).reshape(-1, 6) if uvs is not None else None
    if uva is not None and len(uva) != len(pos):
        raise ValueError("uvs must hold 6 floats per primitive")
    d.uvs = uva.ctypes.data if uva is not None else None
    d.material_of_prim, d.light_of_prim = mop.ctypes.data, lop.ctypes.data
    d.num_materials, d.num_lights = len(materials), len(lights)
    d.materials, d.lights = C.addressof(mats), C.addressof(lts)
    d.camera, d.spp, d.max_depth = camera, spp, max_depth
    imgs = [np.ascontiguousarray(im, np.float32) for im in (images or [])]
    recs = (Image * max(1, len(imgs)))(*[Image(im.shape[1], im.shape[0], im.ctypes.data) for im in imgs])
    d.num_images, d.images = len(imgs), C.addressof(recs)
    if sppm is not None:
        d.integrator = INTEGRATOR_SPPM
        d.sppm = SppmParams(sppm["iterations"], sppm["photons"], sppm["radius"], sppm["max_depth"])
        d.spp, d.max_depth = sppm["iterations"], sppm["max_depth"]
    return d, (pos, nrm, mop, lop, mats, lts, uva, imgs, recs)


class HostScene:
    """A parsed scene on the host (flat primitive arrays, materials, lights, camera)."""

    def __init__(self, handle: int, keep=None):
        self._h = C.c_void_p(handle)
        self._keep = keep

    @classmethod
    def load(cls, path: str) -> "HostScene":
        h = C.c_void_p()
        _check(library().orion_scene_load_ori(os.fsencode(path), C.byref(h)))
        return cls(h.value)

    @classmethod
    def from_arrays(cls, positions, normals, material_of_prim, materials, lights, camera: Camera, spp: int,
                    max_depth: int, light_of_prim=None, uvs=None, images=None, sppm=None) -> "HostScene":
        """images: list of (H, W, 3) float arrays, referenced 1-based by Light.image and Material.tex;
        uvs: texture coordinates per primitive corner (T x 6) or None; sppm: dict (iterations, photons,
        radius, max_depth) for an <Integrator type="sppm"> scene."""
        d, keep = desc_from_arrays(positions, normals, material_of_prim, materials, lights, camera, spp, max_depth,
                                   light_of_prim=light_of_prim, uvs=uvs, images=images, sppm=sppm)
        h = C.c_void_p()
        _check(library().orion_scene_from_desc(C.byref(d), C.byref(h)))
        del keep  # orion_scene_from_desc copied every array
        return cls(h.value)

    def desc(self) -> SceneDesc:
        d = SceneDesc()
        _check(library().orion_scene_get_desc(self._h, C.byref(d)))
        return d

    def arrays(self) -> dict:
        d = self.desc()
        T = d.num_prims

        def arr(ptr, n, dt):
            if not ptr or n == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(C.cast(ptr, C.POINTER(np.ctypeslib.as_ctypes_type(dt))), (n,)).copy()

        return {
            "positions": arr(d.positions, 9 * T, np.float32).reshape(T, 9),
            "normals": arr(d.normals, 9 * T, np.float32).reshape(T, 9),
            "uvs": arr(d.uvs, 6 * T, np.float32).reshape(T, 6),
            "material_of_prim": arr(d.material_of_prim, T, np.int32),
            "light_of_prim": arr(d.light_of_prim, T, np.int32),
            "materials": [Material.from_buffer_copy(C.cast(d.materials, C.POINTER(Material))[i])
                          for i in range(d.num_materials)],
            "lights": [Light.from_buffer_copy(C.cast(d.lights, C.POINTER(Light))[i]) for i in range(d.num_lights)],
            "camera": d.camera, "spp": d.spp, "max_depth": d.max_depth,
            "images": [arr(im.rgb, 3 * im.width * im.height, np.float32).reshape(im.height, im.width, 3)
                       for im in (C.cast(d.images, C.POINTER(Image))[i] for i in range(d.num_images))],
        }

    def __del__(self):
        if getattr(self, "_h", None) and self._h.value and _lib is not None:
            _lib.orion_scene_free(self._h)
            self._h = C.c_void_p()


# ----------------------------------------------------------------- context


class Context:
    """One CUDA device: resident scenes, path-state pool, stream."""

    def __init__(self, device: int = 0, memory_budget: int = 0):
        opts = GpuOpts(device=device, memory_budget=memory_budget, sobol_path=None)
        h = C.c_void_p()
        _check(library().orion_gpu_create(C.byref(opts), C.byref(h)))
        self._h = h
        self._scene_sppm = {}  # scene id -> its sppm parameters

    def close(self):
        if self._h and self._h.value:
            library().orion_gpu_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def upload(self, scene: HostScene) -> int:
        sid = C.c_int32()
        _check(library().orion_gpu_scene_upload(self._h, scene._h, C.byref(sid)))
        p = scene.desc().sppm
        self._scene_sppm[sid.value] = (p.iterations, p.photons_per_iter, p.initial_radius, p.max_depth)
        return sid.value

    def release(self, sid: int) -> None:
        _check(library().orion_gpu_scene_release(self._h, sid))

    def scene_bytes(self, sid: int) -> int:
        b = C.c_int64()
        _check(library().orion_gpu_scene_bytes(self._h, sid, C.byref(b)))
        return b.value

    def render(self, sid: int, width: int, height: int, spp: int = 0, max_depth: int = -1, rr_depth: int = 3,
               first_pass: int = 0, wave_paths: int = 0, fp64: bool = False, out: tuple | None = None):
        """Film sums: FP32 (H, W, 3) sums and (H, W) counts; or FP64 (sum, sumsq) if fp64.
        out: arrays of those shapes and types to write into (reused host buffers), returned."""
        p = RenderParams(spp=spp, max_depth=max_depth, rr_depth=rr_depth, flags=1 if fp64 else 0,
                         first_pass=first_pass, wave_paths=wave_paths)
        if out is not None:
            a, b = out
            want = (np.float64, np.float64) if fp64 else (np.float32, np.uint32)
            if a.shape != (height, width, 3) or b.shape[:2] != (height, width) or (a.dtype, b.dtype) != want \
                    or not (a.flags.c_contiguous and b.flags.c_contiguous):
                raise ValueError("out arrays do not match the film")
        if fp64:
            s, q = out if out is not None else (np.zeros((height, width, 3)), np.zeros((height, width, 3)))
            _check(library().orion_gpu_render_fp64(self._h, sid, C.byref(p), _ptr(s), _ptr(q)))
            return s, q
        img, cnt = out if out is not None else (np.zeros((height, width, 3), np.float32),
                                                np.zeros((height, width), np.uint32))
        _check(library().orion_gpu_render(self._h, sid, C.byref(p), _ptr(img), _ptr(cnt)))
        return img, cnt

    def render_sppm(self, sid: int, width: int, height: int, iterations: int | None = None,
                    photons: int | None = None, radius: float | None = None, max_depth: int | None = None):
        """SPPM::render: FP32 (H, W, 3) film sums (one estimate per iteration) and (H, W) counts.
        Parameters left None come from the scene's <Integrator type="sppm">."""
        p = None
        if any(x is not None for x in (iterations, photons, radius, max_depth)):
            d = self._scene_sppm.get(sid)
            if d is None:
                raise OrionError(-1, "sppm parameters of this scene are unknown: pass all four")
            p = SppmParams(iterations if iterations is not None else d[0], photons if photons is not None else d[1],
                           radius if radius is not None else d[2], max_depth if max_depth is not None else d[3])
        img = np.zeros((height, width, 3), np.float32)
        cnt = np.zeros((height, width), np.uint32)
        _check(library().orion_gpu_render_sppm(self._h, sid, C.byref(p) if p is not None else None, _ptr(img),
                                               _ptr(cnt)))
        return img, cnt

    def last_stats(self) -> dict:
        s = RenderStats()
        _check(library().orion_gpu_last_stats(self._h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in RenderStats._fields_}

    def set_profiling(self, on: bool | int) -> None:
        """True or PROFILE_STAGES: per-stage times; PROFILE_TRAVERSAL: count BVH work; False: off."""
        _check(library().orion_gpu_set_profiling(self._h, int(on)))

    def traversal_work(self) -> dict:
        """BVH work of the last plain render made under PROFILE_TRAVERSAL, per ray kind."""
        t = TraversalWork()
        _check(library().orion_gpu_traversal_work(self._h, C.byref(t)))
        return {kind: {"rays": t.rays[i], "nodes": t.nodes[i], "triangles": t.triangles[i]}
                for i, kind in enumerate(("ext", "shadow", "mis"))}

    def stage_times(self) -> dict:
        t = StageTimes()
        _check(library().orion_gpu_stage_times(self._h, C.byref(t)))
        return {name: {"ms": t.ms[i], "launches": t.launches[i]} for i, name in enumerate(STAGES)}

    def render_batch(self, jobs: list, sumsq: bool = True, fp32: bool = False, outs: list | None = None) -> tuple:
        """jobs: dicts with sid, width, height and optional spp, max_depth, rr_depth, first_pass, camera.

        Returns ([(sum, sumsq, count) per job], stats): FP64 (H, W, 3) sums and
        sums of squares (None when sumsq=False), (H, W) sample counts. fp32: the
        sums come back rounded to FP32 on the device (float32 arrays, sumsq None).
        outs: the list an earlier call returned, to write into again (reused host buffers).
        """
        arr, outs = self._job_array(jobs, films=True, sumsq=sumsq and not fp32, fp32=fp32, reuse=outs)
        st = BatchStats()
        _check(library().orion_gpu_render_batch(self._h, len(jobs), C.cast(arr, C.c_void_p), C.byref(st)))
        return outs, {k: getattr(st, k) for k, _ in BatchStats._fields_}

    @staticmethod
    def _job_array(jobs: list, films: bool, sumsq: bool = True, fp32: bool = False, reuse: list | None = None):
        arr = (Job * max(1, len(jobs)))()
        outs = []
        if reuse is not None and len(reuse) != len(jobs):
            raise ValueError("outs must hold one entry per job")
        for i, j in enumerate(jobs):
            arr[i].scene = j["sid"]
            arr[i].params = RenderParams(spp=j.get("spp", 0), max_depth=j.get("max_depth", -1),
                                         rr_depth=j.get("rr_depth", 3), first_pass=j.get("first_pass", 0))
            if j.get("camera") is not None:
                arr[i].camera = C.addressof(j["camera"])
            if films:
                h, w = j["height"], j["width"]
                if reuse is not None:
                    s, q, c = reuse[i]
                    if s.shape != (h, w, 3) or s.dtype != (np.float32 if fp32 else np.float64) or \
                            (q is None) == sumsq or c.shape != (h, w):
                        raise ValueError(f"outs[{i}] does not match job {i}")
                else:
                    s = np.empty((h, w, 3), np.float32 if fp32 else np.float64)
                    q = np.empty((h, w, 3), np.float64) if sumsq else None
                    c = np.empty((h, w), np.uint32)
                outs.append((s, q, c))
                if fp32:
                    arr[i].sum32 = s.ctypes.data
                else:
                    arr[i].sum = s.ctypes.data
                arr[i].count = c.ctypes.data
                arr[i].sumsq = q.ctypes.data if sumsq else None
        return arr, outs

    def autotune_batch(self, jobs: list, spp_cap: int = 0, budget_ms: float = 4000.0) -> tuple:
        """Tune the batched engine's launch knobs and path-slot count on `jobs` (render_batch job dicts)."""
        arr, _ = self._job_array(jobs, films=False)
        c = LaunchConfig()
        mp = C.c_double()
        _check(library().orion_gpu_autotune_batch(self._h, len(jobs), C.cast(arr, C.c_void_p), spp_cap, budget_ms,
                                                  C.byref(c), C.byref(mp)))
        return {k: getattr(c, k) for k, _ in LaunchConfig._fields_}, mp.value

    def set_batch_mode(self, mode: int) -> None:
        """BATCH_WAVES (default): batches run as waves over the jobs' work list; BATCH_POOLED: a refilled pool."""
        _check(library().orion_gpu_set_batch_mode(self._h, mode))

    def get_config(self) -> dict:
        c = LaunchConfig()
        _check(library().orion_gpu_get_config(self._h, C.byref(c)))
        return {k: getattr(c, k) for k, _ in LaunchConfig._fields_}

    def set_config(self, **kw) -> None:
        cur = self.get_config()
        cur.update(kw)
        _check(library().orion_gpu_set_config(self._h, C.byref(LaunchConfig(**cur))))

    def autotune(self, sid: int, spp: int = 1, budget_ms: float = 2000.0) -> tuple:
        c = LaunchConfig()
        mp = C.c_double()
        _check(library().orion_gpu_autotune(self._h, sid, spp, budget_ms, C.byref(c), C.byref(mp)))
        return {k: getattr(c, k) for k, _ in LaunchConfig._fields_}, mp.value

    # component hooks -----------------------------------------------------
    def sobol(self, index, dim) -> np.ndarray:
        index = np.ascontiguousarray(index, np.uint64)
        dim = np.ascontiguousarray(dim, np.uint32)
        out = np.zeros(len(index), np.float32)
        _check(library().orion_gpu_sobol(self._h, len(index), _ptr(index), _ptr(dim), _ptr(out)))
        return out

    def trace(self, sid: int, rays, any_hit: bool = False):
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        prim = np.zeros(n, np.int32)
        _check(library().orion_gpu_trace(self._h, sid, n, _ptr(rays), int(any_hit), _ptr(t), _ptr(u), _ptr(v),
                                         _ptr(prim)))
        return t, u, v, prim

    def trace_wave(self, sid: int, rays, any_hit: bool = False):
        """trace() through the renderer's persistent trace kernels (rays as a wave's extension or
        shadow rays): tnear must be 0; closest-hit rays are unbounded; occluded rays get prim 1."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        prim = np.zeros(n, np.int32)
        _check(library().orion_gpu_trace_wave(self._h, sid, n, _ptr(rays), int(any_hit), _ptr(t), _ptr(u), _ptr(v),
                                              _ptr(prim)))
        return t, u, v, prim

    def mem_info(self) -> tuple:
        """(free, total) bytes of the context's device."""
        f, t = C.c_int64(), C.c_int64()
        _check(library().orion_gpu_mem_info(self._h, C.byref(f), C.byref(t)))
        return f.value, t.value

    def set_test_limits(self, stack_entries: int = 0, batch_iterations: int = 0) -> None:
        """Failure-path test knobs: a 2-entry traversal stack for plain renders, a batch-loop iteration cap."""
        _check(library().orion_gpu_set_test_limits(self._h, stack_entries, batch_iterations))

    def trace_noalloc(self, sid: int, rays, any_hit: bool = False):
        """trace() through a fixed device scratch of NOALLOC_MAX_RAYS rays: no device allocation."""
        rays = np.ascontiguousarray(rays, np.float32).reshape(-1, 8)
        n = len(rays)
        t, u, v = (np.zeros(n, np.float32) for _ in range(3))
        prim = np.zeros(n, np.int32)
        _check(library().orion_gpu_trace_noalloc(self._h, sid, n, _ptr(rays), int(any_hit), _ptr(t), _ptr(u),
                                                 _ptr(v), _ptr(prim)))
        return t, u, v, prim

    def camera_rays(self, sid: int, sample_index) -> np.ndarray:
        idx = np.ascontiguousarray(sample_index, np.int64)
        out = np.zeros((len(idx), 6), np.float32)
        _check(library().orion_gpu_camera_rays(self._h, sid, len(idx), _ptr(idx), _ptr(out)))
        return out

    def bsdf_eval(self, mat: Material, frame, wo, wi, rnd, type_mask: int = BXDF_ALL) -> dict:
        return _bsdf_call(lambda *a: library().orion_gpu_bsdf_eval(self._h, *a), mat, frame, wo, wi, rnd, type_mask)


def _bsdf_call(fn, mat, frame, wo, wi, rnd, type_mask):
    frame = np.ascontiguousarray(frame, np.float32).reshape(-1, 12)
    n = len(frame)
    wo = np.ascontiguousarray(wo, np.float32).reshape(n, 3)
    wi = np.ascontiguousarray(wi, np.float32).reshape(n, 3)
    rnd = np.ascontiguousarray(rnd, np.float32).reshape(n, 2)
    out = {"f": np.zeros((n, 3), np.float32), "pdf": np.zeros(n, np.float32), "sf": np.zeros((n, 3), np.float32),
           "swi": np.zeros((n, 3), np.float32), "spdf": np.zeros(n, np.float32), "stype": np.zeros(n, np.int32),
           "nbxdf": np.zeros(n, np.int32)}
    _check(fn(C.byref(mat), n, _ptr(frame), _ptr(wo), _ptr(wi), _ptr(rnd), type_mask, _ptr(out["f"]),
              _ptr(out["pdf"]), _ptr(out["sf"]), _ptr(out["swi"]), _ptr(out["spdf"]), _ptr(out["stype"]),
              _ptr(out["nbxdf"])))
    return out


# ------------------------------------------- reference-shaped host surface


class RenderTarget:
    """The film: per-pixel FP32 sums and sample counts (src/texture/rendertarget.h:15-33)."""

    def __init__(self, width: int, height: int):
        self.width, self.height = width, height
        self.data = np.zeros((height, width, 3), np.float32)
        self.counter = np.zeros((height, width), np.uint32)

    def getWidth(self):
        return self.width

    def getHeight(self):
        return self.height

    def sample(self, x: int, y: int):
        return self.data[y, x]

    def getAveraged(self) -> np.ndarray:
        with np.errstate(invalid="ignore", divide="ignore"):
            return self.data / self.counter[..., None].astype(np.float32)


def saveAsBmp(image: np.ndarray, path: str) -> None:
    """saveAsBmp (src/core/texture.cpp:77-136) of an averaged (H, W, 3) film."""
    img = np.ascontiguousarray(image, np.float32)
    if img.ndim != 3 or img.shape[2] != 3:
        raise ValueError("expected an (H, W, 3) image")
    h, w = img.shape[:2]
    _check(library().orion_film_write_bmp(os.fsencode(path), w, h, _ptr(img)))


class CameraHandle:
    def __init__(self, film: RenderTarget):
        self._film = film

    def getFilm(self) -> RenderTarget:
        return self._film


@dataclass
class SceneHandle:
    ctx: Context
    sid: int
    host: HostScene


class PathTracing:
    """GPU stand-in for PathTracing (src/integrator/path.h:16-35): render() fills the camera's film."""

    def __init__(self, camera: CameraHandle, max_depth: int, n_samples: int, rr_depth: int = 3):
        self.camera, self.maxDepth, self.nSamples, self.rr_depth = camera, max_depth, n_samples, rr_depth
        self.stats = None

    def render(self, scene: SceneHandle) -> None:
        film = self.camera.getFilm()
        img, cnt = scene.ctx.render(scene.sid, film.width, film.height, spp=self.nSamples, max_depth=self.maxDepth,
                                    rr_depth=self.rr_depth)
        film.data, film.counter = img, cnt
        self.stats = scene.ctx.last_stats()


class SPPM:
    """GPU stand-in for SPPM (src/integrator/sppm.h:16-29): render() fills the camera's film."""

    def __init__(self, camera: CameraHandle, max_depth: int, n_iterations: int, photons_per_iter: int,
                 radius: float):
        self.camera, self.maxDepth, self.nIterations = camera, max_depth, n_iterations
        self.photonPerIteration, self.initialSearchRadius = photons_per_iter, radius
        self.stats = None

    def render(self, scene: SceneHandle) -> None:
        film = self.camera.getFilm()
        img, cnt = scene.ctx.render_sppm(scene.sid, film.width, film.height, iterations=self.nIterations,
                                         photons=self.photonPerIteration, radius=self.initialSearchRadius,
                                         max_depth=self.maxDepth)
        film.data, film.counter = img, cnt
        self.stats = scene.ctx.last_stats()


@dataclass
class RenderOption:
    scene: SceneHandle
    camera: CameraHandle
    integrator: PathTracing | SPPM


class Parser:
    """Parser(path) -> getRenderOption(), with the scene already resident on `ctx`."""

    def __init__(self, path: str, ctx: Context | None = None):
        self.ctx = ctx or Context()
        self.host = HostScene.load(path)
        d = self.host.desc()
        sid = self.ctx.upload(self.host)
        film = RenderTarget(d.camera.width, d.camera.height)
        cam = CameraHandle(film)
        if d.integrator == INTEGRATOR_SPPM:
            p = d.sppm
            integ = SPPM(cam, p.max_depth, p.iterations, p.photons_per_iter, p.initial_radius)
        else:
            integ = PathTracing(cam, d.max_depth, d.spp)
        self._ro = RenderOption(SceneHandle(self.ctx, sid, self.host), cam, integ)

    def getRenderOption(self) -> RenderOption:
        return self._ro


# ------------------------------------------------------------------ serving


def look_at_camera(eye, look, up, fov: float, width: int, height: int, lens_radius: float = 0.0,
                   focal_distance: float = 0.0) -> Camera:
    """A pinhole / thin-lens view for serving requests (camera-to-world as the reference's lookAt)."""
    f = np.asarray(look, np.float64) - np.asarray(eye, np.float64)
    f /= np.linalg.norm(f)
    s = np.cross(f, np.asarray(up, np.float64))
    s /= np.linalg.norm(s)
    u = np.cross(s, f)
    m = np.eye(4)
    m[:3, 0], m[:3, 1], m[:3, 2], m[:3, 3] = s, u, -f, eye
    cam = Camera()
    cam.c2w[:] = [float(x) for x in m.astype(np.float32).ravel()]
    cam.fov, cam.lens_radius, cam.focal_distance = fov, lens_radius, focal_distance
    cam.width, cam.height = width, height
    return cam


class Server:
    """Request loop on a context: submit(scene, view, params) -> ticket; wait; result; release."""

    def __init__(self, ctx: Context, memory_budget: int = 0, spp_chunk: int = 4, max_jobs: int = 512):
        h = C.c_void_p()
        _check(library().orion_server_create(ctx._h, C.byref(ServerOpts(memory_budget, spp_chunk, max_jobs)),
                                             C.byref(h)))
        self._h, self.ctx = h, ctx
        self._keep = {}

    def submit(self, scene: HostScene, spp: int = 0, max_depth: int = -1, rr_depth: int = 3, first_pass: int = 0,
               camera: Camera | None = None) -> int:
        t = C.c_int64()
        p = RenderParams(spp=spp, max_depth=max_depth, rr_depth=rr_depth, first_pass=first_pass)
        cam = C.byref(camera) if camera is not None else None
        _check(library().orion_server_submit(self._h, scene._h, C.byref(p), cam, C.byref(t)))
        self._keep[t.value] = scene
        return t.value

    def status(self, ticket: int) -> dict:
        st = RequestStatus()
        _check(library().orion_server_status(self._h, ticket, C.byref(st)))
        return {k: getattr(st, k) for k, _ in RequestStatus._fields_}

    def wait(self, ticket: int, timeout: float = 60.0) -> bool:
        rc = library().orion_server_wait(self._h, ticket, timeout)
        if rc == -8:
            return False
        _check(rc)
        return True

    def result(self, ticket: int):
        st = self.status(ticket)
        h, w = st["height"], st["width"]
        s, q = np.zeros((h, w, 3), np.float64), np.zeros((h, w, 3), np.float64)
        c = np.zeros((h, w), np.uint32)
        _check(library().orion_server_result(self._h, ticket, _ptr(s), _ptr(q), _ptr(c)))
        return s, q, c

    def preview(self, ticket: int, bottom_up: bool = False) -> np.ndarray:
        """The request's film so far as (H, W, 4) uint8 B, G, R, 255 (saveAsBmp's pixels), made on the device."""
        st = self.status(ticket)
        out = np.zeros((st["height"], st["width"], 4), np.uint8)
        _check(library().orion_server_preview(self._h, ticket, _ptr(out), 1 if bottom_up else 0))
        return out

    def cancel(self, ticket: int) -> None:
        _check(library().orion_server_cancel(self._h, ticket))

    def release(self, ticket: int) -> None:
        _check(library().orion_server_release(self._h, ticket))
        self._keep.pop(ticket, None)

    def stats(self) -> dict:
        st = ServerStats()
        _check(library().orion_server_stats_get(self._h, C.byref(st)))
        return {k: getattr(st, k) for k, _ in ServerStats._fields_}

    def close(self) -> None:
        if self._h and self._h.value:
            library().orion_server_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
