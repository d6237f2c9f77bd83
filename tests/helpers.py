"""Shared test helpers: deterministic inputs, scene files, fixture access.

Inputs come from SplitMix64 (not numpy's Generator) so the fixture script
and the tests produce identical values on every machine.
"""
from __future__ import annotations

import hashlib
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from orion_gb300 import scenegen  # noqa: E402

FLT_MAX = np.float32(3.4028234663852886e38)


def splitmix_uniform(n: int, seed: int) -> np.ndarray:
    """n doubles in [0, 1) from SplitMix64, vectorised over a counter."""
    m = np.uint64(0xFFFFFFFFFFFFFFFF)
    with np.errstate(over="ignore"):
        x = (np.arange(1, n + 1, dtype=np.uint64) * np.uint64(0x9E3779B97F4A7C15)
             + np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)) & m
        x = (x ^ (x >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        x = (x ^ (x >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        x = x ^ (x >> np.uint64(31))
    return (x >> np.uint64(11)).astype(np.float64) * (1.0 / (1 << 53))


def unit_vectors(n: int, seed: int) -> np.ndarray:
    u = splitmix_uniform(2 * n, seed).reshape(n, 2)
    z = 1.0 - 2.0 * u[:, 0]
    r = np.sqrt(np.maximum(0.0, 1.0 - z * z))
    phi = 2.0 * np.pi * u[:, 1]
    return np.stack([r * np.cos(phi), r * np.sin(phi), z], 1)


def random_rays(n: int, lo, hi, seed: int, pad: float = 0.1) -> np.ndarray:
    """n x 8 rays (o, d, tnear=0, tfar=FLT_MAX): origins in the padded box, uniform directions."""
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    ext = hi - lo
    u = splitmix_uniform(3 * n, seed).reshape(n, 3)
    o = lo - pad * ext + u * (1 + 2 * pad) * ext
    d = unit_vectors(n, seed + 1)
    r = np.zeros((n, 8), np.float32)
    r[:, 0:3], r[:, 3:6], r[:, 6], r[:, 7] = o, d, 0.0, FLT_MAX
    return r


def t_tolerance(rays, t_ref, prim_ref, positions):
    """Allowed |t - t_ref| of a hit: 1e-5 relative, or the float rounding of the ray-plane distance when
    that is larger. Both the GPU's Woop test (t = -(r2.(o - v0)) / (r2.d)) and the oracle's Moller-Trumbore
    test round the coordinates they combine, an error of a few units in the last place (2^-24 relative) of
    the largest coordinate involved (|o|, |v0|, t|d|); the plane distance divides it by the cosine
    between the ray and the triangle's normal, so grazing hits magnify it. 16 ulps of that scale over the
    cosine covers both tests' roundings."""
    o = rays[:, :3].astype(np.float64)
    d = rays[:, 3:6].astype(np.float64)
    tri = positions[np.maximum(prim_ref, 0)].reshape(-1, 3, 3).astype(np.float64)
    nrm = np.cross(tri[:, 1] - tri[:, 0], tri[:, 2] - tri[:, 0])
    nrm /= np.maximum(np.linalg.norm(nrm, axis=1, keepdims=True), 1e-300)
    cos = np.abs((d * nrm).sum(1)) / np.linalg.norm(d, axis=1)
    scale = np.maximum(np.abs(o).max(1), np.abs(tri).max((1, 2))) + np.abs(t_ref) * np.abs(d).max(1)
    return 1e-5 * np.abs(t_ref) + 16 * 2.0 ** -24 * scale / np.maximum(cos, 1e-6)


def random_frames(n: int, seed: int) -> np.ndarray:
    """n x 12 shading frames (ng, ns, u, v) built the way the reference builds them at a hit."""
    ng = unit_vectors(n, seed)
    ns = ng + 0.25 * unit_vectors(n, seed + 7)          # interpolated normals are not unit length
    e = unit_vectors(n, seed + 13)
    e = e - (e * ng).sum(1, keepdims=True) * ng
    su = e / np.linalg.norm(e, axis=1, keepdims=True)
    sv = np.cross(ns, su)
    sv /= np.linalg.norm(sv, axis=1, keepdims=True)
    su = np.cross(sv, ns)
    su /= np.linalg.norm(su, axis=1, keepdims=True)
    return np.concatenate([ng, ns, su, sv], 1).astype(np.float32)


def write_scene(name: str, directory: str, **kw) -> str:
    s = getattr(scenegen, name)(**kw)
    return scenegen.write_ori(s, directory)


# Full-size scenes of the parity fixtures: fixture -> (scenegen function, its arguments).
FULLSIZE = {"fullsize_cornell.npz": ("cornell", {}),
            "fullsize_displaced.npz": ("displaced", {}),
            "fullsize_mixed.npz": ("mixed", {"plastic_distribution": "ggx"}),
            "fullsize_mixed_beckmann.npz": ("mixed", {})}


def fullsize_scene(name: str, **kw) -> str:
    """The scene file of a workload at its full size (written once per machine into a cache directory,
    then reused): the 1024x1024 displaced sphere or the 1920x1080 eight-sphere scene."""
    import tempfile
    tag = "_".join(f"{k}{v}" for k, v in sorted(kw.items()))
    d = os.path.join(tempfile.gettempdir(), "orion_gb300_fullsize", name + ("_" + tag if tag else ""))
    marker = os.path.join(d, "done")
    if not os.path.exists(marker):
        path = write_scene(name, d, **kw)
        with open(marker, "w") as f:
            f.write(path)
    return open(marker).read().strip()


def scene_hash(ori_path: str) -> str:
    """SHA-256 over the scene file and the meshes and images it names."""
    d = os.path.dirname(ori_path)
    h = hashlib.sha256()
    h.update(open(ori_path, "rb").read())
    import re
    text = open(ori_path).read()
    for fn in re.findall(r'filename="([^"]+\.obj)"', text) + re.findall(r'name="([^"]+\.(?:png|bmp|tga|ppm))"', text):
        h.update(open(os.path.join(d, fn), "rb").read())
    return h.hexdigest()


def golden(name: str) -> dict:
    return dict(np.load(os.path.join(GOLDEN, name), allow_pickle=False))


# Material records used by the BSDF fixtures: (name, field values).
BSDF_CASES = [
    ("matte_lambert", dict(type=0, Kd=(0.5, 0.6, 0.7))),
    ("matte_orennayar", dict(type=0, Kd=(0.5, 0.6, 0.7), has_sigma=1, sigma=25.0)),
    ("metal_ggx", dict(type=1, eta_rgb=(0.2, 0.42, 1.37), k=(3.91, 2.45, 2.14), roughness=0.3)),
    ("mirror", dict(type=2, Kr=(0.9, 0.8, 0.7))),
    ("glass_smooth", dict(type=3, Kr=(1, 1, 1), Kt=(1, 1, 1), eta=1.5, roughness=0.0)),
    ("glass_rough", dict(type=3, Kr=(0.9, 0.9, 0.9), Kt=(0.8, 0.9, 1.0), eta=1.33, roughness=0.2)),
    ("plastic", dict(type=4, Kd=(0.3, 0.2, 0.1), Ks=(0.5, 0.5, 0.5), roughness=0.1)),
    ("uber", dict(type=5, Kd=(0.5, 0.3, 0.2), Ks=(0.3, 0.3, 0.3), Kr=(0.2, 0.2, 0.2), Kt=(0.1, 0.1, 0.1),
                  opacity=(0.8, 0.7, 0.9), roughness=0.2, eta=1.4)),
]


def make_material(fields: dict):
    from orion_gb300 import Material
    m = Material()
    for k, v in fields.items():
        if isinstance(v, tuple):
            getattr(m, k)[:] = list(v)
        else:
            setattr(m, k, v)
    return m


def bsdf_inputs(n: int, seed: int):
    frame = random_frames(n, seed)
    wo = unit_vectors(n, seed + 101).astype(np.float32)
    wi = unit_vectors(n, seed + 202).astype(np.float32)
    rnd = splitmix_uniform(2 * n, seed + 303).reshape(n, 2).astype(np.float32)
    return frame, wo, wi, rnd
