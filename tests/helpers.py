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
