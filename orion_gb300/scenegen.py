"""Seeded synthetic scenes in orion's own input format (``.ori`` XML + OBJ).

The reference reads a scene through ``Parser`` (src/util/parser.cpp:45-56):
``<Camera>``, ``<Model type="mesh" filename=...>`` with an OBJ that must carry
``vn`` normals (src/core/triangle.cpp:40-42 indexes them unconditionally),
``<Material>``, ``<AreaLight>``, ``<Light type="point|spot">``, ``<Envmap>``,
``<Integrator type="path">`` and ``<Sampler type="sobol">``.  This module
builds the benchmark workloads as plain numpy geometry and writes them in
exactly that schema, so the same files drive the reference renderer, the CPU
oracle and the GPU path tracer.

Workloads (all seeds fixed and recorded in ``Scene.meta``):

* ``cornell``      -- 256x256, 16 spp, depth 5: five walls (10 tris), two
  subdivision-4 icospheres (Lambert 0.8 and smooth glass eta 1.5), a
  0.5x0.5 quad light at y=0.99 with Le (17,12,4), pinhole fov 40 at z=3.5.
* ``displaced``    -- 1024x1024, 64 spp, depth 8: subdivision-8 icosphere
  (1,310,720 tris, radius 1) displaced by 3-octave value noise (amplitude
  0.05, frequency 4) on a 20x20 ground quad; GGX conductor with eta
  (0.20,0.42,1.37), k (3.91,2.45,2.14), roughness U(0.05,0.5); spotlight
  (intensity 50, cone 30 deg, falloff 5 deg) plus a constant environment of
  radiance 0.1.
* ``mixed``        -- 1920x1080, 128 spp, depth 16: eight displaced icospheres
  (subdivision 5-7), five materials round robin, two quad lights and a point
  light, thin-lens camera.
* ``job(seed)``    -- the batched / served job distribution: 1-6 displaced
  spheres, log-uniform 1k-500k triangles, a ground quad, random materials,
  1-3 lights, resolution from {128,256,512,1024}^2, spp from {4,16,64},
  depth 4-12.

Every workload can be scaled down (``res_scale``/``spp``/``subdiv``) for the
parity tests without changing anything else about it.
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# --------------------------------------------------------------------------
# deterministic random numbers
#
# numpy's Generator streams are not guaranteed to match across numpy
# versions, and the scenes must be identical on every machine that renders
# or checks them, so all randomness here comes from SplitMix64 (Steele,
# Lea and Flood, "Fast splittable pseudorandom number generators", 2014).

_M64 = (1 << 64) - 1


class Rng:
    def __init__(self, seed: int):
        self.state = (seed * 0x9E3779B97F4A7C15 + 0x632BE59BD9B4E019) & _M64

    def next_u64(self) -> int:
        self.state = (self.state + 0x9E3779B97F4A7C15) & _M64
        z = self.state
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def random(self) -> float:  # [0, 1) with 53 bits
        return (self.next_u64() >> 11) * (1.0 / (1 << 53))

    def uniform(self, lo=0.0, hi=1.0, size=None):
        if size is None:
            return lo + (hi - lo) * self.random()
        n = int(np.prod(size))
        return np.array([lo + (hi - lo) * self.random() for _ in range(n)]).reshape(size)

    def integers(self, lo: int, hi: int) -> int:  # [lo, hi)
        return lo + self.next_u64() % (hi - lo)

    def choice(self, items):
        return items[self.integers(0, len(items))]

    def normal(self, size=3):
        out = []
        while len(out) < size:
            u1, u2 = self.random(), self.random()
            r = math.sqrt(-2.0 * math.log(1.0 - u1))
            out += [r * math.cos(2 * math.pi * u2), r * math.sin(2 * math.pi * u2)]
        return np.array(out[:size])

    def permutation(self, n: int) -> np.ndarray:
        a = list(range(n))
        for i in range(n - 1, 0, -1):
            j = self.integers(0, i + 1)
            a[i], a[j] = a[j], a[i]
        return np.array(a, dtype=np.int64)


# --------------------------------------------------------------------------
# geometry


def icosphere(subdiv: int):
    """Unit icosphere: (vertices Vx3 float64, faces Fx3 int64), 20*4^subdiv faces."""
    t = (1.0 + 5.0 ** 0.5) / 2.0
    v = np.array(
        [[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0],
         [0, -1, t], [0, 1, t], [0, -1, -t], [0, 1, -t],
         [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], dtype=np.float64)
    f = np.array(
        [[0, 11, 5], [0, 5, 1], [0, 1, 7], [0, 7, 10], [0, 10, 11],
         [1, 5, 9], [5, 11, 4], [11, 10, 2], [10, 7, 6], [7, 1, 8],
         [3, 9, 4], [3, 4, 2], [3, 2, 6], [3, 6, 8], [3, 8, 9],
         [4, 9, 5], [2, 4, 11], [6, 2, 10], [8, 6, 7], [9, 8, 1]], dtype=np.int64)
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    for _ in range(subdiv):
        nv = v.shape[0]
        edges = np.concatenate([f[:, [0, 1]], f[:, [1, 2]], f[:, [2, 0]]], axis=0)
        key = np.sort(edges, axis=1)
        uniq, inv = np.unique(key[:, 0] * (nv + 1) + key[:, 1], return_inverse=True)
        a = uniq // (nv + 1)
        b = uniq % (nv + 1)
        mid = v[a] + v[b]
        mid /= np.linalg.norm(mid, axis=1, keepdims=True)
        mid_idx = nv + inv.reshape(3, -1).T  # per face: (m01, m12, m20)
        v = np.concatenate([v, mid], axis=0)
        i0, i1, i2 = f[:, 0], f[:, 1], f[:, 2]
        m01, m12, m20 = mid_idx[:, 0], mid_idx[:, 1], mid_idx[:, 2]
        f = np.concatenate([
            np.stack([i0, m01, m20], 1), np.stack([i1, m12, m01], 1),
            np.stack([i2, m20, m12], 1), np.stack([m01, m12, m20], 1)], axis=0)
    return v, f


def value_noise(p: np.ndarray, seed: int) -> np.ndarray:
    """Seeded 3-D value noise in [-1, 1]: hashed lattice values, smoothstep-trilinear."""
    rng = Rng(seed)
    table = rng.uniform(-1.0, 1.0, size=(256,))
    perm = rng.permutation(256)
    perm = np.concatenate([perm, perm])

    def lattice(ix, iy, iz):
        return table[perm[(perm[(perm[ix & 255] + iy) & 255] + iz) & 255]]

    fl = np.floor(p)
    i = fl.astype(np.int64)
    fr = p - fl
    w = fr * fr * (3.0 - 2.0 * fr)
    out = np.zeros(p.shape[0])
    for dx in (0, 1):
        wx = w[:, 0] if dx else 1.0 - w[:, 0]
        for dy in (0, 1):
            wy = w[:, 1] if dy else 1.0 - w[:, 1]
            for dz in (0, 1):
                wz = w[:, 2] if dz else 1.0 - w[:, 2]
                out += wx * wy * wz * lattice(i[:, 0] + dx, i[:, 1] + dy, i[:, 2] + dz)
    return out


def displaced_sphere(subdiv: int, radius: float, amplitude: float, frequency: float, seed: int,
                     octaves: int = 3):
    """Icosphere displaced radially by `octaves` of value noise; smooth vertex normals."""
    v, f = icosphere(subdiv)
    n = np.zeros(v.shape[0])
    amp, freq = 1.0, frequency
    norm = 0.0
    for o in range(octaves):
        n += amp * value_noise(v * freq, seed * 7919 + o)
        norm += amp
        amp *= 0.5
        freq *= 2.0
    n /= norm
    pos = v * (radius * (1.0 + amplitude * n))[:, None] if amplitude else v * radius
    return pos, f, vertex_normals(pos, f)


def vertex_normals(pos: np.ndarray, f: np.ndarray) -> np.ndarray:
    fn = np.cross(pos[f[:, 1]] - pos[f[:, 0]], pos[f[:, 2]] - pos[f[:, 0]])
    vn = np.zeros_like(pos)
    for k in range(3):
        np.add.at(vn, f[:, k], fn)
    ln = np.linalg.norm(vn, axis=1, keepdims=True)
    ln[ln == 0] = 1.0
    return vn / ln


def quad(corners, normal):
    """Two triangles (CCW seen from `normal`) for 4 corners in order around the quad."""
    c = np.asarray(corners, dtype=np.float64)
    f = np.array([[0, 1, 2], [0, 2, 3]], dtype=np.int64)
    e = np.cross(c[1] - c[0], c[2] - c[0])
    if np.dot(e, normal) < 0:
        f = f[:, ::-1].copy()
    n = np.tile(np.asarray(normal, dtype=np.float64), (4, 1))
    return c, f, n


def rotation(axis, degrees):
    a = np.asarray(axis, dtype=np.float64)
    a = a / np.linalg.norm(a)
    th = math.radians(degrees)
    c, s = math.cos(th), math.sin(th)
    x, y, z = a
    return np.array([[c + x * x * (1 - c), x * y * (1 - c) - z * s, x * z * (1 - c) + y * s],
                     [y * x * (1 - c) + z * s, c + y * y * (1 - c), y * z * (1 - c) - x * s],
                     [z * x * (1 - c) - y * s, z * y * (1 - c) + x * s, c + z * z * (1 - c)]])


# --------------------------------------------------------------------------
# scene description


@dataclass
class Mesh:
    name: str
    pos: np.ndarray      # V x 3
    faces: np.ndarray    # F x 3
    normals: np.ndarray  # V x 3
    material: dict
    area_le: tuple | None = None  # emitted radiance if this mesh is an area light
    uvs: np.ndarray | None = None  # V x 2 texture coordinates (written as OBJ vt), or none (0, 0)

    @property
    def num_tris(self):
        return int(self.faces.shape[0])


@dataclass
class Scene:
    name: str
    width: int
    height: int
    spp: int
    max_depth: int
    eye: tuple
    look: tuple
    up: tuple
    fov: float
    meshes: list = field(default_factory=list)
    lights: list = field(default_factory=list)    # dicts: point / spot / distant
    envmaps: list = field(default_factory=list)   # dicts: constant radiance L, worldUp
    lens_radius: float = 0.0
    focal_distance: float = 0.0
    sppm: dict | None = None  # <Integrator type="sppm">: iterations, photons, radius, max_depth
    meta: dict = field(default_factory=dict)

    @property
    def num_tris(self):
        return sum(m.num_tris for m in self.meshes)

    def flat(self, text_rounding: bool = True):
        """De-indexed corner arrays in primitive order: (P Tx9, N Tx9, mesh index per tri).

        text_rounding: round to the 7 significant digits the OBJ writer emits (slow, exact
        agreement with a written-and-loaded scene); else plain float32 of the generated values."""
        rnd = _f32 if text_rounding else (lambda a: np.asarray(a, np.float32))
        ps, ns, ids = [], [], []
        for i, m in enumerate(self.meshes):
            p = rnd(m.pos)[m.faces].reshape(-1, 9)
            n = rnd(m.normals)[m.faces].reshape(-1, 9)
            ps.append(p)
            ns.append(n)
            ids.append(np.full(m.num_tris, i, dtype=np.int32))
        return np.concatenate(ps), np.concatenate(ns), np.concatenate(ids)

    def flat_uvs(self, text_rounding: bool = True) -> np.ndarray:
        """Texture coordinates per primitive corner (T x 6); (0, 0) where a mesh has none."""
        rnd = _f32 if text_rounding else (lambda a: np.asarray(a, np.float32))
        return np.concatenate([rnd(m.uvs)[m.faces].reshape(-1, 6) if m.uvs is not None
                               else np.zeros((m.num_tris, 6), np.float32) for m in self.meshes])


def _f32(a):
    """Round to 7 significant digits, the precision written to OBJ/XML, as float32."""
    return np.char.mod("%.7g", np.asarray(a, dtype=np.float64)).astype(np.float64).astype(np.float32)


def matte(kd, sigma=None):
    return {"type": "matte", "Kd": tuple(kd), **({"sigma": sigma} if sigma is not None else {})}


def metal(eta, k, roughness):
    return {"type": "metal", "eta": tuple(eta), "k": tuple(k), "roughness": roughness}


def glass(eta, roughness=0.0, kr=(1, 1, 1), kt=(1, 1, 1)):
    return {"type": "glass", "Kr": tuple(kr), "Kt": tuple(kt), "eta": eta, "roughness": roughness}


def mirror(kr=(1, 1, 1)):
    return {"type": "mirror", "Kr": tuple(kr)}


def plastic(kd, ks, roughness, distribution="ggx"):
    m = {"type": "plastic", "Kd": tuple(kd), "Ks": tuple(ks), "roughness": roughness}
    if distribution != "ggx":
        m["distribution"] = distribution
    return m


# --------------------------------------------------------------------------
# workloads


def cornell(res: int = 256, spp: int = 16, subdiv: int = 4, max_depth: int = 5) -> Scene:
    s = Scene("cornell", res, res, spp, max_depth, (0, 0, 3.5), (0, 0, 0), (0, 1, 0), 40.0,
              meta={"config": "cornell box", "seed": 0})
    white, red, green = matte((0.73, 0.73, 0.73)), matte((0.65, 0.05, 0.05)), matte((0.12, 0.45, 0.15))
    walls = [
        ("floor", [(-1, -1, -1), (1, -1, -1), (1, -1, 1), (-1, -1, 1)], (0, 1, 0), white),
        ("ceiling", [(-1, 1, -1), (1, 1, -1), (1, 1, 1), (-1, 1, 1)], (0, -1, 0), white),
        ("back", [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1)], (0, 0, 1), white),
        ("left", [(-1, -1, -1), (-1, 1, -1), (-1, 1, 1), (-1, -1, 1)], (1, 0, 0), red),
        ("right", [(1, -1, -1), (1, 1, -1), (1, 1, 1), (1, -1, 1)], (-1, 0, 0), green),
    ]
    for name, c, n, mat in walls:
        p, f, nn = quad(c, n)
        s.meshes.append(Mesh(name, p, f, nn, mat))
    for name, centre, mat in [("sphere_diffuse", (-0.4, -0.7, 0.2), matte((0.8, 0.8, 0.8))),
                              ("sphere_glass", (0.4, -0.7, -0.3), glass(1.5, 0.0))]:
        v, f = icosphere(subdiv)
        s.meshes.append(Mesh(name, v * 0.3 + np.asarray(centre), f, v.copy(), mat))
    p, f, nn = quad([(-0.25, 0.99, -0.25), (0.25, 0.99, -0.25), (0.25, 0.99, 0.25), (-0.25, 0.99, 0.25)],
                    (0, -1, 0))
    s.meshes.append(Mesh("light", p, f, nn, matte((0, 0, 0)), area_le=(17.0, 12.0, 4.0)))
    return s


def caustics(res: int = 64, iterations: int = 8, photons: int = 20000, radius: float = 0.05, max_depth: int = 5,
             subdiv: int = 3) -> Scene:
    """The Cornell box for SPPM: smooth and rough glass and a metal sphere under the area light, plus a
    point light, a spotlight, a distant light and a constant environment (every Light::sample_Le)."""
    s = cornell(res, 1, subdiv, max_depth)
    s.name = "caustics"
    s.meta = {"config": "sppm caustics box", "seed": 0}
    s.meshes = [m for m in s.meshes if not m.name.startswith("sphere")]
    for name, centre, mat in [("sphere_glass", (-0.35, -0.7, 0.1), glass(1.5, 0.0)),
                              ("sphere_rough", (0.4, -0.7, -0.3), glass(1.4, 0.3)),
                              ("sphere_metal", (0.05, -0.75, 0.55), metal((0.2, 0.42, 1.37), (3.9, 2.4, 2.1), 0.2))]:
        v, f = icosphere(subdiv)
        s.meshes.insert(len(s.meshes) - 1, Mesh(name, v * 0.25 + np.asarray(centre), f, v.copy(), mat))
    s.lights.append({"type": "point", "I": (0.6, 0.6, 0.5), "from": (0.0, 0.5, 0.5)})
    s.lights.append({"type": "spot", "intensity": (1.5, 1.5, 2.0), "angle": 25.0, "delta": 5.0,
                     "from": (-0.6, 0.8, 0.8), "to": (0.0, -1.0, 0.0)})
    s.lights.append({"type": "distant", "L": (0.3, 0.3, 0.3), "from": (0.0, -1.0, -1.0), "to": (0.0, 0.0, 0.0)})
    s.envmaps.append({"L": (0.05, 0.05, 0.06), "worldUp": (0, 1, 0)})
    s.sppm = {"iterations": iterations, "photons": photons, "radius": radius, "max_depth": max_depth}
    return s


def with_sppm(scene: Scene, iterations: int = 4, photons: int = 10000, radius: float = 0.08,
              max_depth: int = 5) -> Scene:
    """The scene rendered by <Integrator type="sppm"> instead of the path tracer."""
    scene.sppm = {"iterations": iterations, "photons": photons, "radius": radius, "max_depth": max_depth}
    scene.name = scene.name + "_sppm"
    return scene


def envlit_sppm(res: int = 32, iterations: int = 4, photons: int = 10000, radius: float = 0.08,
                subdiv: int = 2) -> Scene:
    """`envlit` (image environment map: photons emitted by its Distribution2D) under SPPM."""
    return with_sppm(envlit(res, 1, 5, subdiv), iterations, photons, radius)


def textured_sppm(res: int = 32, iterations: int = 4, photons: int = 10000, radius: float = 0.08,
                  subdiv: int = 2) -> Scene:
    """`textured` (image textures on every material input) under SPPM."""
    return with_sppm(textured(res, 1, 5, subdiv), iterations, photons, radius)


def displaced(res: int = 1024, spp: int = 64, subdiv: int = 8, max_depth: int = 8, seed: int = 1) -> Scene:
    rng = Rng(seed)
    roughness = float(rng.uniform(0.05, 0.5))
    s = Scene("displaced", res, res, spp, max_depth, (0.0, 1.2, 4.0), (0.0, -0.1, 0.0), (0, 1, 0), 40.0,
              meta={"config": "displaced sphere", "seed": seed, "roughness": roughness})
    pos, f, n = displaced_sphere(subdiv, 1.0, 0.05, 4.0, seed)
    s.meshes.append(Mesh("sphere", pos, f, n,
                         metal((0.20, 0.42, 1.37), (3.91, 2.45, 2.14), roughness)))
    p, f, nn = quad([(-10, -1.05, -10), (10, -1.05, -10), (10, -1.05, 10), (-10, -1.05, 10)], (0, 1, 0))
    s.meshes.append(Mesh("ground", p, f, nn, matte((0.5, 0.5, 0.5))))
    s.lights.append({"type": "spot", "intensity": (50.0, 50.0, 50.0), "angle": 30.0, "delta": 5.0,
                     "from": (2.0, 4.0, 2.0), "to": (0.0, 0.0, 0.0)})
    s.envmaps.append({"L": (0.1, 0.1, 0.1), "worldUp": (0, 1, 0)})
    return s


def mixed(width: int = 1920, height: int = 1080, spp: int = 128, max_depth: int = 16, seed: int = 3,
          subdivs=(5, 6, 7, 5, 6, 7, 6, 7), plastic_distribution: str = "beckmann") -> Scene:
    """plastic_distribution "ggx": the plastic coat with the reference's only microfacet distribution
    (the reference ignores distribution="beckmann" and renders GGX)."""
    rng = Rng(seed)
    s = Scene("mixed", width, height, spp, max_depth, (0.0, 2.0, 12.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0,
              lens_radius=0.025, focal_distance=5.0, meta={"config": "mixed materials", "seed": seed})
    mats = [matte((0.6, 0.55, 0.5)), metal((0.2, 0.92, 1.1), (3.9, 2.45, 2.14), 0.2), glass(1.5, 0.1),
            mirror(), plastic((0.4, 0.1, 0.1), (0.5, 0.5, 0.5), 0.15, distribution=plastic_distribution)]
    for i, sd in enumerate(subdivs):
        pos, f, n = displaced_sphere(sd, 1.0, 0.05, 4.0, seed * 100 + i)
        scale = rng.uniform(0.5, 1.5)
        rot = rotation(rng.normal(size=3), rng.uniform(0, 360))
        centre = rng.uniform(-5 + scale, 5 - scale, size=(3,))
        centre[1] = rng.uniform(-4 + scale, 2)
        pos = pos @ (rot.T * scale) + centre
        n = n @ rot.T
        s.meshes.append(Mesh(f"sphere{i}", pos, f, n, mats[i % len(mats)]))
    p, f, nn = quad([(-5, -5, -5), (5, -5, -5), (5, -5, 5), (-5, -5, 5)], (0, 1, 0))
    s.meshes.append(Mesh("ground", p, f, nn, matte((0.5, 0.5, 0.5))))
    for i, (c, le) in enumerate([((-2.0, 4.9, 0.0), (8.0, 8.0, 8.0)), ((2.5, 4.9, -2.0), (6.0, 5.0, 4.0))]):
        h = 0.75
        p, f, nn = quad([(c[0] - h, c[1], c[2] - h), (c[0] + h, c[1], c[2] - h), (c[0] + h, c[1], c[2] + h),
                         (c[0] - h, c[1], c[2] + h)], (0, -1, 0))
        s.meshes.append(Mesh(f"light{i}", p, f, nn, matte((0, 0, 0)), area_le=le))
    s.lights.append({"type": "point", "I": (20.0, 20.0, 20.0), "from": (0.0, 3.0, 4.0)})
    return s


def job(seed: int, tri_budget_scale: float = 1.0) -> Scene:
    """One render job of the batched / served distribution, fully determined by `seed`."""
    rng = Rng(10_000 + seed)
    res = int(rng.choice([128, 256, 512, 1024]))
    spp = int(rng.choice([4, 16, 64]))
    depth = int(rng.integers(4, 13))
    s = Scene(f"job{seed}", res, res, spp, depth, (0.0, 1.5, 7.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0,
              meta={"config": "job", "seed": seed})
    n_spheres = int(rng.integers(1, 7))
    total = math.exp(rng.uniform(math.log(1e3), math.log(5e5))) * tri_budget_scale
    choices = [matte((0.7, 0.6, 0.5)), metal((0.2, 0.42, 1.37), (3.91, 2.45, 2.14), 0.2), glass(1.5, 0.1),
               mirror(), plastic((0.3, 0.3, 0.6), (0.5, 0.5, 0.5), 0.2)]
    for i in range(n_spheres):
        per = max(20.0, total / n_spheres)
        sd = int(np.clip(round(math.log(per / 20.0, 4)), 0, 8))
        pos, f, n = displaced_sphere(sd, 1.0, 0.05, 4.0, seed * 131 + i)
        scale = rng.uniform(0.4, 1.0)
        centre = np.array([rng.uniform(-3, 3), -1.0 + scale * 1.05, rng.uniform(-3, 1)])
        s.meshes.append(Mesh(f"sphere{i}", pos * scale + centre, f, n, choices[int(rng.integers(0, 5))]))
    p, f, nn = quad([(-8, -1, -8), (8, -1, -8), (8, -1, 8), (-8, -1, 8)], (0, 1, 0))
    s.meshes.append(Mesh("ground", p, f, nn, matte((0.5, 0.5, 0.5))))
    n_lights = int(rng.integers(1, 4))
    for i in range(n_lights):
        kind = int(rng.integers(0, 3))
        if kind == 0:
            c = (rng.uniform(-3, 3), 4.0, rng.uniform(-3, 3))
            h = 0.6
            p, f, nn = quad([(c[0] - h, c[1], c[2] - h), (c[0] + h, c[1], c[2] - h), (c[0] + h, c[1], c[2] + h),
                             (c[0] - h, c[1], c[2] + h)], (0, -1, 0))
            s.meshes.append(Mesh(f"light{i}", p, f, nn, matte((0, 0, 0)), area_le=(10.0, 9.0, 8.0)))
        elif kind == 1:
            s.lights.append({"type": "point", "I": (15.0, 15.0, 15.0),
                             "from": (rng.uniform(-3, 3), 3.5, rng.uniform(-3, 3))})
        else:
            s.lights.append({"type": "spot", "intensity": (40.0, 40.0, 40.0), "angle": 35.0, "delta": 5.0,
                             "from": (rng.uniform(-3, 3), 5.0, rng.uniform(-1, 4)), "to": (0.0, 0.0, 0.0)})
    return s


# --------------------------------------------------------------------------
# writer


def _fmt(v):
    return ",".join("%.7g" % float(x) for x in np.ravel(v))


def _is_image(v) -> bool:
    return isinstance(v, np.ndarray) and v.ndim == 3


def _tex_color(tag, rgb, image_file=None):
    if _is_image(rgb):  # an image texture: written as PNG beside the scene
        return (f'      <{tag}>\n        <Param type="image"/>\n        <Param filename="{image_file(rgb)}"/>\n'
                f'      </{tag}>\n')
    return f'      <{tag}>\n        <Param type="constant"/>\n        <Param color="{_fmt(rgb)}"/>\n      </{tag}>\n'


def _tex_float(tag, v):
    return f'      <{tag}>\n        <Param type="float"/>\n        <Param value="{_fmt([v])}"/>\n      </{tag}>\n'


def material_xml(m: dict, name: str, image_file=None) -> str:
    """image_file(rgb8) -> file name: writes an image texture and names it."""
    t = m["type"]
    out = f'    <Material type="{t}" name="{name}">\n'
    if "distribution" in m:
        out += f'      <Param distribution="{m["distribution"]}"/>\n'

    def col(tag):
        return _tex_color(tag, m[tag], image_file)
    if t == "matte":
        out += col("Kd")
        if "sigma" in m:
            out += _tex_float("sigma", m["sigma"])
    elif t == "metal":
        out += col("eta") + col("k") + _tex_float("roughness", m["roughness"])
    elif t == "mirror":
        out += col("Kr")
    elif t == "glass":
        out += col("Kr") + col("Kt") + _tex_float("eta", m["eta"]) + _tex_float("roughness", m["roughness"])
    elif t == "plastic":
        out += col("Kd") + col("Ks") + _tex_float("roughness", m["roughness"])
    elif t == "uber":
        for k in ("Kd", "Ks", "Kr", "Kt", "opacity"):
            out += col(k)
        out += _tex_float("roughness", m["roughness"]) + _tex_float("eta", m["eta"])
    else:
        raise ValueError(t)
    return out + "    </Material>\n"


def write_obj(path: str, pos: np.ndarray, faces: np.ndarray, normals: np.ndarray, uvs=None) -> None:
    p = np.char.mod("%.7g", np.asarray(pos, dtype=np.float64))
    n = np.char.mod("%.7g", np.asarray(normals, dtype=np.float64))
    f = (np.asarray(faces) + 1).astype(str)
    with open(path, "w") as fh:
        fh.write("\n".join("v " + " ".join(r) for r in p))
        fh.write("\n")
        if uvs is not None:
            t = np.char.mod("%.7g", np.asarray(uvs, dtype=np.float64))
            fh.write("\n".join("vt " + " ".join(r) for r in t))
            fh.write("\n")
        fh.write("\n".join("vn " + " ".join(r) for r in n))
        fh.write("\n")
        if uvs is not None:
            fh.write("\n".join(f"f {a}/{a}/{a} {b}/{b}/{b} {c}/{c}/{c}" for a, b, c in f))
        else:
            fh.write("\n".join(f"f {a}//{a} {b}//{b} {c}//{c}" for a, b, c in f))
        fh.write("\n")


def write_ori(scene: Scene, directory: str, mesh_prefix: str | None = None) -> str:
    """Write `scene` as <directory>/<name>.ori plus one OBJ per mesh; returns the .ori path.

    Material names carry the scene name: the reference keeps named materials
    in a process-wide table (src/util/parser.cpp:268) whose first entry for a
    name wins, so names must not repeat across scenes parsed in one process.
    """
    os.makedirs(directory, exist_ok=True)
    prefix = mesh_prefix or scene.name
    out = ["<Scene>\n", '  <Resource filename="./"/>\n', '  <Camera type="pinhole">\n',
           "    <Transform>\n",
           f'      <Param lookat="{_fmt(scene.eye)}, {_fmt(scene.look)}, {_fmt(scene.up)}"/>\n',
           "    </Transform>\n", f'    <Param fov="{_fmt([scene.fov])}"/>\n',
           f'    <Param filmsize="{scene.width},{scene.height}"/>\n']
    if scene.lens_radius > 0:
        out.append(f'    <Param lensRadius="{_fmt([scene.lens_radius])}"/>\n')
        out.append(f'    <Param focalDistance="{_fmt([scene.focal_distance])}"/>\n')
    out.append("  </Camera>\n")
    written = {}

    def image_file(rgb8):  # each texture image once, as PNG beside the scene
        if id(rgb8) not in written:
            fn = f"{scene.name}_tex{len(written)}.png"
            write_png(os.path.join(directory, fn), rgb8)
            written[id(rgb8)] = fn
        return written[id(rgb8)]
    for i, m in enumerate(scene.meshes):
        fn = f"{prefix}_{m.name}.obj"
        write_obj(os.path.join(directory, fn), m.pos, m.faces, m.normals, m.uvs)
        out.append(f'  <Model type="mesh" filename="{fn}">\n')
        out.append(material_xml(m.material, f"{scene.name}_m{i}", image_file))
        if m.area_le is not None:
            out.append(f'    <AreaLight>\n      <Param Le="{_fmt(m.area_le)}"/>\n'
                       f'      <Param nLightSamples="1"/>\n    </AreaLight>\n')
        out.append("  </Model>\n")
    for l in scene.lights:
        if l["type"] == "point":
            out.append(f'  <Light type="point">\n    <Param I="{_fmt(l["I"])}"/>\n'
                       f'    <Param from="{_fmt(l["from"])}"/>\n  </Light>\n')
        elif l["type"] == "spot":
            out.append(f'  <Light type="spot">\n    <Param intensity="{_fmt(l["intensity"])}"/>\n'
                       f'    <Param angle="{_fmt([l["angle"]])}"/>\n    <Param delta="{_fmt([l["delta"]])}"/>\n'
                       f'    <Param from="{_fmt(l["from"])}"/>\n    <Param to="{_fmt(l["to"])}"/>\n  </Light>\n')
        elif l["type"] == "distant":
            out.append(f'  <Light type="distant">\n    <Param L="{_fmt(l["L"])}"/>\n'
                       f'    <Param from="{_fmt(l["from"])}"/>\n    <Param to="{_fmt(l["to"])}"/>\n  </Light>\n')
    for k, e in enumerate(scene.envmaps):
        name = ""
        if e.get("image") is not None:  # an image map: written as PNG beside the scene
            fn = f"{scene.name}_env{k}.png"
            write_png(os.path.join(directory, fn), e["image"])
            name = f'    <Param name="{fn}"/>\n'
        out.append(f'  <Envmap>\n    <Param L="{_fmt(e["L"])}"/>\n    <Param nLightSamples="1"/>\n{name}'
                   f'    <Param worldUp="{_fmt(e["worldUp"])}"/>\n  </Envmap>\n')
    if scene.sppm is not None:
        q = scene.sppm
        out.append(f'  <Integrator type="sppm">\n    <Param numIterations="{q["iterations"]}"/>\n'
                   f'    <Param maxDepth="{q["max_depth"]}"/>\n'
                   f'    <Param photonsPerIteration="{q["photons"]}"/>\n'
                   f'    <Param initRadius="{_fmt([q["radius"]])}"/>\n  </Integrator>\n')
    else:
        out.append(f'  <Integrator type="path">\n    <Param maxDepth="{scene.max_depth}"/>\n'
                   f'    <Param nSamplesPerPixel="{scene.spp}"/>\n  </Integrator>\n')
    out.append('  <Sampler type="sobol"/>\n</Scene>\n')
    path = os.path.join(directory, f"{scene.name}.ori")
    with open(path, "w") as fh:
        fh.write("".join(out))
    return path


def write_png(path: str, rgb8) -> None:
    """An 8-bit RGB image as a PNG file (filter 0 rows, one zlib stream)."""
    import struct
    import zlib
    img = np.ascontiguousarray(rgb8, np.uint8)
    h, w = img.shape[:2]
    raw = b"".join(b"\x00" + img[j].tobytes() for j in range(h))

    def chunk(kind: bytes, data: bytes) -> bytes:
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, 2, 0, 0, 0))
                + chunk(b"IDAT", zlib.compress(raw, 9)) + chunk(b"IEND", b""))


def sky_image(width: int = 64, height: int = 32, seed: int = 11) -> np.ndarray:
    """A procedural 8-bit sky: a vertical gradient, value noise and one bright sun disc."""
    rng = Rng(seed)
    v = (np.arange(height) + 0.5)[:, None] / height
    u = (np.arange(width) + 0.5)[None, :] / width
    base = np.stack([60 + 120 * (1 - v) + 0 * u, 90 + 110 * (1 - v) + 0 * u, 140 + 90 * (1 - v) + 0 * u], -1)
    noise = np.array([[rng.uniform(-18, 18) for _ in range(width)] for _ in range(height)])[..., None]
    su, sv = rng.uniform(0.2, 0.8), rng.uniform(0.2, 0.4)
    d2 = ((u - su) * 2.0) ** 2 + (v - sv) ** 2
    sun = np.where(d2 < 0.004, 255.0, 0.0)[..., None]
    return np.clip(np.maximum(base + noise, sun), 0, 255).astype(np.uint8)


def envlit(res: int = 64, spp: int = 16, max_depth: int = 6, subdiv: int = 3) -> Scene:
    """Spheres of several materials on a ground quad, lit only by an image environment map."""
    s = Scene("envlit", res, res, spp, max_depth, (0.0, 1.2, 5.0), (0.0, 0.3, 0.0), (0, 1, 0), 40.0,
              meta={"config": "envlit"})
    mats = [matte((0.7, 0.7, 0.7)), metal((0.2, 0.42, 1.37), (3.91, 2.45, 2.14), 0.3), glass(1.5, 0.0),
            plastic((0.2, 0.5, 0.3), (0.5, 0.5, 0.5), 0.15)]
    for i, m in enumerate(mats):
        v, f = icosphere(subdiv)
        x = -1.8 + 1.2 * i
        s.meshes.append(Mesh(f"ball{i}", v * 0.5 + np.array([x, -0.5, 0.0]), f, v.copy(), m))
    p, f, nn = quad([(-6, -1, -6), (6, -1, -6), (6, -1, 6), (-6, -1, 6)], (0, 1, 0))
    s.meshes.append(Mesh("ground", p, f, nn, matte((0.5, 0.45, 0.4))))
    s.envmaps.append({"L": (1.5, 1.5, 1.5), "worldUp": (0, 1, 0), "image": sky_image()})
    return s


def pattern_image(kind: str, width: int, height: int, seed: int) -> np.ndarray:
    """A procedural 8-bit RGB texture: "checker" (8 x 8 cells of two seeded colours), "stripes"
    (vertical bands of seeded colours) or "noise" (per-texel seeded values)."""
    rng = Rng(seed)
    if kind == "noise":
        return np.array([[[int(rng.integers(0, 256)) for _ in range(3)] for _ in range(width)]
                         for _ in range(height)], np.uint8)
    cols = np.array([[int(rng.integers(20, 256)) for _ in range(3)] for _ in range(8)], np.uint8)
    x = np.arange(width)[None, :]
    y = np.arange(height)[:, None]
    if kind == "checker":
        idx = ((x * 8 // width) + (y * 8 // height)) % 2 + 0 * y
    else:
        idx = (x * 8 // width) % len(cols) + 0 * y
    return cols[idx]


def sphere_uvs(v: np.ndarray) -> np.ndarray:
    """Longitude / latitude texture coordinates of unit-sphere vertices."""
    u = 0.5 + np.arctan2(v[:, 2], v[:, 0]) / (2 * np.pi)
    w = np.arccos(np.clip(v[:, 1], -1.0, 1.0)) / np.pi
    return np.stack([u, w], 1)


def textured(res: int = 64, spp: int = 16, max_depth: int = 6, subdiv: int = 3) -> Scene:
    """Image textures on every kind of material input: a checkered matte ground whose texture
    coordinates run past [0, 1) on both sides (wrap filter), and spheres with a textured plastic
    Kd, metal eta, rough-glass Kt, mirror Kr and uber Kd + opacity; area light and a constant
    environment."""
    s = Scene("textured", res, res, spp, max_depth, (0.0, 1.4, 5.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0,
              meta={"config": "image textures"})
    checker = pattern_image("checker", 32, 32, 3)
    stripes = pattern_image("stripes", 24, 12, 4)
    noise = pattern_image("noise", 16, 8, 5)
    p, f, nn = quad([(-6, -1, -6), (6, -1, -6), (6, -1, 6), (-6, -1, 6)], (0, 1, 0))
    # u in [-0.65, 0.85], v in [-0.35, 1.15]: negative coordinates wrap, but none reaches -1, where the
    # reference's wrap reads past the texel array (src/core/texture.cpp:16-24)
    s.meshes.append(Mesh("ground", p, f, nn, {"type": "matte", "Kd": checker},
                         uvs=np.stack([p[:, 0] / 8.0 + 0.1, p[:, 2] / 8.0 + 0.4], 1)))
    mats = [{"type": "plastic", "Kd": stripes, "Ks": (0.4, 0.4, 0.4), "roughness": 0.2},
            {"type": "metal", "eta": noise, "k": (3.9, 2.4, 2.1), "roughness": 0.25},
            {"type": "glass", "Kr": (1.0, 1.0, 1.0), "Kt": stripes, "eta": 1.5, "roughness": 0.2},
            {"type": "mirror", "Kr": checker},
            {"type": "uber", "Kd": noise, "Ks": (0.3, 0.3, 0.3), "Kr": (0.1, 0.1, 0.1), "Kt": (0.2, 0.2, 0.2),
             "opacity": checker, "roughness": 0.3, "eta": 1.4}]
    for i, m in enumerate(mats):
        v, fc = icosphere(subdiv)
        c = np.array([-2.0 + 1.0 * i, -0.55, -0.3 + 0.25 * (i % 2)])
        s.meshes.append(Mesh(f"ball{i}", v * 0.42 + c, fc, v.copy(), m, uvs=sphere_uvs(v)))
    p, f, nn = quad([(-0.6, 2.8, -0.6), (0.6, 2.8, -0.6), (0.6, 2.8, 0.6), (-0.6, 2.8, 0.6)], (0, -1, 0))
    s.meshes.append(Mesh("panel", p, f, nn, matte((0, 0, 0)), area_le=(8.0, 7.5, 7.0)))
    s.envmaps.append({"L": (0.2, 0.22, 0.25), "worldUp": (0, 1, 0)})
    return s


def zoo(res: int = 64, spp: int = 16, max_depth: int = 6, subdiv: int = 2, beckmann: bool = False) -> Scene:
    """Every material and light type of the path tracer in one small scene.

    Matte (Lambert and Oren-Nayar), GGX metal, mirror, smooth and rough glass,
    plastic and uber spheres in front of a plastic back wall, lit by an area
    quad, a point light, a spotlight, a distant light and a constant
    environment. `beckmann` switches the plastic wall to the Beckmann
    distribution (an extension the reference does not have).
    """
    s = Scene("zoo", res, res, spp, max_depth, (0.0, 1.0, 5.0), (0.0, 0.0, 0.0), (0, 1, 0), 45.0,
              meta={"config": "material zoo", "seed": 0})
    floor_m = matte((0.6, 0.6, 0.55), sigma=20.0)
    p, f, nn = quad([(-4, -1, -4), (4, -1, -4), (4, -1, 4), (-4, -1, 4)], (0, 1, 0))
    s.meshes.append(Mesh("floor", p, f, nn, floor_m))
    p, f, nn = quad([(-4, -1, -2), (4, -1, -2), (4, 3, -2), (-4, 3, -2)], (0, 0, 1))
    s.meshes.append(Mesh("wall", p, f, nn, plastic((0.2, 0.3, 0.5), (0.4, 0.4, 0.4), 0.3,
                                                   distribution="beckmann" if beckmann else "ggx")))
    uber = {"type": "uber", "Kd": (0.5, 0.3, 0.2), "Ks": (0.3, 0.3, 0.3), "Kr": (0.2, 0.2, 0.2),
            "Kt": (0.1, 0.1, 0.1), "opacity": (0.8, 0.8, 0.8), "roughness": 0.2, "eta": 1.4}
    mats = [matte((0.8, 0.2, 0.2)), metal((0.2, 0.92, 1.1), (3.9, 2.45, 2.14), 0.15), mirror((0.9, 0.9, 0.9)),
            glass(1.5, 0.0), glass(1.33, 0.25), plastic((0.1, 0.5, 0.1), (0.5, 0.5, 0.5), 0.05), uber]
    for i, m in enumerate(mats):
        v, fc = icosphere(subdiv)
        c = np.array([-2.4 + 0.8 * i, -0.6 + 0.25 * (i % 2), -0.5 + 0.3 * (i % 3)])
        s.meshes.append(Mesh(f"ball{i}", v * 0.38 + c, fc, v.copy(), m))
    p, f, nn = quad([(-0.5, 2.5, -0.5), (0.5, 2.5, -0.5), (0.5, 2.5, 0.5), (-0.5, 2.5, 0.5)], (0, -1, 0))
    s.meshes.append(Mesh("panel", p, f, nn, matte((0, 0, 0)), area_le=(6.0, 6.0, 5.0)))
    s.lights.append({"type": "point", "I": (3.0, 2.5, 2.0), "from": (2.0, 1.5, 2.0)})
    s.lights.append({"type": "spot", "intensity": (8.0, 8.0, 10.0), "angle": 25.0, "delta": 6.0,
                     "from": (-2.0, 3.0, 2.0), "to": (-1.0, -1.0, 0.0)})
    s.lights.append({"type": "distant", "L": (0.4, 0.35, 0.3), "from": (1.0, 3.0, 1.0), "to": (0.0, 0.0, 0.0)})
    s.envmaps.append({"L": (0.05, 0.06, 0.08), "worldUp": (0, 1, 0)})
    return s


# --------------------------------------------------------------------------
# in-memory host scenes (no OBJ text): for the batched and served workloads


TEX_INPUTS = ("Kd", "Ks", "Kr", "Kt", "opacity", "eta", "k")  # ORION_TEX_* order


def _material_record(m: dict, image_index=None):
    """image_index(rgb8) -> 1-based index of a texture image in the scene's image list."""
    from orion_gb300 import Material
    r = Material()
    kinds = {"matte": 0, "metal": 1, "mirror": 2, "glass": 3, "plastic": 4, "uber": 5}
    r.type = kinds[m["type"]]
    r.distribution = 1 if m.get("distribution") == "beckmann" else 0
    for slot, (src, dst) in enumerate([("Kd", "Kd"), ("Ks", "Ks"), ("Kr", "Kr"), ("Kt", "Kt"), ("opacity", "opacity"),
                                       ("eta", "eta_rgb" if m["type"] == "metal" else None), ("k", "k")]):
        if src in m and dst is not None:
            if _is_image(m[src]):
                r.tex[slot] = image_index(m[src])
            else:
                getattr(r, dst)[:] = [float(np.float32(x)) for x in m[src]]
    if m["type"] == "matte" and "sigma" in m:
        r.has_sigma, r.sigma = 1, m["sigma"]
    if "roughness" in m:
        r.roughness = m["roughness"]
    if m["type"] in ("glass", "uber"):
        r.eta = m["eta"]
    return r


def _basis_rows(d):
    """Rows (x, y, d) of the frame the reference builds for a spot light (coordinateSystem)."""
    d = np.asarray(d, np.float64) / np.linalg.norm(d)
    if abs(d[0]) > abs(d[1]):
        y = np.array([-d[2], 0.0, d[0]]) / np.hypot(d[0], d[2])
    else:
        y = np.array([0.0, d[2], -d[1]]) / np.hypot(d[1], d[2])
    return np.cross(y, d), y, d


def to_host_scene(scene: Scene, text_rounding: bool = False):
    """The scene as an orion_gb300.HostScene built from arrays.

    Materials and light order are identical to writing the scene out and loading it. Geometry
    is too with text_rounding (slow); without it, vertices are the generated values in float32
    (within 1e-7 relative of the written text). Light frames agree with the loader's to float
    rounding (computed here in float64)."""
    import orion_gb300 as og
    return og.HostScene.from_arrays(**scene_arrays(scene, text_rounding))


def scene_desc(scene: Scene, text_rounding: bool = False):
    """(orion_scene_desc, keep-alive) of the scene, built in Python without loading the library
    (the same arrays to_host_scene hands it)."""
    import orion_gb300 as og
    return og.desc_from_arrays(**scene_arrays(scene, text_rounding))


def scene_arrays(scene: Scene, text_rounding: bool = False) -> dict:
    """Keyword arguments of HostScene.from_arrays / desc_from_arrays for the scene."""
    import orion_gb300 as og
    P, N, mesh_of = scene.flat(text_rounding)
    images, image_ids = [], {}

    def image_index(rgb8):  # 8-bit texels as the loader converts them (byte * 1/255 in float)
        if id(rgb8) not in image_ids:
            images.append(np.asarray(rgb8, np.uint8).astype(np.float32) * np.float32(1.0 / 255.0))
            image_ids[id(rgb8)] = len(images)
        return image_ids[id(rgb8)]
    mats = [_material_record(m.material, image_index) for m in scene.meshes]
    uvs = scene.flat_uvs(text_rounding) if any(m.uvs is not None for m in scene.meshes) else None
    lights, light_of = [], np.full(len(P), -1, np.int32)
    for i, m in enumerate(scene.meshes):
        if m.area_le is None:
            continue
        for prim in np.flatnonzero(mesh_of == i):
            L = og.Light()
            L.type, L.prim = og.LIGHT_AREA, int(prim)
            L.L[:] = list(m.area_le)
            light_of[prim] = len(lights)
            lights.append(L)
    for l in scene.lights:
        L = og.Light()
        if l["type"] == "point":
            L.type = og.LIGHT_POINT
            L.L[:], L.p[:] = list(l["I"]), list(l["from"])
        elif l["type"] == "spot":
            L.type = og.LIGHT_SPOT
            L.L[:], L.p[:] = list(l["intensity"]), list(l["from"])
            x, y, d = _basis_rows(np.asarray(l["to"], np.float64) - np.asarray(l["from"], np.float64))
            w2l = np.zeros((3, 4))
            w2l[:, :3] = np.stack([x, y, d])
            w2l[:, 3] = -w2l[:, :3] @ np.asarray(l["from"], np.float64)
            l2w = np.zeros((3, 4))
            l2w[:, :3] = w2l[:, :3].T
            l2w[:, 3] = np.asarray(l["from"], np.float64)
            L.w2l[:] = [float(v) for v in w2l.astype(np.float32).ravel()]
            L.l2w[:] = [float(v) for v in l2w.astype(np.float32).ravel()]
            L.cos_total = float(np.float32(math.cos(math.radians(l["angle"]))))
            L.cos_falloff = float(np.float32(math.cos(math.radians(l["angle"] - l["delta"]))))
        elif l["type"] == "distant":
            L.type = og.LIGHT_DISTANT
            L.L[:] = list(l["L"])
            d = np.asarray(l["to"], np.float64) - np.asarray(l["from"], np.float64)
            L.dir[:] = list(d / np.linalg.norm(d))
        lights.append(L)
    for e in scene.envmaps:
        L = og.Light()
        L.type = og.LIGHT_ENV
        L.L[:] = list(e["L"])
        if e.get("image") is not None:  # 8-bit texels as the loader converts them (byte * 1/255 in float)
            images.append(np.asarray(e["image"], np.uint8).astype(np.float32) * np.float32(1.0 / 255.0))
            L.image = len(images)
        up = np.asarray(e["worldUp"], np.float64)
        up /= np.linalg.norm(up)
        z = np.array([0.0, 0.0, 1.0])
        R = np.eye(3)
        c = float(up @ z)
        if -0.99 < c < 0.99:
            R = rotation(np.cross(z, up), math.degrees(math.acos(c)))
        l2w = np.zeros((3, 4))
        l2w[:, :3] = R
        w2l = np.zeros((3, 4))
        w2l[:, :3] = R.T
        L.l2w[:] = [float(v) for v in l2w.astype(np.float32).ravel()]
        L.w2l[:] = [float(v) for v in w2l.astype(np.float32).ravel()]
        lights.append(L)
    cam = og.look_at_camera(scene.eye, scene.look, scene.up, scene.fov, scene.width, scene.height,
                            scene.lens_radius, scene.focal_distance)
    return dict(positions=P, normals=N, material_of_prim=mesh_of, materials=mats, lights=lights, camera=cam,
                spp=scene.spp, max_depth=scene.max_depth, light_of_prim=light_of, uvs=uvs, images=images,
                sppm=scene.sppm)


def job_views(s: Scene, views: int = 16):
    """`views` cameras orbiting a job's scene (serving: one resident scene, many views)."""
    import orion_gb300 as og
    out = []
    for v in range(views):
        ang = 2 * math.pi * v / views
        eye = (7.0 * math.sin(ang), 1.5 + 0.5 * math.sin(3 * ang), 7.0 * math.cos(ang))
        out.append(og.look_at_camera(eye, (0.0, 0.0, 0.0), (0, 1, 0), 45.0, s.width, s.height))
    return out
