"""CPU tests of the C ABI library: exports, scene loader, error handling.

No GPU is touched here: the library loads without a device, the loader is
host code, and context creation without a device must fail with a status
code, not crash.
"""
from __future__ import annotations

import ctypes as C
import hashlib
import os
import re
import shutil
import tempfile

import numpy as np
import pytest

import helpers

ROOT = helpers.ROOT


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "orion_gpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(orion_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_every_declared_symbol(built):
    import orion_gb300 as og
    lib = og.library()
    syms = declared_symbols()
    assert len(syms) >= 15
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, f"declared but not exported: {missing}"


def test_loader_matches_reference_geometry(built, tmp_path):
    import orion_gb300 as og
    g = helpers.golden("geometry.npz")
    path = helpers.write_scene("cornell", str(tmp_path / "cornell256"))
    assert helpers.scene_hash(path) == bytes(helpers.golden("trace.npz")["hash"]).decode()
    a = og.HostScene.load(path).arrays()
    assert hashlib.sha256(a["positions"].tobytes()).hexdigest() == bytes(g["cornell/positions_sha"]).decode()
    assert hashlib.sha256(a["normals"].tobytes()).hexdigest() == bytes(g["cornell/normals_sha"]).decode()
    assert np.array_equal(a["light_of_prim"], g["cornell/light_of_prim"])
    assert len(a["lights"]) == len(g["cornell/light_power"])
    assert a["spp"] == 16 and a["max_depth"] == 5
    assert (a["camera"].width, a["camera"].height) == (256, 256)


def test_loader_zoo_lights_and_order(built, tmp_path):
    import orion_gb300 as og
    g = helpers.golden("geometry.npz")
    path = helpers.write_scene("zoo", str(tmp_path / "zoo"), res=48, spp=16)
    a = og.HostScene.load(path).arrays()
    assert hashlib.sha256(a["positions"].tobytes()).hexdigest() == bytes(g["zoo/positions_sha"]).decode()
    kinds = [l.type for l in a["lights"]]
    # area lights first (one per emissive triangle), then point, spot, distant, then the environment
    assert kinds == [og.LIGHT_AREA, og.LIGHT_AREA, og.LIGHT_POINT, og.LIGHT_SPOT, og.LIGHT_DISTANT, og.LIGHT_ENV]
    assert len(a["lights"]) == len(g["zoo/light_power"])


def test_context_without_device_reports_error(built):
    import orion_gb300 as og
    if shutil.which("nvidia-smi") and os.system("nvidia-smi -L > /dev/null 2>&1") == 0:
        pytest.skip("a GPU is present")
    with pytest.raises(og.OrionError) as e:
        og.Context(0)
    assert e.value.code in (-4, -1)


def _write(d, name, text):
    p = os.path.join(d, name)
    with open(p, "w") as f:
        f.write(text)
    return p


GOOD = """<Scene>
  <Resource filename="./"/>
  <Camera type="pinhole"><Transform><Param lookat="0,0,3, 0,0,0, 0,1,0"/></Transform>
    <Param fov="40"/><Param filmsize="8,8"/></Camera>
  <Model type="meshHandy">
    <Param p="-1,-1,0, 1,-1,0, 1,1,0"/><Param n="0,0,1"/>
    <Material type="matte"><Kd><Param type="constant"/><Param color="0.5,0.5,0.5"/></Kd></Material>
    <AreaLight><Param Le="1,1,1"/><Param nLightSamples="1"/></AreaLight>
  </Model>
  <Integrator type="path"><Param maxDepth="3"/><Param nSamplesPerPixel="2"/></Integrator>
  <Sampler type="sobol"/>
</Scene>
"""


@pytest.mark.parametrize("mutate,code", [
    (lambda s: s.replace("</Scene>", ""), -3),                                  # truncated XML
    (lambda s: s.replace('type="meshHandy"', 'type="mesh" filename="missing.obj"'), -2),
    (lambda s: s.replace('<Param n="0,0,1"/>', ""), -3),                        # normals are required
    (lambda s: s.replace('type="sobol"', 'type="pseudo"'), -6),
    (lambda s: s.replace('type="path"', 'type="sppm"'), -3),                    # sppm needs its parameters
    (lambda s: s.replace('type="path"', 'type="bdpt"'), -6),
    (lambda s: s.replace('<Kd><Param type="constant"/><Param color="0.5,0.5,0.5"/></Kd>', ""), -3),
    (lambda s: s.replace('<Param fov="40"/>', ""), -3),
])
def test_loader_rejects_bad_scenes(built, mutate, code):
    import orion_gb300 as og
    with tempfile.TemporaryDirectory() as d:
        og.HostScene.load(_write(d, "ok.ori", GOOD))
        with pytest.raises(og.OrionError) as e:
            og.HostScene.load(_write(d, "bad.ori", mutate(GOOD)))
        assert e.value.code == code, str(e.value)


def test_obj_without_normals_rejected(built, tmp_path):
    import orion_gb300 as og
    (tmp_path / "m.obj").write_text("v 0 0 0\nv 1 0 0\nv 0 1 0\nf 1 2 3\n")
    text = GOOD.replace('type="meshHandy"', 'type="mesh" filename="m.obj"')
    p = tmp_path / "s.ori"
    p.write_text(text)
    with pytest.raises(og.OrionError) as e:
        og.HostScene.load(str(p))
    assert e.value.code == -3 and "normal" in str(e.value)


def test_obj_quads_are_fan_triangulated(built, tmp_path):
    import orion_gb300 as og
    (tmp_path / "q.obj").write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1 4//1\n")
    p = tmp_path / "s.ori"
    p.write_text(GOOD.replace('type="meshHandy"', 'type="mesh" filename="q.obj"'))
    a = og.HostScene.load(str(p)).arrays()
    assert a["positions"].shape == (2, 9)
    assert np.allclose(a["positions"][1], [0, 0, 0, 1, 1, 0, 0, 1, 0])


def test_scene_from_desc_validates(built):
    import orion_gb300 as og
    m = helpers.make_material(dict(type=0, Kd=(0.5, 0.5, 0.5)))
    cam = og.Camera(width=4, height=4, fov=40.0)
    pos = np.zeros((1, 9), np.float32)
    with pytest.raises(og.OrionError):
        og.HostScene.from_arrays(pos, pos, [3], [m], [], cam, 1, 2)        # material index out of range
    s = og.HostScene.from_arrays(pos, pos, [0], [m], [], cam, 1, 2)
    assert s.desc().num_prims == 1


def _reference_obj(text):
    """Straight sequential reading of an OBJ (the rules of the loader): fan triangulation,
    1-based or relative indices, corners (p, n, uv)."""
    v, vn, vt, tris = [], [], [], []
    for line in text.splitlines():
        f = line.split()
        if not f:
            continue
        if f[0] == "v":
            v.append([np.float32(x) for x in f[1:4]])
        elif f[0] == "vn":
            vn.append([np.float32(x) for x in f[1:4]])
        elif f[0] == "vt":
            vt.append([np.float32(x) for x in f[1:3]])
        elif f[0] == "f":
            cs = []
            for c in f[1:]:
                a = (c.split("/") + ["", ""])[:3]
                res = lambda s, n: (int(s) - 1 if int(s) > 0 else n + int(s)) if s else -1
                cs.append((res(a[0], len(v)), res(a[1], len(vt)), res(a[2], len(vn))))
            for k in range(1, len(cs) - 1):
                tris.append([cs[0], cs[k], cs[k + 1]])
    P = np.array([[v[c[0]] for c in t] for t in tris], np.float32).reshape(-1, 9)
    N = np.array([[vn[c[2]] for c in t] for t in tris], np.float32).reshape(-1, 9)
    return P, N


def test_large_obj_parsed_in_pieces_equals_sequential_reading(built, tmp_path):
    """A multi-megabyte OBJ (read in parallel pieces) with relative indices and polygons."""
    import orion_gb300 as og
    rng = np.random.default_rng(3)
    lines, nv = [], 0
    for blk in range(1500):  # blocks of 40 vertices, faces referring back with negative indices
        pts = rng.uniform(-1, 1, size=(40, 3))
        lines += ["v %.6f %.6f %.6f" % tuple(p) for p in pts]
        lines += ["vn %.6f %.6f %.6f" % tuple(p) for p in pts]
        nv += 40
        for k in range(30):
            a, b, c, d = rng.choice(40, 4, replace=False)
            if k % 3 == 0:  # absolute quad
                base = nv - 40 + 1
                lines.append("f %d//%d %d//%d %d//%d %d//%d" % (base + a, base + a, base + b, base + b, base + c,
                                                              base + c, base + d, base + d))
            else:  # relative triangle
                lines.append("f %d//%d %d//%d %d//%d" % (a - 40, a - 40, b - 40, b - 40, c - 40, c - 40))
    text = "\n".join(lines) + "\n"
    assert len(text) > (1 << 21)
    (tmp_path / "big.obj").write_text(text)
    p = tmp_path / "s.ori"
    p.write_text(GOOD.replace('type="meshHandy"', 'type="mesh" filename="big.obj"'))
    a = og.HostScene.load(str(p)).arrays()
    P, N = _reference_obj(text)
    assert a["positions"].shape == P.shape
    assert np.array_equal(a["positions"], P) and np.array_equal(a["normals"], N)


def test_sppm_integrator_parameters_load_and_round_trip(tmp_path):
    """<Integrator type="sppm"> (src/util/parser.cpp:132-133, src/integrator/sppm.cpp:324-333)."""
    import orion_gb300 as og
    from orion_gb300 import scenegen
    sc = scenegen.caustics(res=16, iterations=3, photons=-1, radius=0.125, max_depth=4, subdiv=1)
    host = og.HostScene.load(scenegen.write_ori(sc, str(tmp_path)))
    d = host.desc()
    assert d.integrator == og.INTEGRATOR_SPPM
    assert (d.sppm.iterations, d.sppm.photons_per_iter, d.sppm.initial_radius, d.sppm.max_depth) == (3, -1, 0.125, 4)
    mem = scenegen.to_host_scene(sc).desc()
    assert mem.integrator == og.INTEGRATOR_SPPM and mem.sppm.photons_per_iter == -1
    bad = tmp_path / "bad.ori"
    bad.write_text(open(scenegen.write_ori(sc, str(tmp_path))).read().replace('<Param initRadius="0.125"/>', ""))
    with pytest.raises(og.OrionError, match="initRadius"):
        og.HostScene.load(str(bad))


def test_sobol_table_is_the_references():
    """data/sobol_matrices.bin holds the direction numbers of src/sampler/sobol.cpp (where the reference tree
    is present; elsewhere the committed table is what the GPU and the oracle load)."""
    from oracle import build as oracle_build
    from orion_gb300 import gen_sobol
    ref = oracle_build.reference_root()
    if ref is None:
        pytest.skip("reference tree not present")
    import struct
    vals = gen_sobol.extract(os.path.join(ref, "src", "sampler", "sobol.cpp"))
    assert open(gen_sobol.OUT, "rb").read() == struct.pack("<%dI" % len(vals), *vals)


def test_reference_side_adapter_builds_links_and_runs(built, tmp_path):
    """The GpuPathTracing integrator of INTEGRATION.md compiles against the reference's headers and links with
    the reference's objects and liborion_gb300.so (oracle/_ref/gpupath_demo, the reference's main() with that
    integrator). Run on the Cornell box: without a CUDA device it stops at orion_gpu_create with the library's
    message (exit status 3); with one it writes the averaged film as a BMP."""
    import subprocess
    from oracle import build as oracle_build
    if oracle_build.reference_root() is None:
        pytest.skip("reference tree not present")
    demo = os.path.join(helpers.ROOT, "oracle", "_ref", "gpupath_demo")
    assert os.path.exists(demo), "gpupath_demo was not built"
    libs = subprocess.run(["ldd", demo], capture_output=True, text=True).stdout
    assert "liborion_gb300.so" in libs and "liborion_ref.so" in libs
    path = helpers.write_scene("cornell", str(tmp_path / "c"), res=32, spp=2)
    out = str(tmp_path / "out.bmp")
    r = subprocess.run([demo, path, "5", "2", out], capture_output=True, text=True, cwd=os.path.dirname(path),
                       timeout=300)
    if r.returncode == 3:
        assert "orion_gpu_create" in r.stdout + r.stderr
    else:
        assert r.returncode == 0, r.stdout + r.stderr
        assert os.path.getsize(out) == 54 + 32 * 32 * 4
