"""Image files as the scene loader reads them: environment maps and textures.

The reference loads `<Envmap><Param name=.../>` through stb_image and accepts
3- or 4-channel images only (src/texture/imagetexture.cpp:20-36); texels are
the 8-bit values times 1/255. The loader here reads PNG (8-bit, every row
filter, RGB / RGBA / palette), uncompressed BMP (24/32-bit, either row order),
TGA (raw and run-length) and binary PPM; every format must give the same
texels for the same picture.
"""
from __future__ import annotations

import os
import re
import struct
import zlib

import numpy as np
import pytest

from orion_gb300 import scenegen


def _png(path, px, ctype, palette=None, filters=(0,)):
    h, w = px.shape[:2]
    ch = px.shape[2] if px.ndim == 3 else 1
    flat = px.reshape(h, w * ch).astype(np.int32)
    rows = []
    for y in range(h):
        ft = filters[y % len(filters)]
        cur = flat[y]
        up = flat[y - 1] if y else np.zeros_like(cur)
        a = np.concatenate([np.zeros(ch, np.int32), cur[:-ch]])
        c = np.concatenate([np.zeros(ch, np.int32), up[:-ch]])
        if ft == 0:
            pred = np.zeros_like(cur)
        elif ft == 1:
            pred = a
        elif ft == 2:
            pred = up
        elif ft == 3:
            pred = (a + up) >> 1
        else:  # Paeth
            p = a + up - c
            pa, pb, pc = np.abs(p - a), np.abs(p - up), np.abs(p - c)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, up, c))
        rows.append(bytes([ft]) + ((cur - pred) & 255).astype(np.uint8).tobytes())

    def chunk(kind, data):
        return struct.pack(">I", len(data)) + kind + data + struct.pack(">I", zlib.crc32(kind + data) & 0xFFFFFFFF)

    body = chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0))
    if palette is not None:
        body += chunk(b"PLTE", palette.astype(np.uint8).tobytes())
    raw = zlib.compress(b"".join(rows), 6)
    body += chunk(b"IDAT", raw[: len(raw) // 2]) + chunk(b"IDAT", raw[len(raw) // 2:])  # split stream
    with open(path, "wb") as f:
        f.write(b"\x89PNG\r\n\x1a\n" + body + chunk(b"IEND", b""))


def _bmp(path, rgb, bpp=24, top_down=False):
    h, w = rgb.shape[:2]
    bgr = rgb[..., ::-1]
    if bpp == 32:
        bgr = np.concatenate([bgr, np.full((h, w, 1), 255, np.uint8)], 2)
    stride = (w * bpp // 8 + 3) & ~3
    rows = [bgr[y].tobytes().ljust(stride, b"\0") for y in (range(h) if top_down else range(h - 1, -1, -1))]
    data = b"".join(rows)
    hdr = b"BM" + struct.pack("<IHHI", 54 + len(data), 0, 0, 54)
    dib = struct.pack("<IiiHHIIiiII", 40, w, -h if top_down else h, 1, bpp, 0, len(data), 2835, 2835, 0, 0)
    with open(path, "wb") as f:
        f.write(hdr + dib + data)


def _tga(path, rgb, rle=False, top_first=False):
    h, w = rgb.shape[:2]
    bgr = rgb[..., ::-1]
    order = range(h) if top_first else range(h - 1, -1, -1)
    px = [bytes(bgr[y, x]) for y in order for x in range(w)]
    if rle:  # alternate literal and repeat packets, each within the pixel stream
        out, i = [], 0
        while i < len(px):
            j = i
            while j + 1 < len(px) and px[j + 1] == px[i] and j - i < 127:
                j += 1
            if j > i:
                out.append(bytes([0x80 | (j - i)]) + px[i])
                i = j + 1
            else:
                n = min(128, len(px) - i)
                out.append(bytes([n - 1]) + b"".join(px[i:i + n]))
                i += n
        data = b"".join(out)
    else:
        data = b"".join(px)
    hdr = struct.pack("<BBBHHBHHHHBB", 3, 0, 10 if rle else 2, 0, 0, 0, 0, 0, w, h, 24, 0x20 if top_first else 0)
    with open(path, "wb") as f:
        f.write(hdr + b"abc" + data)


def _ppm(path, rgb):
    h, w = rgb.shape[:2]
    with open(path, "wb") as f:
        f.write(f"P6\n# sky\n{w} {h}\n255\n".encode() + rgb.tobytes())


@pytest.fixture(scope="module")
def scene_dir(tmp_path_factory):
    d = tmp_path_factory.mktemp("envimg")
    ori = scenegen.write_ori(scenegen.envlit(res=16, spp=1, subdiv=1), str(d))
    return d, open(ori).read()


def _load(scene_dir, fname):
    import orion_gb300 as og
    d, text = scene_dir
    path = d / f"scene_{fname}.ori"
    path.write_text(re.sub(r'name="[^"]+\.png"', f'name="{fname}"', text))
    return og.HostScene.load(str(path)).arrays()["images"]


def _expect(rgb):
    return rgb.astype(np.float32) * np.float32(1.0 / 255.0)


SKY = scenegen.sky_image(37, 19, seed=5)  # odd width: BMP rows are padded


@pytest.mark.parametrize("fname,writer", [
    ("f0.png", lambda p: _png(p, SKY, 2)),
    ("fall.png", lambda p: _png(p, SKY, 2, filters=(0, 1, 2, 3, 4))),
    ("rgba.png", lambda p: _png(p, np.concatenate([SKY, np.full(SKY.shape[:2] + (1,), 7, np.uint8)], 2), 6,
                                filters=(4, 3, 1))),
    ("b24.bmp", lambda p: _bmp(p, SKY)),
    ("b32.bmp", lambda p: _bmp(p, SKY, bpp=32, top_down=True)),
    ("raw.tga", lambda p: _tga(p, SKY)),
    ("rle.tga", lambda p: _tga(p, SKY, rle=True, top_first=True)),
    ("sky.ppm", lambda p: _ppm(p, SKY)),
])
def test_every_format_gives_the_same_texels(scene_dir, fname, writer):
    writer(str(scene_dir[0] / fname))
    images = _load(scene_dir, fname)
    assert len(images) == 1 and np.array_equal(images[0], _expect(SKY))


def test_palette_png_expands_to_rgb(scene_dir):
    pal = np.array([[10, 20, 30], [200, 100, 50], [0, 255, 128], [255, 255, 255]], np.uint8)
    idx = (np.arange(12 * 9).reshape(9, 12) * 7 % 4).astype(np.uint8)
    _png(str(scene_dir[0] / "pal.png"), idx, 3, palette=pal, filters=(1, 2))
    images = _load(scene_dir, "pal.png")
    assert np.array_equal(images[0], _expect(pal[idx]))


def test_rle_runs_and_literals_decode(scene_dir):
    img = np.zeros((6, 40, 3), np.uint8)
    img[:, :20] = (9, 8, 7)  # long runs
    img[:, 20:] = SKY[:6, :20]  # literals
    _tga(str(scene_dir[0] / "mixed.tga"), img, rle=True)
    assert np.array_equal(_load(scene_dir, "mixed.tga")[0], _expect(img))


def test_rejected_images_raise(scene_dir):
    import orion_gb300 as og
    d = scene_dir[0]
    grey = SKY[..., 0]
    _png(str(d / "grey.png"), grey, 0)  # one channel: the reference's 3-or-4-channel check rejects it
    with pytest.raises(og.OrionError, match="channel"):
        _load(scene_dir, "grey.png")
    _png(str(d / "good.png"), SKY, 2)
    data = open(d / "good.png", "rb").read()
    open(d / "cut.png", "wb").write(data[: len(data) // 2])
    with pytest.raises(og.OrionError):
        _load(scene_dir, "cut.png")
    with pytest.raises(og.OrionError):
        _load(scene_dir, "missing.png")
    open(d / "junk.tga", "wb").write(os.urandom(11))
    with pytest.raises(og.OrionError):
        _load(scene_dir, "junk.tga")


def test_image_textures_load_into_material_slots(tmp_path):
    """<Kd><Param type="image"/><Param filename=.../></Kd> (src/util/parser.cpp:433-461): the loaded scene
    equals the in-memory one, with each image loaded once and referenced from its material inputs."""
    import orion_gb300 as og
    sc = scenegen.textured(res=16, spp=1, subdiv=1)
    path = scenegen.write_ori(sc, str(tmp_path))
    host = og.HostScene.load(path)
    a = host.arrays()
    b = scenegen.to_host_scene(sc, text_rounding=True).arrays()
    assert len(a["images"]) == 3 and all(np.array_equal(x, y) for x, y in zip(a["images"], b["images"]))
    assert np.array_equal(a["uvs"], b["uvs"])
    tex = [list(m.tex) for m in a["materials"]]
    assert tex == [list(m.tex) for m in b["materials"]]
    slots = dict(zip(scenegen.TEX_INPUTS, range(7)))
    # ground Kd, plastic Kd, metal eta, glass Kt, mirror Kr, uber Kd + opacity; the light panel is constant
    expect = [{"Kd": 1}, {"Kd": 2}, {"eta": 3}, {"Kt": 2}, {"Kr": 1}, {"Kd": 3, "opacity": 1}, {}]
    for t, e in zip(tex, expect):
        want = [0] * 8
        for k, v in e.items():
            want[slots[k]] = v
        assert t == want


def test_texture_files_resolve_from_the_scene_directory(tmp_path, monkeypatch):
    import orion_gb300 as og
    sc = scenegen.textured(res=16, spp=1, subdiv=1)
    path = scenegen.write_ori(sc, str(tmp_path / "s"))
    monkeypatch.chdir(tmp_path)  # not the scene's directory
    assert len(og.HostScene.load(path).arrays()["images"]) == 3
    text = open(path).read()
    absolute = re.sub(r'filename="(textured_tex\d\.png)"', lambda m: f'filename="{tmp_path / "s" / m.group(1)}"', text)
    p2 = tmp_path / "s" / "abs.ori"
    p2.write_text(absolute)
    assert len(og.HostScene.load(str(p2)).arrays()["images"]) == 3
    missing = tmp_path / "s" / "missing.ori"
    missing.write_text(text.replace("textured_tex1.png", "nothing_here.png"))
    with pytest.raises(og.OrionError, match="nothing_here"):
        og.HostScene.load(str(missing))
