"""saveAsBmp (src/core/texture.cpp:77-136): the BMP the film writer produces.

Known-answer test restating the reference's writer: 54-byte Windows header,
32 bits per pixel, rows bottom-up, bytes B, G, R, 255, channel value
clamp(c, 0, 1) * 255 truncated.
"""
import struct

import numpy as np
import pytest


def _expected_byte(c):
    c = np.where(np.isnan(c), 0.0, c)
    return (np.clip(c, 0.0, 1.0).astype(np.float32) * np.float32(255.0)).astype(np.int32).astype(np.uint8)


def test_bmp_matches_reference_layout(built, tmp_path):
    import orion_gb300 as og
    rng = np.random.default_rng(5)
    h, w = 7, 5
    img = rng.uniform(-0.2, 1.3, size=(h, w, 3)).astype(np.float32)
    img[0, 0] = [0.5, 1.0, 0.0]
    img[1, 1, 0] = np.nan
    path = str(tmp_path / "film.bmp")
    og.saveAsBmp(img, path)
    data = open(path, "rb").read()
    assert data[:2] == b"BM"
    size, r1, r2, off = struct.unpack("<IHHI", data[2:14])
    bi = struct.unpack("<IiiHHIIiiII", data[14:54])
    assert (size, r1, r2, off) == (54 + w * h * 4, 0, 0, 54) and len(data) == size
    assert bi[:5] == (40, w, h, 1, 32) and bi[5] == 0
    px = np.frombuffer(data[54:], np.uint8).reshape(h, w, 4)[::-1]  # back to top-down rows
    want = _expected_byte(img)
    assert np.array_equal(px[..., 0], want[..., 2])
    assert np.array_equal(px[..., 1], want[..., 1])
    assert np.array_equal(px[..., 2], want[..., 0])
    assert (px[..., 3] == 255).all()
    assert tuple(px[0, 0, :3]) == (0, 255, 127)


def test_bmp_rejects_bad_arguments(built, tmp_path):
    import orion_gb300 as og
    with pytest.raises(ValueError):
        og.saveAsBmp(np.zeros((4, 4)), str(tmp_path / "x.bmp"))
    with pytest.raises(og.OrionError):
        og.saveAsBmp(np.zeros((2, 2, 3)), str(tmp_path / "no" / "such" / "dir.bmp"))
