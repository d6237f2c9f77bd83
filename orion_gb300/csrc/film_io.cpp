// Film output: the averaged film as a 32-bit BMP (saveAsBmp,
// src/core/texture.cpp:77-136).
//
// Same pixels as the reference: rows bottom-up, bytes B, G, R, 255, each
// channel clamp(c, 0, 1) * 255 truncated; no tone mapping or gamma. The
// headers are the 14 + 40-byte Windows layout the reference's structs have
// where `long` is 32 bits (its target platform); they are written field by
// field in little-endian order, so the file is the same on any host.
#include <stdint.h>

#include <cstdio>
#include <string>
#include <vector>

#include "../../include/orion_gpu.h"
#include "internal.h"

namespace {

void put16(std::vector<uint8_t>& b, uint32_t v) {
  b.push_back((uint8_t)(v & 0xff));
  b.push_back((uint8_t)((v >> 8) & 0xff));
}

void put32(std::vector<uint8_t>& b, uint32_t v) {
  put16(b, v & 0xffff);
  put16(b, v >> 16);
}

uint8_t to_byte(float f) {
  // clamp (src/core/geometry.h) then (char)(f * 255): truncation.
  if (!(f > 0.f)) f = 0.f;  // NaN clamps to 0 as well
  if (f > 1.f) f = 1.f;
  return (uint8_t)(int)(f * 255.f);
}

}  // namespace

extern "C" int orion_film_write_bmp(const char* path, int32_t width, int32_t height, const float* rgb) {
  if (!path || !rgb || width <= 0 || height <= 0)
    return orion_gb300::ctx_fail(ORION_ERR_INVALID, "orion_film_write_bmp: bad argument");
  if ((int64_t)width * height > (1LL << 28))
    return orion_gb300::ctx_fail(ORION_ERR_INVALID, "orion_film_write_bmp: image too large for a BMP");
  const uint32_t bytes = (uint32_t)width * (uint32_t)height * 4u;
  std::vector<uint8_t> out;
  out.reserve(54 + (size_t)bytes);
  out.push_back('B');
  out.push_back('M');
  put32(out, 54u + bytes);  // bfSize
  put16(out, 0);            // bfReserved1
  put16(out, 0);            // bfReserved2
  put32(out, 54u);          // bfOffBits
  put32(out, 40u);          // biSize
  put32(out, (uint32_t)width);
  put32(out, (uint32_t)height);
  put16(out, 1);            // biPlanes
  put16(out, 32);           // biBitCount
  for (int k = 0; k < 6; ++k) put32(out, 0);  // compression, image size, resolution, palette
  const size_t base = out.size();
  out.resize(base + bytes);
  for (int j = 0; j < height; ++j) {
    uint8_t* row = out.data() + base + (size_t)(height - j - 1) * width * 4;
    const float* src = rgb + (size_t)j * width * 3;
    for (int i = 0; i < width; ++i) {
      row[4 * i + 0] = to_byte(src[3 * i + 2]);
      row[4 * i + 1] = to_byte(src[3 * i + 1]);
      row[4 * i + 2] = to_byte(src[3 * i + 0]);
      row[4 * i + 3] = 255;
    }
  }
  FILE* f = std::fopen(path, "wb");
  if (!f) return orion_gb300::ctx_fail(ORION_ERR_IO, (std::string("cannot open ") + path).c_str());
  const size_t wrote = std::fwrite(out.data(), 1, out.size(), f);
  const bool ok = std::fclose(f) == 0 && wrote == out.size();
  if (!ok) return orion_gb300::ctx_fail(ORION_ERR_IO, (std::string("cannot write ") + path).c_str());
  return ORION_OK;
}
