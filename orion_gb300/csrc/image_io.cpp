// 8-bit RGB image files for environment maps and image textures.
//
// The reference reads images with stb_image's 8-bit interface and keeps 3- or
// 4-channel images only, dropping alpha (src/texture/imagetexture.cpp:20-52).
// This reader decodes the lossless formats whose bytes such a decoder returns
// exactly: PNG (8-bit greyscale / RGB / RGBA / palette, non-interlaced; the
// zlib stream is inflated by the system's libz, loaded at run time), BMP
// (uncompressed 24 / 32 bit), TGA (true colour, raw or run-length, 24 / 32
// bit) and binary PPM (P6, maxval 255). Rows are returned top first.
#include "image_io.h"

#include <dlfcn.h>

#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace orion_gb300 {

namespace {

bool read_all(const std::string& path, std::vector<uint8_t>* out) {
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return false;
  std::fseek(f, 0, SEEK_END);
  const long n = std::ftell(f);
  std::fseek(f, 0, SEEK_SET);
  out->resize(n > 0 ? (size_t)n : 0);
  const bool ok = n >= 0 && std::fread(out->data(), 1, out->size(), f) == out->size();
  std::fclose(f);
  return ok;
}

uint32_t be32(const uint8_t* p) { return (uint32_t)p[0] << 24 | (uint32_t)p[1] << 16 | (uint32_t)p[2] << 8 | p[3]; }
uint32_t le32(const uint8_t* p) { return (uint32_t)p[3] << 24 | (uint32_t)p[2] << 16 | (uint32_t)p[1] << 8 | p[0]; }
uint32_t le16(const uint8_t* p) { return (uint32_t)p[1] << 8 | p[0]; }

// zlib's uncompress(), from the shared library (its C signature is part of
// zlib's stable interface).
typedef int (*uncompress_fn)(unsigned char*, unsigned long*, const unsigned char*, unsigned long);

uncompress_fn zlib_uncompress() {
  static uncompress_fn fn = [] {
    for (const char* name : {"libz.so.1", "libz.so"}) {
      if (void* h = dlopen(name, RTLD_NOW | RTLD_LOCAL))
        if (void* s = dlsym(h, "uncompress")) return reinterpret_cast<uncompress_fn>(s);
    }
    return (uncompress_fn) nullptr;
  }();
  return fn;
}

int paeth(int a, int b, int c) {
  const int p = a + b - c, pa = p > a ? p - a : a - p, pb = p > b ? p - b : b - p, pc = p > c ? p - c : c - p;
  if (pa <= pb && pa <= pc) return a;
  return pb <= pc ? b : c;
}

bool decode_png(const std::vector<uint8_t>& f, Image8* img, std::string* err) {
  static const uint8_t sig[8] = {137, 80, 78, 71, 13, 10, 26, 10};
  if (f.size() < 8 || std::memcmp(f.data(), sig, 8) != 0) return *err = "not a PNG file", false;
  uint32_t w = 0, h = 0;
  int depth = 0, ctype = -1, interlace = 0;
  std::vector<uint8_t> idat, palette;
  size_t pos = 8;
  bool end = false;
  while (!end && pos + 12 <= f.size()) {
    const uint32_t len = be32(&f[pos]);
    if (pos + 12 + (size_t)len > f.size()) return *err = "truncated PNG chunk", false;
    const uint8_t* type = &f[pos + 4];
    const uint8_t* data = &f[pos + 8];
    if (!std::memcmp(type, "IHDR", 4)) {
      if (len < 13) return *err = "bad PNG header", false;
      w = be32(data);
      h = be32(data + 4);
      depth = data[8];
      ctype = data[9];
      interlace = data[12];
    } else if (!std::memcmp(type, "PLTE", 4)) {
      palette.assign(data, data + len);
    } else if (!std::memcmp(type, "IDAT", 4)) {
      idat.insert(idat.end(), data, data + len);
    } else if (!std::memcmp(type, "IEND", 4)) {
      end = true;
    }
    pos += 12 + (size_t)len;
  }
  if (w == 0 || h == 0 || w > (1u << 15) || h > (1u << 15)) return *err = "PNG size out of range", false;
  if (depth != 8) return *err = "PNG bit depth other than 8 is not supported", false;
  if (interlace != 0) return *err = "interlaced PNG is not supported", false;
  int channels;
  switch (ctype) {
    case 0: channels = 1; break;  // greyscale
    case 2: channels = 3; break;  // RGB
    case 3: channels = 1; break;  // palette index
    case 4: channels = 2; break;  // greyscale + alpha
    case 6: channels = 4; break;  // RGBA
    default: return *err = "unknown PNG colour type", false;
  }
  if (ctype == 3 && palette.size() < 3) return *err = "PNG palette missing", false;
  uncompress_fn inflate = zlib_uncompress();
  if (!inflate) return *err = "PNG needs the system zlib (libz.so.1), which could not be loaded", false;
  const size_t stride = (size_t)w * channels;
  std::vector<uint8_t> raw((stride + 1) * h);
  unsigned long raw_len = (unsigned long)raw.size();
  if (inflate(raw.data(), &raw_len, idat.data(), (unsigned long)idat.size()) != 0 || raw_len != raw.size())
    return *err = "corrupt PNG image data", false;
  // Undo the per-row filters (PNG specification, section 9).
  std::vector<uint8_t> px(stride * h);
  for (uint32_t y = 0; y < h; ++y) {
    const uint8_t ft = raw[y * (stride + 1)];
    const uint8_t* in = &raw[y * (stride + 1) + 1];
    uint8_t* out = &px[y * stride];
    const uint8_t* up = y ? &px[(y - 1) * stride] : nullptr;
    for (size_t i = 0; i < stride; ++i) {
      const int a = i >= (size_t)channels ? out[i - channels] : 0, b = up ? up[i] : 0,
                c = (up && i >= (size_t)channels) ? up[i - channels] : 0;
      int v = in[i];
      switch (ft) {
        case 0: break;
        case 1: v += a; break;
        case 2: v += b; break;
        case 3: v += (a + b) >> 1; break;
        case 4: v += paeth(a, b, c); break;
        default: return *err = "bad PNG row filter", false;
      }
      out[i] = (uint8_t)v;
    }
  }
  img->width = (int)w;
  img->height = (int)h;
  img->channels = ctype == 3 ? 3 : channels;  // a palette expands to RGB
  img->rgb.resize((size_t)w * h * 3);
  for (size_t i = 0; i < (size_t)w * h; ++i) {
    uint8_t* o = &img->rgb[3 * i];
    if (ctype == 3) {
      const size_t e = 3 * (size_t)px[i];
      if (e + 2 >= palette.size()) return *err = "PNG palette index out of range", false;
      o[0] = palette[e], o[1] = palette[e + 1], o[2] = palette[e + 2];
    } else if (channels <= 2) {
      o[0] = o[1] = o[2] = px[i * channels];
    } else {
      o[0] = px[i * channels], o[1] = px[i * channels + 1], o[2] = px[i * channels + 2];
    }
  }
  return true;
}

bool decode_bmp(const std::vector<uint8_t>& f, Image8* img, std::string* err) {
  if (f.size() < 54 || f[0] != 'B' || f[1] != 'M') return *err = "not a BMP file", false;
  const uint32_t off = le32(&f[10]), dib = le32(&f[14]);
  if (dib < 40) return *err = "unsupported BMP header", false;
  const int32_t w = (int32_t)le32(&f[18]), hs = (int32_t)le32(&f[22]);
  const int bpp = (int)le16(&f[28]);
  const uint32_t comp = le32(&f[30]);
  if (w <= 0 || hs == 0 || w > (1 << 15) || hs > (1 << 15) || hs < -(1 << 15)) return *err = "BMP size out of range", false;
  if ((bpp != 24 && bpp != 32) || !(comp == 0 || (comp == 3 && bpp == 32)))
    return *err = "only uncompressed 24/32-bit BMP is supported", false;
  const int h = hs < 0 ? -hs : hs;
  const size_t stride = (((size_t)w * bpp / 8) + 3) & ~(size_t)3;
  if (off + stride * h > f.size()) return *err = "truncated BMP", false;
  img->width = w;
  img->height = h;
  img->channels = bpp / 8;
  img->rgb.resize((size_t)w * h * 3);
  for (int y = 0; y < h; ++y) {
    const int src_row = hs > 0 ? h - 1 - y : y;  // positive height: stored bottom-up
    const uint8_t* row = &f[off + stride * src_row];
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = row + (size_t)x * (bpp / 8);
      uint8_t* o = &img->rgb[3 * ((size_t)y * w + x)];
      o[0] = p[2], o[1] = p[1], o[2] = p[0];
    }
  }
  return true;
}

bool decode_tga(const std::vector<uint8_t>& f, Image8* img, std::string* err) {
  if (f.size() < 18) return *err = "not a TGA file", false;
  const int idlen = f[0], cmap = f[1], type = f[2];
  const int w = (int)le16(&f[12]), h = (int)le16(&f[14]), bpp = f[16], desc = f[17];
  if (cmap != 0 || (type != 2 && type != 10)) return *err = "only true-colour TGA is supported", false;
  if ((bpp != 24 && bpp != 32) || w <= 0 || h <= 0) return *err = "unsupported TGA pixel format", false;
  const int bytes = bpp / 8;
  std::vector<uint8_t> px((size_t)w * h * bytes);
  size_t pos = 18 + idlen, o = 0;
  if (type == 2) {
    if (pos + px.size() > f.size()) return *err = "truncated TGA", false;
    std::memcpy(px.data(), &f[pos], px.size());
  } else {  // run-length packets
    while (o < px.size()) {
      if (pos >= f.size()) return *err = "truncated TGA", false;
      const int hdr = f[pos++], count = (hdr & 0x7f) + 1;
      if (o + (size_t)count * bytes > px.size()) return *err = "corrupt TGA run", false;
      if (hdr & 0x80) {
        if (pos + bytes > f.size()) return *err = "truncated TGA", false;
        for (int k = 0; k < count; ++k, o += bytes) std::memcpy(&px[o], &f[pos], bytes);
        pos += bytes;
      } else {
        if (pos + (size_t)count * bytes > f.size()) return *err = "truncated TGA", false;
        std::memcpy(&px[o], &f[pos], (size_t)count * bytes);
        pos += (size_t)count * bytes;
        o += (size_t)count * bytes;
      }
    }
  }
  const bool top_first = (desc & 0x20) != 0;
  img->width = w;
  img->height = h;
  img->channels = bytes;
  img->rgb.resize((size_t)w * h * 3);
  for (int y = 0; y < h; ++y) {
    const int src = top_first ? y : h - 1 - y;
    for (int x = 0; x < w; ++x) {
      const uint8_t* p = &px[((size_t)src * w + x) * bytes];
      uint8_t* q = &img->rgb[3 * ((size_t)y * w + x)];
      q[0] = p[2], q[1] = p[1], q[2] = p[0];
    }
  }
  return true;
}

bool decode_ppm(const std::vector<uint8_t>& f, Image8* img, std::string* err) {
  size_t pos = 2;
  auto number = [&](long* v) {
    while (pos < f.size()) {  // whitespace and comments
      if (f[pos] == '#') {
        while (pos < f.size() && f[pos] != '\n') ++pos;
      } else if (f[pos] == ' ' || f[pos] == '\t' || f[pos] == '\r' || f[pos] == '\n') {
        ++pos;
      } else {
        break;
      }
    }
    long n = 0;
    const size_t start = pos;
    while (pos < f.size() && f[pos] >= '0' && f[pos] <= '9') n = n * 10 + (f[pos++] - '0');
    *v = n;
    return pos > start && n < (1L << 20);
  };
  long w, h, maxval;
  if (f.size() < 2 || f[0] != 'P' || f[1] != '6' || !number(&w) || !number(&h) || !number(&maxval))
    return *err = "not a binary PPM (P6) file", false;
  if (maxval != 255 || w <= 0 || h <= 0) return *err = "only 8-bit PPM is supported", false;
  ++pos;  // the single whitespace byte after maxval
  if (pos + (size_t)w * h * 3 > f.size()) return *err = "truncated PPM", false;
  img->width = (int)w;
  img->height = (int)h;
  img->channels = 3;
  img->rgb.assign(f.begin() + pos, f.begin() + pos + (size_t)w * h * 3);
  return true;
}

}  // namespace

bool load_image8(const std::string& path, Image8* img, std::string* err) {
  std::vector<uint8_t> f;
  if (!read_all(path, &f)) return *err = "cannot read image " + path, false;
  bool ok;
  if (f.size() >= 8 && f[0] == 137 && f[1] == 'P' && f[2] == 'N' && f[3] == 'G')
    ok = decode_png(f, img, err);
  else if (f.size() >= 2 && f[0] == 'B' && f[1] == 'M')
    ok = decode_bmp(f, img, err);
  else if (f.size() >= 2 && f[0] == 'P' && f[1] == '6')
    ok = decode_ppm(f, img, err);
  else
    ok = decode_tga(f, img, err);  // TGA has no signature
  if (!ok) *err = path + ": " + *err;
  return ok;
}

}  // namespace orion_gb300
