// Device light sampling (src/core/light.h, src/light/*.cpp) and the
// light-selection distribution (Distribution1D::sampleDiscrete,
// src/sampler/sampling.h:71-125 with findInterval, src/core/geometry.h:877-889).
#pragma once
#include "device_types.h"
#include "dmath.cuh"

namespace orion_gb300 {

struct LightDistrib {
  const float* func;  // n light powers (intensity)
  const float* cdf;   // n + 1
  float func_int;
  int n;
};

__device__ __forceinline__ int find_interval(const float* cdf, int size, float u) {
  int first = 0, len = size;
  while (len > 0) {
    int half = len >> 1, middle = first + half;
    if (__ldg(cdf + middle) <= u) {
      first = middle + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  int r = first - 1;
  return r < 0 ? 0 : (r > size - 2 ? size - 2 : r);
}

__device__ __forceinline__ int sample_discrete(const LightDistrib& d, float u, float* pdf) {
  int off = find_interval(d.cdf, d.n + 1, u);
  *pdf = d.func_int > 0.f ? __ldg(d.func + off) / (d.func_int * d.n) : 0.f;
  return off;
}

// What a light sample needs from the shading point.
struct LightSample {
  V3 Li;       // incident radiance (before visibility)
  V3 wi;       // unit direction to the light
  float pdf;   // solid-angle pdf (1 for delta lights)
  V3 p_light;  // the point the shadow ray ends at
  bool valid;
};

__device__ __forceinline__ V3 mat3_mul(const float* m, V3 v) {
  return V3{m[0] * v.x + m[1] * v.y + m[2] * v.z, m[3] * v.x + m[4] * v.y + m[5] * v.z,
            m[6] * v.x + m[7] * v.y + m[8] * v.z};
}

// ------------------------------------------------ image environment maps

// Distribution1D::sampleContinuous (src/sampler/sampling.h:93-109).
__device__ __forceinline__ float dist1d_sample(const float* func, const float* cdf, int n, float func_int, float u,
                                               float* pdf, int* off) {
  const int offset = find_interval(cdf, n + 1, u);
  if (off) *off = offset;
  const float c0 = __ldg(cdf + offset), c1 = __ldg(cdf + offset + 1);
  float du = u - c0;
  if (c1 - c0 > 0.f) du /= (c1 - c0);
  *pdf = func_int > 0.f ? __ldg(func + offset) / func_int : 0.f;
  return (offset + du) / n;
}

// Distribution2D::SampleContinuous (src/sampler/sampling.h:131-138): the
// marginal picks the row with u1, the row's conditional the column with u0.
__device__ __forceinline__ void dist2d_sample(const DevEnvMap& e, float u0, float u1, float* su, float* sv,
                                              float* pdf) {
  float p0, p1;
  int v;
  *sv = dist1d_sample(e.marg_func, e.marg_cdf, e.height, e.marg_int, u1, &p1, &v);
  *su = dist1d_sample(e.cond_func + (size_t)v * e.width, e.cond_cdf + (size_t)v * (e.width + 1), e.width,
                      __ldg(e.cond_int + v), u0, &p0, nullptr);
  *pdf = p0 * p1;
}

// Distribution2D::Pdf (src/sampler/sampling.h:139-145).
__device__ __forceinline__ float dist2d_pdf(const DevEnvMap& e, float pu, float pv) {
  const int iu = min(max((int)(pu * e.width), 0), e.width - 1);
  const int iv = min(max((int)(pv * e.height), 0), e.height - 1);
  return __ldg(e.cond_func + (size_t)iv * e.width + iu) / e.marg_int;
}

// Texture::sample(u, v) with the default wrap filter (src/core/texture.cpp:3-7,
// 12-27) on an ImageTexture (src/texture/imagetexture.cpp:4-11).
__device__ __forceinline__ V3 env_texel(const DevEnvMap& e, float u, float v) {
  int x = (int)(u * e.width), y = (int)(v * e.height);
  x = x >= 0 ? x % e.width : e.width - (-x) % e.width;
  y = y >= 0 ? y % e.height : e.height - (-y) % e.height;
  const float* t = e.texels + 3 * ((size_t)y * e.width + x);
  return V3{__ldg(t), __ldg(t + 1), __ldg(t + 2)};
}

// Envmap::Le (src/light/envmap.cpp:44-49): the map in the direction of `d`.
__device__ __forceinline__ V3 env_le(const DevLight& L, const DevEnvMap* envmaps, V3 d) {
  if (L.image < 0) return ld3(L.L);
  const V3 w = normalize(mat3_mul(L.minv, d));
  return env_texel(envmaps[L.image], spherical_phi(w) * kInv2Pi, spherical_theta(w) * kInvPi);
}

// Light::sample_Li for every light type. `prims` gives the emissive
// triangle of an area light; `world_radius` bounds the scene for distant and
// environment lights (Bounds3::boundingSphere, src/core/geometry.h:551-554).
static __device__ __noinline__ LightSample sample_li(const DevLight& L, const PrimShade* __restrict__ prims,
                                                    const DevEnvMap* envmaps, V3 ref_p, float u0, float u1,
                                                    float world_radius) {
  LightSample s;
  s.valid = false;
  s.pdf = 0.f;
  s.Li = V3{0, 0, 0};
  s.wi = V3{0, 0, 1};
  s.p_light = ref_p;
  switch (L.kind) {
    case DL_AREA: {
      // Triangle::sample (src/core/triangle.cpp:85-121) + DiffuseAreaLight::sample_Li (diffuse.cpp:12-26)
      const PrimShade& sh = prims[L.prim];
      V3 p0 = ld3(sh.p), p1 = ld3(sh.p + 3), p2 = ld3(sh.p + 6);
      V3 n0 = ld3(sh.n), n1 = ld3(sh.n + 3), n2 = ld3(sh.n + 6);
      float b0, b1;
      uniform_sample_triangle(u0, u1, &b0, &b1);
      float b2 = 1.f - b0 - b1;
      V3 p = b0 * p0 + b1 * p1 + b2 * p2;
      V3 ng = normalize(cross(p1 - p0, p2 - p0));
      V3 ns = n0 * b0 + n1 * b1 + n2 * b2;
      ng = faceforward(ng, ns);
      float pdf = 1.f / L.area;
      V3 w = p - ref_p;
      if (length_sq(w) == 0.f) {
        pdf = 0.f;
      } else {
        w = normalize(w);
        pdf *= length_sq(ref_p - p) / absdot(ng, -w);
        if (isinf(pdf)) pdf = 0.f;
      }
      s.p_light = p;
      if (pdf == 0.f || length_sq(p - ref_p) == 0.f) return s;
      s.wi = normalize(p - ref_p);
      s.pdf = pdf;
      s.Li = dot(ng, -s.wi) > 0.f ? ld3(L.L) : V3{0, 0, 0};
      s.valid = true;
      return s;
    }
    case DL_POINT: {  // src/light/point.cpp:10-19
      V3 lp = ld3(L.p);
      s.wi = normalize(lp - ref_p);
      s.pdf = 1.f;
      s.p_light = lp;
      s.Li = sdiv(ld3(L.L), length_sq(lp - ref_p));
      s.valid = true;
      return s;
    }
    case DL_SPOT: {  // src/light/spot.cpp:10-29
      V3 lp = ld3(L.p);
      s.wi = normalize(lp - ref_p);
      s.pdf = 1.f;
      s.p_light = lp;
      V3 wl = normalize(mat3_mul(L.m, -s.wi));
      float c = wl.z, fall;
      if (c < L.cos_total)
        fall = 0.f;
      else if (c > L.cos_falloff)
        fall = 1.f;
      else {
        float delta = (c - L.cos_total) / (L.cos_falloff - L.cos_total);
        fall = (delta * delta) * (delta * delta);
      }
      s.Li = sdiv(ld3(L.L) * fall, length_sq(lp - ref_p));
      s.valid = true;
      return s;
    }
    case DL_DISTANT: {  // src/light/distant.cpp:15-25
      s.wi = ld3(L.p);
      s.pdf = 1.f;
      s.p_light = ref_p + s.wi * (2.f * world_radius);
      s.Li = ld3(L.L);
      s.valid = true;
      return s;
    }
    case DL_ENV: {  // src/light/envmap.cpp:50-68
      if (L.image >= 0) {
        const DevEnvMap& e = envmaps[L.image];
        float su, sv, map_pdf;
        dist2d_sample(e, u0, u1, &su, &sv, &map_pdf);
        if (map_pdf == 0.f) return s;
        const float theta = sv * kPi, phi = su * 2.f * kPi;
        const float ct = cosf(theta), st = sinf(theta), sp = sinf(phi), cp = cosf(phi);
        s.wi = mat3_mul(L.m, V3{st * cp, st * sp, ct});
        s.pdf = map_pdf / (2.f * kPi * kPi * st);
        if (st == 0.f) s.pdf = 0.f;
        s.p_light = ref_p + s.wi * (2.f * world_radius);
        s.Li = env_texel(e, su, sv);
        s.valid = true;
        return s;
      }
      // Constant map: a 1x1 Distribution2D (uv = u, mapPdf = 1).
      if (L.area == 0.f) return s;  // zero-intensity map: the distribution's pdf is 0
      float theta = u1 * kPi, phi = u0 * 2.f * kPi;
      float ct = cosf(theta), st = sinf(theta), sp = sinf(phi), cp = cosf(phi);
      s.wi = mat3_mul(L.m, V3{st * cp, st * sp, ct});
      s.pdf = 1.f / (2.f * kPi * kPi * st);
      if (st == 0.f) s.pdf = 0.f;
      s.p_light = ref_p + s.wi * (2.f * world_radius);
      s.Li = ld3(L.L);
      s.valid = true;  // the reference returns the radiance even when the pdf is 0
      return s;
    }
  }
  return s;
}

// Envmap::pdf_Li (src/light/envmap.cpp:70-80). As written there, the map's
// v coordinate is theta / (2 pi) (not theta / pi), and its sin(theta) == 0
// test compares a function with 0, so it never returns early.
__device__ __forceinline__ float env_pdf_li(const DevLight& L, const DevEnvMap* envmaps, V3 wi) {
  V3 w = mat3_mul(L.minv, wi);
  float theta = spherical_theta(w);
  float st = sinf(theta);
  if (L.image < 0) return 1.f / (2.f * kPi * kPi * st);  // constant map: Pdf = 1
  const float phi = spherical_phi(w);
  return dist2d_pdf(envmaps[L.image], phi * kInv2Pi, theta * kInv2Pi) / (2.f * kPi * kPi * st);
}

// Light::sample_Le for every light type (src/light/diffuse.cpp:32-44,
// point.cpp:20-27, spot.cpp:30-38, distant.cpp:28-41, envmap.cpp:82-104):
// an emitted ray (origin, direction), the emitter normal, and the position
// and direction pdfs. r0 / r1 are the reference's two Point2f samples.
struct EmittedRay {
  V3 Le, o, d, n;
  float pdf_pos, pdf_dir;
};

static __device__ __noinline__ EmittedRay sample_le(const DevLight& L, const PrimShade* __restrict__ prims,
                                                    const DevEnvMap* envmaps, const float* world_center,
                                                    float world_radius, float r0x, float r0y, float r1x, float r1y) {
  EmittedRay e;
  e.Le = V3{0, 0, 0};
  e.o = e.d = e.n = V3{0, 0, 1};
  e.pdf_pos = e.pdf_dir = 0.f;
  const V3 wc = ld3(world_center);
  switch (L.kind) {
    case DL_AREA: {  // Triangle::sample (triangle.cpp:85-106), cosine-weighted direction about ng
      const PrimShade& sh = prims[L.prim];
      V3 p0 = ld3(sh.p), p1 = ld3(sh.p + 3), p2 = ld3(sh.p + 6);
      V3 n0 = ld3(sh.n), n1 = ld3(sh.n + 3), n2 = ld3(sh.n + 6);
      float b0, b1;
      uniform_sample_triangle(r0x, r0y, &b0, &b1);
      float b2 = 1.f - b0 - b1;
      V3 p = b0 * p0 + b1 * p1 + b2 * p2;
      V3 ng = normalize(cross(p1 - p0, p2 - p0));
      V3 ns = n0 * b0 + n1 * b1 + n2 * b2;
      ng = faceforward(ng, ns);
      e.pdf_pos = 1.f / L.area;
      e.n = ng;
      V3 w = cosine_sample_hemisphere(r1x, r1y);
      e.pdf_dir = w.z * kInvPi;
      V3 x, y;
      coordinate_system(ng, &x, &y);
      w = w.x * x + w.y * y + w.z * ng;
      e.o = offset_ray_origin(p, ng, w);
      e.d = w;
      e.Le = dot(ng, w) > 0.f ? ld3(L.L) : V3{0, 0, 0};
      return e;
    }
    case DL_POINT:
      e.o = ld3(L.p);
      e.d = uniform_sample_sphere(r0x, r0y);
      e.n = e.d;
      e.pdf_pos = 1.f;
      e.pdf_dir = kInv4Pi;
      e.Le = ld3(L.L);
      return e;
    case DL_SPOT: {
      e.o = ld3(L.p);
      e.d = mat3_mul(L.minv, uniform_sample_cone(r0x, r0y, L.cos_total));
      e.n = e.d;
      e.pdf_pos = 1.f;
      e.pdf_dir = 1.f / (2.f * kPi * (1.f - L.cos_total));
      V3 wl = normalize(mat3_mul(L.m, e.d));
      float c = wl.z, fall;
      if (c < L.cos_total)
        fall = 0.f;
      else if (c > L.cos_falloff)
        fall = 1.f;
      else {
        float delta = (c - L.cos_total) / (L.cos_falloff - L.cos_total);
        fall = (delta * delta) * (delta * delta);
      }
      e.Le = ld3(L.L) * fall;
      return e;
    }
    case DL_DISTANT: {
      const V3 dir = ld3(L.p);
      V3 v1, v2;
      coordinate_system(dir, &v1, &v2);
      float cx, cy;
      concentric_sample_disk(r0x, r0y, &cx, &cy);
      V3 pd = wc + world_radius * (cx * v1 + cy * v2);
      e.o = pd + world_radius * dir;
      e.d = -dir;
      e.n = e.d;
      e.pdf_pos = 1.f / (kPi * world_radius * world_radius);
      e.pdf_dir = 1.f;
      e.Le = ld3(L.L);
      return e;
    }
    case DL_ENV: {
      float su, sv, map_pdf;
      if (L.image >= 0) {
        dist2d_sample(envmaps[L.image], r0x, r0y, &su, &sv, &map_pdf);
      } else {  // 1x1 distribution: uv = u, mapPdf = 1 (0 for a zero-intensity map)
        su = r0x;
        sv = r0y;
        map_pdf = L.area == 0.f ? 0.f : 1.f;
      }
      if (map_pdf == 0.f) return e;
      const float theta = sv * kPi, phi = su * 2.f * kPi;
      const float ct = cosf(theta), st = sinf(theta), sp = sinf(phi), cp = cosf(phi);
      const V3 d = -mat3_mul(L.m, V3{st * cp, st * sp, ct});
      e.n = d;
      V3 v1, v2;
      coordinate_system(-d, &v1, &v2);
      float cx, cy;
      concentric_sample_disk(r1x, r1y, &cx, &cy);
      V3 pd = wc + world_radius * (cx * v1 + cy * v2);
      e.o = pd + world_radius * -d;
      e.d = d;
      e.pdf_dir = st == 0.f ? 0.f : map_pdf / (2.f * kPi * kPi * st);
      e.pdf_pos = 1.f / (kPi * world_radius * world_radius);
      e.Le = L.image >= 0 ? env_texel(envmaps[L.image], su, sv) : ld3(L.L);
      return e;
    }
  }
  return e;
}

__device__ __forceinline__ bool is_delta_light(int kind) { return kind == DL_POINT || kind == DL_SPOT || kind == DL_DISTANT; }

}  // namespace orion_gb300
