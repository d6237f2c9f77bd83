// Device math for the path tracer: FP32 vectors and RGB spectra with the
// reference's operation order, its sampling warps and the Sobol sampler.
//
// Conventions copied from the reference because results depend on them:
//   * Vector / scalar multiplies by the reciprocal (src/core/geometry.h:169-173),
//     Spectrum / scalar divides each channel (src/core/spectrum.h:138-141);
//   * normalize(v) = v * (1 / length(v)) (src/core/geometry.h:794-798);
//   * dot products sum left to right.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace orion_gb300 {

constexpr float kPi = 3.14159265358979323846f;
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv2Pi = 0.15915494309189533577f;
constexpr float kInv4Pi = 0.07957747154594766788f;
constexpr float kPiOver2 = 1.57079632679489661923f;
constexpr float kPiOver4 = 0.78539816339744830961f;
constexpr float kEpsilon = 0.000001f;        // src/orion.h:48
constexpr float kShadowEpsilon = 0.01f;      // src/orion.h:49
constexpr float kOneMinusEpsilon = 0.99999994f;
constexpr float kFloatMax = 3.402823466e+38f;  // fInfinity, src/orion.h:51

struct V3 {
  float x, y, z;
};

__device__ __forceinline__ V3 v3(float x, float y, float z) { return V3{x, y, z}; }
__device__ __forceinline__ V3 operator+(V3 a, V3 b) { return V3{a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ V3 operator-(V3 a, V3 b) { return V3{a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ V3 operator-(V3 a) { return V3{-a.x, -a.y, -a.z}; }
__device__ __forceinline__ V3 operator*(V3 a, float s) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 operator*(float s, V3 a) { return V3{a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ V3 mul(V3 a, V3 b) { return V3{a.x * b.x, a.y * b.y, a.z * b.z}; }
// Spectrum / float: per-channel division.
__device__ __forceinline__ V3 sdiv(V3 a, float f) { return V3{a.x / f, a.y / f, a.z / f}; }
// Vector / float: multiply by the reciprocal.
__device__ __forceinline__ V3 vdiv(V3 a, float f) {
  float inv = 1.f / f;
  return V3{a.x * inv, a.y * inv, a.z * inv};
}
__device__ __forceinline__ float dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ float absdot(V3 a, V3 b) { return fabsf(dot(a, b)); }
__device__ __forceinline__ V3 cross(V3 a, V3 b) {
  return V3{a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ float length_sq(V3 a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
__device__ __forceinline__ float length(V3 a) { return sqrtf(length_sq(a)); }
__device__ __forceinline__ V3 normalize(V3 a) { return vdiv(a, length(a)); }
__device__ __forceinline__ V3 vabs(V3 a) { return V3{fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
__device__ __forceinline__ bool is_black(V3 s) { return s.x == 0.f && s.y == 0.f && s.z == 0.f; }
__device__ __forceinline__ float max_comp(V3 s) { return fmaxf(s.x, fmaxf(s.y, s.z)); }
__device__ __forceinline__ V3 sclamp0(V3 s) {  // Spectrum::clamp(): low 0, no upper bound
  return V3{s.x < 0.f ? 0.f : s.x, s.y < 0.f ? 0.f : s.y, s.z < 0.f ? 0.f : s.z};
}
__device__ __forceinline__ float clampf(float f, float lo, float hi) { return f < lo ? lo : (f > hi ? hi : f); }
__device__ __forceinline__ V3 ld3(const float* p) { return V3{p[0], p[1], p[2]}; }
__device__ __forceinline__ V3 xyz(float4 f) { return V3{f.x, f.y, f.z}; }
__device__ __forceinline__ float4 f4(V3 a, float w) { return make_float4(a.x, a.y, a.z, w); }
__device__ __forceinline__ V3 faceforward(V3 n, V3 v) { return dot(n, v) < 0.f ? -n : n; }

// Shading-frame trigonometry (src/sampler/sampling.h:13-34). cosPhi/sinPhi
// in the reference compare a function pointer with zero, so their
// sinTheta == 0 branch never runs; that is kept.
__device__ __forceinline__ float cos_theta(V3 w) { return w.z; }
__device__ __forceinline__ float cos2_theta(V3 w) { return w.z * w.z; }
__device__ __forceinline__ float abs_cos_theta(V3 w) { return fabsf(w.z); }
__device__ __forceinline__ float sin2_theta(V3 w) { return fmaxf(0.f, 1.f - cos2_theta(w)); }
__device__ __forceinline__ float sin_theta(V3 w) { return sqrtf(sin2_theta(w)); }
__device__ __forceinline__ float tan_theta(V3 w) { return sin_theta(w) / cos_theta(w); }
__device__ __forceinline__ float tan2_theta(V3 w) { return sin2_theta(w) / cos2_theta(w); }
__device__ __forceinline__ float cos_phi(V3 w) { return clampf(w.x / sin_theta(w), -1.f, 1.f); }
__device__ __forceinline__ float sin_phi(V3 w) { return clampf(w.y / sin_theta(w), -1.f, 1.f); }
__device__ __forceinline__ bool same_hemisphere(V3 a, V3 b) { return a.z * b.z > 0.f; }

// ---------------------------------------------------------------- warps

// src/sampler/sampling.cpp:29-33
__device__ __forceinline__ void uniform_sample_disk(float u0, float u1, float* x, float* y) {
  float r = sqrtf(u0);
  float theta = 2.f * kPi * u1;
  *x = r * cosf(theta);
  *y = r * sinf(theta);
}

// src/sampler/sampling.cpp:56-61
__device__ __forceinline__ V3 cosine_sample_hemisphere(float u0, float u1) {
  float x, y;
  uniform_sample_disk(u0, u1, &x, &y);
  float z = sqrtf(fmaxf(0.f, 1.f - x * x - y * y));
  return V3{x, y, z};
}

// src/sampler/sampling.cpp:35-54
__device__ __forceinline__ void concentric_sample_disk(float u0, float u1, float* x, float* y) {
  float ox = 2.f * u0 - 1.f, oy = 2.f * u1 - 1.f;
  if (ox == 0.f && oy == 0.f) {
    *x = 0.f;
    *y = 0.f;
    return;
  }
  float theta, r;
  if (fabsf(ox) > fabsf(oy)) {
    r = ox;
    theta = kPiOver4 * (oy / ox);
  } else {
    r = oy;
    theta = kPiOver2 - kPiOver4 * (ox / oy);
  }
  *x = cosf(theta) * r;
  *y = sinf(theta) * r;
}

// src/sampler/sampling.cpp:14-18
__device__ __forceinline__ void uniform_sample_triangle(float u0, float u1, float* b0, float* b1) {
  float su0 = sqrtf(u0);
  *b0 = 1.f - su0;
  *b1 = u1 * su0;
}

// src/sampler/sampling.cpp:5-11
__device__ __forceinline__ V3 uniform_sample_sphere(float u0, float u1) {
  float z = 1.f - 2.f * u0;
  float r = sqrtf(fmaxf(0.f, 1.f - z * z));
  float phi = 2.f * kPi * u1;
  return V3{r * cosf(phi), r * sinf(phi), z};
}

// src/sampler/sampling.cpp:20-27
__device__ __forceinline__ V3 uniform_sample_cone(float u0, float u1, float cos_max) {
  float cos_t = (1.f - u0) + u0 * cos_max;
  float sin_t = sqrtf(1.f - cos_t * cos_t);
  float phi = u1 * 2.f * kPi;
  return V3{cosf(phi) * sin_t, sinf(phi) * sin_t, cos_t};
}

// coordinateSystem (src/core/geometry.h:902-909): x, y completing z.
__device__ __forceinline__ void coordinate_system(V3 z, V3* x, V3* y) {
  if (fabsf(z.x) > fabsf(z.y))
    *y = vdiv(V3{-z.z, 0.f, z.x}, sqrtf(z.x * z.x + z.z * z.z));
  else
    *y = vdiv(V3{0.f, z.z, -z.y}, sqrtf(z.y * z.y + z.z * z.z));
  *x = cross(*y, z);
}

// Spectrum::intensity (src/core/spectrum.h:88-91)
__device__ __forceinline__ float spectrum_intensity(V3 c) { return 0.212671f * c.x + 0.715160f * c.y + 0.072169f * c.z; }

// src/sampler/sampling.h:49-52
__device__ __forceinline__ float power_heuristic(float fpdf, float gpdf) {
  float f = fpdf, g = gpdf;
  return (f * f) / (f * f + g * g);
}

// src/sampler/sampling.h:61-69
__device__ __forceinline__ float spherical_theta(V3 v) { return acosf(clampf(v.z, -1.f, 1.f)); }
__device__ __forceinline__ float spherical_phi(V3 v) {
  float p = atan2f(v.y, v.x);
  return p < 0.f ? p + 2.f * kPi : p;
}

// ------------------------------------------------- ray origin offsetting

// src/core/geometry.h:824-848
__device__ __forceinline__ float next_float_up(float v) {
  if (isinf(v) && v > 0.f) return v;
  if (v == -0.f) v = 0.f;
  uint32_t ui = __float_as_uint(v);
  ui = v >= 0.f ? ui + 1 : ui - 1;
  return __uint_as_float(ui);
}
__device__ __forceinline__ float next_float_down(float v) {
  if (isinf(v) && v < 0.f) return v;
  if (v == 0.f) v = -0.f;
  uint32_t ui = __float_as_uint(v);
  ui = v > 0.f ? ui - 1 : ui + 1;
  return __uint_as_float(ui);
}

// src/core/geometry.h:850-866: push p off the surface along +-n by
// 1e-6 * max|p| * |n|_1, then one more ulp away.
__device__ __forceinline__ V3 offset_ray_origin(V3 p, V3 n, V3 w) {
  float m = fmaxf(fmaxf(fabsf(p.x), fabsf(p.y)), fabsf(p.z));
  float e = m * kEpsilon;
  float d = fabsf(n.x) * e + fabsf(n.y) * e + fabsf(n.z) * e;
  V3 off = n * d;
  if (dot(w, n) < 0.f) off = -off;
  V3 po = p + off;
  if (off.x > 0.f) po.x = next_float_up(po.x); else if (off.x < 0.f) po.x = next_float_down(po.x);
  if (off.y > 0.f) po.y = next_float_up(po.y); else if (off.y < 0.f) po.y = next_float_down(po.y);
  if (off.z > 0.f) po.z = next_float_up(po.z); else if (off.z < 0.f) po.z = next_float_down(po.z);
  return po;
}

// ----------------------------------------------------------------- Sobol

// sobol::sample (src/sampler/sobol.h:28-43): XOR of the dimension's
// direction numbers for the set bits of the index, scaled by 2^-32.
// Unscrambled; can return exactly 1.0f like the reference. The device holds
// the direction numbers as tables: entry [dim][k][v] is the XOR of the
// numbers of the set bits of v placed at index bits 8k..8k+7, so the XOR over
// the index's set bits is one lookup per index byte (four for an index below
// 2^32, against one per set bit: 13 on average for 26-bit indices). Indices
// of 2^52 and above, beyond the reference's direction numbers, get none for
// their bits 52 and up.
__device__ __forceinline__ uint32_t sobol_bits(const uint32_t* __restrict__ t, uint64_t index) {
  uint32_t r = __ldg(t + (uint32_t)(index & 0xffu)) ^ __ldg(t + 256 + (uint32_t)((index >> 8) & 0xffu)) ^
               __ldg(t + 512 + (uint32_t)((index >> 16) & 0xffu)) ^ __ldg(t + 768 + (uint32_t)((index >> 24) & 0xffu));
  if (index >> 32) {
#pragma unroll
    for (int k = 4; k < kSobolBytes; ++k) r ^= __ldg(t + 256 * k + (uint32_t)((index >> (8 * k)) & 0xffu));
  }
  return r;
}

__device__ __forceinline__ float sobol_sample(const uint32_t* __restrict__ tables, uint64_t index, uint32_t dim) {
  return __uint2float_rn(sobol_bits(tables + (size_t)dim * kSobolBytes * 256, index)) * 2.3283064365386963e-10f;
}

// N consecutive dimensions d0..d0+N-1 of one index (their lookups are
// independent and issue together). Values are identical to sobol_sample.
template <int N>
__device__ __forceinline__ void sobol_dims(const uint32_t* __restrict__ tables, uint64_t index, uint32_t d0,
                                           float out[N]) {
  const uint32_t* t = tables + (size_t)d0 * kSobolBytes * 256;
#pragma unroll
  for (int k = 0; k < N; ++k)
    out[k] = __uint2float_rn(sobol_bits(t + (size_t)k * kSobolBytes * 256, index)) * 2.3283064365386963e-10f;
}

// A path's sampler: fixed sample index, advancing dimension
// (src/core/sampler.h:15-34, dimension starts at 5).
struct PathSampler {
  const uint32_t* tables;
  uint64_t index;
  uint32_t dim;
  __device__ __forceinline__ float next() { return sobol_sample(tables, index, dim++); }
};

}  // namespace orion_gb300
