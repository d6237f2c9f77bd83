// CPU oracle: a scalar C++ restatement of the reference's path-tracing hot
// path. TEST INFRASTRUCTURE ONLY -- loaded by tests/, the smoke check and
// bench.py's CPU-baseline leg; never by the product library.
//
// It follows the reference function by function (file:line cited at each),
// one path per OpenMP thread iteration like PathTracing::render, in FP32
// with the reference's operation order, and is compiled without FP
// contraction so x86 and Arm produce identical results. Closest hits come
// from the project CPU BVH (oracle/cpu_bvh.h) standing in for Embree.
// Parity of this file with the reference itself is pinned by the golden
// fixtures under tests/golden (generated from the reference compiled here).
//
// Input is the flat scene record of include/orion_gpu.h.
#include <omp.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <limits>
#include <memory>
#include <vector>

#include "../../include/orion_gpu.h"
#include "../cpu_bvh.h"

namespace port {

constexpr float kPi = 3.14159265358979323846f;     // src/orion.h:52-58
constexpr float kInvPi = 0.31830988618379067154f;
constexpr float kInv2Pi = 0.15915494309189533577f;
constexpr float kInv4Pi = 0.07957747154594766788f;
constexpr float kPiOver2 = 1.57079632679489661923f;
constexpr float kPiOver4 = 0.78539816339744830961f;
constexpr float kEpsilon = 0.000001f;
constexpr float kShadowEpsilon = 0.01f;
constexpr float kInfinity = std::numeric_limits<float>::max();
constexpr float kOneMinusEpsilon = 0.99999994f;

// ------------------------------------------------------------------- math

struct V {
  float x = 0, y = 0, z = 0;
  V() = default;
  V(float a, float b, float c) : x(a), y(b), z(c) {}
  explicit V(float a) : x(a), y(a), z(a) {}
  float operator[](int i) const { return i == 0 ? x : (i == 1 ? y : z); }
  float& operator[](int i) { return i == 0 ? x : (i == 1 ? y : z); }
};
inline V operator+(V a, V b) { return V(a.x + b.x, a.y + b.y, a.z + b.z); }
inline V operator-(V a, V b) { return V(a.x - b.x, a.y - b.y, a.z - b.z); }
inline V operator-(V a) { return V(-a.x, -a.y, -a.z); }
inline V operator*(V a, float s) { return V(a.x * s, a.y * s, a.z * s); }
inline V operator*(float s, V a) { return V(a.x * s, a.y * s, a.z * s); }
inline V mul(V a, V b) { return V(b.x * a.x, b.y * a.y, b.z * a.z); }          // Spectrum * Spectrum
inline V sdiv(V a, float f) { return V(a.x / f, a.y / f, a.z / f); }          // Spectrum / float
inline V vdiv(V a, float f) {                                                  // Vector / float
  float inv = 1.f / f;
  return V(a.x * inv, a.y * inv, a.z * inv);
}
inline float dot(V a, V b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
inline float absdot(V a, V b) { return std::abs(a.x * b.x + a.y * b.y + a.z * b.z); }
inline V cross(V a, V b) {
  float ax = a.x, ay = a.y, az = a.z, bx = b.x, by = b.y, bz = b.z;
  return V((ay * bz) - (az * by), (az * bx) - (ax * bz), (ax * by) - (ay * bx));
}
inline float len_sq(V a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
inline V normalize(V a) { return vdiv(a, std::sqrt(len_sq(a))); }
inline bool black(V s) { return !(s.x != 0.0f || s.y != 0.0f || s.z != 0.0f); }
inline float maxc(V s) { return std::max(s.x, std::max(s.y, s.z)); }
inline float clampf(float f, float lo, float hi) { return f < lo ? lo : (f > hi ? hi : f); }
inline V clamp0(V s) { return V(clampf(s.x, 0, kInfinity), clampf(s.y, 0, kInfinity), clampf(s.z, 0, kInfinity)); }
inline V faceforward(V n, V v) { return dot(n, v) < 0.f ? -n : n; }
inline float intensity(V s) { return 0.212671f * s.x + 0.715160f * s.y + 0.072169f * s.z; }  // spectrum.h:88-91
inline V ld(const float* p) { return V(p[0], p[1], p[2]); }

// src/sampler/sampling.h:13-34 (cosPhi/sinPhi compare a function pointer,
// so the sinTheta == 0 guard never fires)
inline float cosT(V w) { return w.z; }
inline float cos2T(V w) { return w.z * w.z; }
inline float absCosT(V w) { return std::abs(w.z); }
inline float sin2T(V w) { return std::max(0.0f, 1.0f - cos2T(w)); }
inline float sinT(V w) { return std::sqrt(sin2T(w)); }
inline float tanT(V w) { return sinT(w) / cosT(w); }
inline float tan2T(V w) { return sin2T(w) / cos2T(w); }
inline float cosP(V w) { return clampf(w.x / sinT(w), -1.0f, 1.0f); }
inline float sinP(V w) { return clampf(w.y / sinT(w), -1.0f, 1.0f); }
inline bool sameHemi(V a, V b) { return a.z * b.z > 0; }

// src/sampler/sampling.cpp
inline void uniformSampleDisk(float u0, float u1, float* x, float* y) {
  float r = std::sqrt(u0);
  float theta = 2 * kPi * u1;
  *x = r * std::cos(theta);
  *y = r * std::sin(theta);
}
inline V cosineSampleHemisphere(float u0, float u1) {
  float x, y;
  uniformSampleDisk(u0, u1, &x, &y);
  float z = std::sqrt(std::max(0.0f, 1 - x * x - y * y));
  return V(x, y, z);
}
inline void concentricSampleDisk(float u0, float u1, float* x, float* y) {
  float ox = 2.f * u0 - 1.0f, oy = 2.f * u1 - 1.0f;
  if (ox == 0 && oy == 0) {
    *x = 0;
    *y = 0;
    return;
  }
  float theta, r;
  if (std::abs(ox) > std::abs(oy)) {
    r = ox;
    theta = kPiOver4 * (oy / ox);
  } else {
    r = oy;
    theta = kPiOver2 - kPiOver4 * (ox / oy);
  }
  *x = std::cos(theta) * r;
  *y = std::sin(theta) * r;
}
inline float powerHeuristic(float f, float g) { return (f * f) / (f * f + g * g); }  // sampling.h:49-52

// src/core/geometry.h:824-866
inline float bitsf(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
inline uint32_t fbits(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}
inline float nextUp(float v) {
  if (std::isinf(v) && v > 0.) return v;
  if (v == -0.f) v = 0.f;
  uint32_t ui = fbits(v);
  ui = v >= 0 ? ui + 1 : ui - 1;
  return bitsf(ui);
}
inline float nextDown(float v) {
  if (std::isinf(v) && v < 0.) return v;
  if (v == 0.f) v = -0.f;
  uint32_t ui = fbits(v);
  ui = v > 0 ? ui - 1 : ui + 1;
  return bitsf(ui);
}
inline V offsetRayOrigin(V p, V n, V w) {
  float m = std::max(std::max(std::abs(p.x), std::abs(p.y)), std::abs(p.z));
  V e(m * kEpsilon);
  float d = dot(V(std::abs(n.x), std::abs(n.y), std::abs(n.z)), e);
  V off = n * d;
  if (dot(w, n) < 0) off = -off;
  V po = p + off;
  for (int i = 0; i < 3; ++i) {
    if (off[i] > 0)
      po[i] = nextUp(po[i]);
    else if (off[i] < 0)
      po[i] = nextDown(po[i]);
  }
  return po;
}

// ------------------------------------------------------------------ Sobol

static std::vector<uint32_t> g_sobol;

// src/sampler/sobol.h:28-43
inline float sobolSample(uint64_t index, uint32_t dim) {
  uint32_t r = 0;
  for (size_t i = (size_t)dim * 52; index; index >>= 1, ++i)
    if (index & 1) r ^= g_sobol[i];
  return r * (1.f / (1ULL << 32));
}

struct Sampler {  // src/core/sampler.h:15-34, src/sampler/sobol.h:48-60
  uint64_t index;
  uint32_t dim = 5;
  float next() { return sobolSample(index, dim++); }
};

// ------------------------------------------------------------------- BSDF

enum { REFL = 1, TRANS = 2, DIFF = 4, GLOSSY = 8, SPEC = 16, ALL = 31 };
enum Kind { LAMBERT, OREN, MF_R, MF_T, SPEC_R, SPEC_T, FRES_SPEC };
enum Fres { F_NOOP, F_COND, F_DIEL };

struct Lobe {
  Kind kind;
  int type;
  Fres fres = F_NOOP;
  int beckmann = 0;
  V c, c2;
  float alpha = 0, etaA = 1, etaB = 1, A = 0, B = 0;
  V fr_eta, fr_k;
  bool photon = false;  // TransportMode::Photon: no radiance scaling on transmission
};

struct Mat {
  std::vector<Lobe> lobes;
};

// src/core/bsdf.cpp:149-170
float frDielectric(float cosI, float etaI, float etaT) {
  cosI = clampf(cosI, -1.0f, 1.0f);
  bool entering = cosI > 0.f;
  if (!entering) {
    std::swap(etaI, etaT);
    cosI = std::abs(cosI);
  }
  float sinI = std::sqrt(std::max((float)0, 1 - cosI * cosI));
  float sinTt = etaI / etaT * sinI;
  if (sinTt >= 1) return 1;
  float cosTt = std::sqrt(std::max((float)0, 1 - sinTt * sinTt));
  float rpa = ((etaT * cosI) - (etaI * cosTt)) / ((etaT * cosI) + (etaI * cosTt));
  float rpe = ((etaI * cosI) - (etaT * cosTt)) / ((etaI * cosI) + (etaT * cosTt));
  return (rpa * rpa + rpe * rpe) / 2;
}

// src/core/bsdf.cpp:124-147 with etai = 1
V frConductor(float cosI, V etat, V k) {
  cosI = clampf(cosI, -1.0f, 1.0f);
  V one(1.f);
  V eta(etat.x / one.x, etat.y / one.y, etat.z / one.z);
  V etak(k.x / one.x, k.y / one.y, k.z / one.z);
  float c2 = cosI * cosI, s2 = 1.f - c2;
  V eta2 = mul(eta, eta), etak2 = mul(etak, etak);
  V t0 = (eta2 - etak2) - V(s2);
  V q = mul(t0, t0) + mul(eta2 * 4.f, etak2);
  V a2b2(std::sqrt(q.x), std::sqrt(q.y), std::sqrt(q.z));
  V t1 = a2b2 + V(c2);
  V h = (a2b2 + t0) * 0.5f;
  V a(std::sqrt(h.x), std::sqrt(h.y), std::sqrt(h.z));
  V t2 = a * (2.f * cosI);
  V rs((t1.x - t2.x) / (t1.x + t2.x), (t1.y - t2.y) / (t1.y + t2.y), (t1.z - t2.z) / (t1.z + t2.z));
  V t3 = a2b2 * c2 + V(s2 * s2);
  V t4 = t2 * s2;
  V n3 = mul(rs, t3 - t4), d3 = t3 + t4;
  V rp(n3.x / d3.x, n3.y / d3.y, n3.z / d3.z);
  return (rp + rs) * 0.5f;
}

V fresnel(const Lobe& l, float cosI) {
  if (l.fres == F_COND) return frConductor(std::abs(cosI), l.fr_eta, l.fr_k);
  if (l.fres == F_DIEL) return V(frDielectric(std::abs(cosI), l.etaA, l.etaB));
  return V(1.0f);
}

V reflect(V wo, V n) { return -wo + n * (2 * dot(wo, n)); }  // bsdf.h:101-103
bool refract(V wi, V n, float eta, V* wt) {                 // bsdf.h:105-115
  float cosI = dot(n, wi);
  float s2i = std::max(float(0), float(1 - cosI * cosI));
  float s2t = eta * eta * s2i;
  if (s2t >= 1) return false;
  float cosTt = std::sqrt(1 - s2t);
  *wt = (-wi) * eta + n * (eta * cosI - cosTt);
  return true;
}

// src/bsdf/microfacet.cpp:4-40 (GGX); Beckmann from Walter et al. 2007.
float mfD(const Lobe& l, V wh) {
  float t2 = tan2T(wh);
  if (std::isinf(t2)) return 0;
  float c4 = cos2T(wh) * cos2T(wh);
  float a2 = l.alpha * l.alpha;
  if (l.beckmann) return std::exp(-t2 / a2) / (kPi * a2 * c4);
  float e = t2 / a2;
  return 1 / (kPi * a2 * c4 * (1 + e) * (1 + e));
}
float mfLambda(const Lobe& l, V w) {
  float at = std::abs(tanT(w));
  if (std::isinf(at)) return 0.;
  if (l.beckmann) {
    float a = 1 / (l.alpha * at);
    if (a >= 1.6f) return 0;
    return (1 - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
  }
  float a2t2 = (l.alpha * at) * (l.alpha * at);
  return (-1 + std::sqrt(1.f + a2t2)) / 2;
}
float mfG(const Lobe& l, V wi, V wo) { return 1 / (1 + mfLambda(l, wi) + mfLambda(l, wo)); }
V mfSampleWh(const Lobe& l, V wo, float u0, float u1) {
  float tan2;
  if (l.beckmann) {
    float ls = std::log(1 - u0);
    if (std::isinf(ls)) ls = 0;
    tan2 = -l.alpha * l.alpha * ls;
  } else {
    tan2 = l.alpha * l.alpha * u0 / (1.0f - u0);
  }
  float c = 1 / std::sqrt(1 + tan2);
  float s = std::sqrt(std::max((float)0., (float)1. - c * c));
  float phi = (2 * kPi) * u1;
  V wh(s * std::cos(phi), s * std::sin(phi), c);
  if (!sameHemi(wo, wh)) wh = -wh;
  return wh;
}
float mfPdf(const Lobe& l, V wh) { return mfD(l, wh) * absCosT(wh); }

V lobeF(const Lobe& l, V wi, V wo) {
  switch (l.kind) {
    case LAMBERT:  // src/bsdf/lambert.cpp:5-8
      return l.c * kInvPi;
    case OREN: {  // src/bsdf/orennayar.cpp:13-37
      float si = sinT(wi), so = sinT(wo);
      float cosTerm = 0;
      if (si > 1e-4 && so > 1e-4) {
        float d = cosP(wi) * cosP(wo) + sinP(wi) * sinP(wo);
        cosTerm = std::max((float)0, d);
      }
      float sa, tb;
      if (absCosT(wi) > absCosT(wo)) {
        sa = so;
        tb = si / absCosT(wi);
      } else {
        sa = si;
        tb = so / absCosT(wo);
      }
      return (l.c * kInvPi) * (l.A + l.B * cosTerm * sa * tb);
    }
    case MF_R: {  // src/bsdf/microfacet.cpp:55-65 (G evaluated at (wi, wi))
      float co = absCosT(wo), ci = absCosT(wi);
      if (ci == 0 || co == 0) return V(0.f);
      V wh = wi + wo;
      if (wh.x == 0 && wh.y == 0 && wh.z == 0) return V(0.f);
      wh = normalize(wh);
      V F = fresnel(l, dot(wi, wh));
      return sdiv(mul((l.c * mfD(l, wh)) * mfG(l, wi, wi), F), 4 * ci * co);
    }
    case MF_T: {  // src/bsdf/microfacet.cpp:87-108
      if (sameHemi(wi, wo)) return V(0.f);
      float co = cosT(wo), ci = cosT(wi);
      if (ci == 0 || co == 0) return V(0.f);
      float eta = cosT(wo) > 0 ? (l.etaB / l.etaA) : (l.etaA / l.etaB);
      V wh = normalize(wo + wi * eta);
      if (wh.z < 0) wh = -wh;
      float F = frDielectric(std::abs(dot(wo, wh)), l.etaA, l.etaB);
      float sd = dot(wo, wh) + eta * dot(wi, wh);
      float factor = l.photon ? 1 : 1 / eta;  // microfacet.cpp:102
      return mul(V(1.f - F), l.c) * std::abs(mfD(l, wh) * mfG(l, wi, wo) * eta * eta * absdot(wi, wh) *
                                             absdot(wo, wh) * factor * factor / (ci * co * sd * sd));
    }
    default:
      return V(0.f);
  }
}

float lobePdf(const Lobe& l, V wi, V wo) {
  switch (l.kind) {
    case LAMBERT:
    case OREN:  // src/core/bsdf.cpp:118-121
      return sameHemi(wi, wo) ? absCosT(wi) * kInvPi : 0;
    case MF_R: {  // src/bsdf/microfacet.cpp:67-73
      if (!sameHemi(wi, wo)) return 0;
      V wh = normalize(wi + wo);
      return mfPdf(l, wh) / (4 * dot(wo, wh));
    }
    case MF_T: {  // src/bsdf/microfacet.cpp:110-120
      if (sameHemi(wo, wi)) return 0;
      float eta = cosT(wo) > 0 ? (l.etaB / l.etaA) : (l.etaA / l.etaB);
      V wh = normalize(wo + wi * eta);
      float sd = dot(wo, wh) + eta * dot(wi, wh);
      float dwh = std::abs((eta * eta * dot(wi, wh)) / (sd * sd));
      return mfPdf(l, wh) * dwh;
    }
    default:
      return 0;
  }
}

V lobeSample(const Lobe& l, V wo, float u0, float u1, V* wi, float* pdf, int* st) {
  switch (l.kind) {
    case LAMBERT:
    case OREN:  // src/core/bsdf.cpp:109-116
      *wi = cosineSampleHemisphere(u0, u1);
      if (wo.z < 0) wi->z *= -1;
      *pdf = lobePdf(l, *wi, wo);
      return lobeF(l, *wi, wo);
    case MF_R: {  // src/bsdf/microfacet.cpp:42-53
      if (wo.z == 0) return V(0.f);
      V wh = mfSampleWh(l, wo, u0, u1);
      *wi = reflect(wo, wh);
      if (!sameHemi(*wi, wo)) return V(0.f);
      *pdf = mfPdf(l, wh) / (4 * dot(wo, wh));
      return lobeF(l, *wi, wo);
    }
    case MF_T: {  // src/bsdf/microfacet.cpp:76-85: pdf is never written
      if (wo.z == 0) return V(0.f);
      V wh = mfSampleWh(l, wo, u0, u1);
      float eta = cosT(wo) > 0 ? (l.etaA / l.etaB) : (l.etaB / l.etaA);
      if (!refract(wo, wh, eta, wi)) return V(0.f);
      return lobeF(l, *wi, wo);
    }
    case SPEC_R:  // src/bsdf/specular.cpp:20-25
      *wi = V(-wo.x, -wo.y, wo.z);
      *pdf = 1;
      return sdiv(mul(fresnel(l, cosT(*wi)), l.c), absCosT(*wi));
    case SPEC_T: {  // src/bsdf/specular.cpp:4-18
      bool entering = cosT(wo) > 0;
      float ei = entering ? l.etaA : l.etaB, et = entering ? l.etaB : l.etaA;
      if (!refract(wo, faceforward(V(0, 0, 1), wo), ei / et, wi)) return V(0.f);
      *pdf = 1.0f;
      V ft = mul(l.c, V(1.0f) - V(frDielectric(std::abs(cosT(*wi)), l.etaA, l.etaB)));
      if (!l.photon) ft = mul(ft, V((ei * ei) / (et * et)));
      return sdiv(ft, absCosT(*wi));
    }
    case FRES_SPEC: {  // src/bsdf/specular.cpp:28-54
      float F = frDielectric(cosT(wo), l.etaA, l.etaB);
      if (u0 < F) {
        *wi = V(-wo.x, -wo.y, wo.z);
        *st = SPEC | REFL;
        *pdf = F;
        return sdiv(l.c * F, absCosT(*wi));
      }
      bool entering = cosT(wo) > 0;
      float ei = entering ? l.etaA : l.etaB, et = entering ? l.etaB : l.etaA;
      if (!refract(wo, faceforward(V(0, 0, 1), wo), ei / et, wi)) return V(0.f);
      V ft = l.c2 * (1 - F);
      if (!l.photon) ft = mul(ft, V((ei * ei) / (et * et)));
      *st = SPEC | TRANS;
      *pdf = 1 - F;
      return sdiv(ft, absCosT(*wi));
    }
  }
  return V(0.f);
}

struct Frame {
  V ng, ns, u, v;
  V toLocal(V w) const { return V(dot(w, u), dot(w, v), dot(w, ns)); }
  V toWorld(V w) const {
    return V(u.x * w.x + v.x * w.y + ns.x * w.z, u.y * w.x + v.y * w.y + ns.y * w.z,
             u.z * w.x + v.z * w.y + ns.z * w.z);
  }
};

inline bool matches(const Lobe& l, int t) { return (l.type & t) == l.type; }
int numMatching(const Mat& m, int t) {
  int n = 0;
  for (const Lobe& l : m.lobes) n += matches(l, t);
  return n;
}

// src/core/bsdf.cpp:16-28
V bsdfF(const Mat& m, const Frame& fr, V wi, V wo, int t) {
  V r(0.f);
  V swi = fr.toLocal(wi), swo = fr.toLocal(wo);
  for (const Lobe& l : m.lobes)
    if (matches(l, t)) r = r + lobeF(l, swi, swo);
  return r;
}

// src/core/bsdf.cpp:89-106
float bsdfPdf(const Mat& m, const Frame& fr, V wi, V wo, int t) {
  if (m.lobes.empty()) return 0;
  V swi = fr.toLocal(wi), swo = fr.toLocal(wo);
  if (swo.z == 0) return 0;
  float pdf = 0;
  int n = 0;
  for (const Lobe& l : m.lobes)
    if (matches(l, t)) {
      ++n;
      pdf += lobePdf(l, swi, swo);
    }
  return n > 0 ? pdf / n : 0.f;
}

// src/core/bsdf.cpp:30-87
V bsdfSample(const Mat& m, const Frame& fr, V wo, float r0, float r1, int t, V* wi, float* pdf, int* st) {
  int n = numMatching(m, t);
  *pdf = 0;
  *st = 0;
  if (n == 0) return V(0.f);
  int pos = std::min((int)std::floor(r0 * n), n - 1);
  int count = pos, sel = -1;
  for (size_t i = 0; i < m.lobes.size(); ++i)
    if (matches(m.lobes[i], t) && count-- == 0) {
      sel = (int)i;
      break;
    }
  const Lobe& b = m.lobes[sel];
  float nr0 = std::min(r0 * n - pos, kOneMinusEpsilon);
  V swi, swo = fr.toLocal(wo);
  if (swo.z == 0) return V(0.f);
  *pdf = 0;
  *st = b.type;
  V f = lobeSample(b, swo, nr0, r1, &swi, pdf, st);
  if (*pdf == 0) {
    *st = 0;
    return V(0.f);
  }
  *wi = fr.toWorld(swi);
  bool spec = (b.type & SPEC) != 0;
  if (!spec && n > 1)
    for (size_t i = 0; i < m.lobes.size(); ++i)
      if ((int)i != sel && matches(m.lobes[i], t)) *pdf += lobePdf(m.lobes[i], swi, swo);
  if (n > 1) *pdf /= n;
  if (!spec && n > 1) {
    bool refl = dot(*wi, fr.ng) * dot(wo, fr.ng) > 0;
    f = V(0.f);
    for (const Lobe& l : m.lobes) {
      bool hr = (l.type & REFL) != 0, ht = (l.type & TRANS) != 0;
      if (matches(l, t) && ((refl && hr) || (!refl && ht))) f = f + lobeF(l, swi, swo);
    }
  }
  return f;
}

// src/bsdf/microfacet.h:44-50
float roughnessToAlpha(float r) {
  r = std::max(r, (float)1e-3);
  float x = std::log(r);
  return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x + 0.000640711f * x * x * x * x;
}

Lobe mk(Kind k, int t) {
  Lobe l;
  l.kind = k;
  l.type = t;
  return l;
}

// Material::getBSDF (src/material/*.cpp)
Mat makeMat(const orion_material& m) {
  Mat r;
  int bk = m.distribution == ORION_DIST_BECKMANN;
  auto mf_r = [&](V c, float alpha) {
    Lobe l = mk(MF_R, REFL | GLOSSY);
    l.c = c;
    l.alpha = alpha;
    l.beckmann = bk;
    return l;
  };
  switch (m.type) {
    case ORION_MAT_MATTE: {  // matte.cpp:9-21
      V kd = clamp0(ld(m.Kd));
      float sig = m.has_sigma ? clampf(m.sigma, 0.0f, kInfinity) : 0.f;
      if (!black(kd)) {
        if (sig == 0) {
          Lobe l = mk(LAMBERT, REFL | DIFF);
          l.c = kd;
          r.lobes.push_back(l);
        } else {  // orennayar.cpp:5-12
          Lobe l = mk(OREN, REFL | DIFF);
          l.c = kd;
          float s = sig * static_cast<float>(0.01745329251994329576923690768489);
          float s2 = s * s;
          l.A = 1.f - (s2 / (2.f * (s2 + 0.33f)));
          l.B = 0.45f * s2 / (s2 + 0.09f);
          r.lobes.push_back(l);
        }
      }
      break;
    }
    case ORION_MAT_METAL: {  // metal.cpp:8-17
      Lobe l = mf_r(V(1.0f), roughnessToAlpha(m.roughness));
      l.fres = F_COND;
      l.fr_eta = ld(m.eta_rgb);
      l.fr_k = ld(m.k);
      r.lobes.push_back(l);
      break;
    }
    case ORION_MAT_MIRROR: {  // mirror.cpp:6-13
      V kr = clamp0(ld(m.Kr));
      if (!black(kr)) {
        Lobe l = mk(SPEC_R, REFL | SPEC);
        l.c = kr;
        r.lobes.push_back(l);
      }
      break;
    }
    case ORION_MAT_GLASS: {  // glass.cpp:9-37
      V R = ld(m.Kr), T = ld(m.Kt);
      if (black(R) && black(T)) break;
      float alpha = roughnessToAlpha(m.roughness);
      if (m.roughness == 0) {
        Lobe l = mk(FRES_SPEC, REFL | TRANS | SPEC);
        l.c = R;
        l.c2 = T;
        l.etaA = 1.0f;
        l.etaB = m.eta;
        r.lobes.push_back(l);
      } else {
        if (!black(R)) {
          Lobe l = mf_r(R, alpha);
          l.fres = F_DIEL;
          l.etaA = 1.0f;
          l.etaB = m.eta;
          r.lobes.push_back(l);
        }
        if (!black(T)) {
          Lobe l = mk(MF_T, TRANS | GLOSSY);
          l.c = T;
          l.alpha = alpha;
          l.beckmann = bk;
          l.etaA = 1.0f;
          l.etaB = m.eta;
          r.lobes.push_back(l);
        }
      }
      break;
    }
    case ORION_MAT_PLASTIC: {  // plastic.cpp:8-24
      V kd = clamp0(ld(m.Kd));
      if (!black(kd)) {
        Lobe l = mk(LAMBERT, REFL | DIFF);
        l.c = kd;
        r.lobes.push_back(l);
      }
      V ks = clamp0(ld(m.Ks));
      if (!black(ks)) {
        Lobe l = mf_r(ks, roughnessToAlpha(m.roughness));
        l.fres = F_DIEL;
        l.etaA = 1.5f;
        l.etaB = 1.0f;
        r.lobes.push_back(l);
      }
      break;
    }
    case ORION_MAT_UBER: {  // uber.cpp:9-42
      V op = ld(m.opacity);
      float e = m.eta;
      V t = clamp0(V(1.0f) - op);
      if (!black(t)) {
        Lobe l = mk(SPEC_T, TRANS | SPEC);
        l.c = t;
        r.lobes.push_back(l);
      }
      V kd = mul(op, clamp0(ld(m.Kd)));
      if (!black(kd)) {
        Lobe l = mk(LAMBERT, REFL | DIFF);
        l.c = kd;
        r.lobes.push_back(l);
      }
      V ks = mul(op, clamp0(ld(m.Ks)));
      if (!black(ks)) {
        Lobe l = mf_r(ks, roughnessToAlpha(m.roughness));
        l.fres = F_DIEL;
        l.etaA = 1.0f;
        l.etaB = e;
        r.lobes.push_back(l);
      }
      V kr = mul(op, clamp0(ld(m.Kr)));
      if (!black(kr)) {
        Lobe l = mk(SPEC_R, REFL | SPEC);
        l.c = kr;
        l.fres = F_DIEL;
        l.etaA = 1.0f;
        l.etaB = e;
        r.lobes.push_back(l);
      }
      V kt = mul(op, clamp0(ld(m.Kt)));
      if (!black(kt)) {
        Lobe l = mk(SPEC_T, TRANS | SPEC);
        l.c = kt;
        l.etaA = 1.f;
        l.etaB = e;
        r.lobes.push_back(l);
      }
      break;
    }
  }
  return r;
}

// ------------------------------------------------------------------ scene

// findInterval (geometry.h:877-889) over a cdf of `size` entries.
int findIntervalCdf(const float* cdf, int size, float u) {
  int first = 0, len = size;
  while (len > 0) {
    int half = len >> 1, mid = first + half;
    if (cdf[mid] <= u) {
      first = mid + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  return std::max(0, std::min(first - 1, size - 2));
}

// Distribution1D (sampling.h:71-110).
struct Distribution1D {
  std::vector<float> func, cdf;
  float funcInt = 0;
  Distribution1D(const float* f, int n) : func(f, f + n), cdf(n + 1) {
    cdf[0] = 0;
    for (int i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + func[i - 1] / n;
    funcInt = cdf[n];
    if (funcInt == 0)
      for (int i = 1; i < n + 1; ++i) cdf[i] = float(i) / float(n);
    else
      for (int i = 1; i < n + 1; ++i) cdf[i] /= funcInt;
  }
  int count() const { return (int)func.size(); }
  float sampleContinuous(float u, float* pdf, int* off) const {
    int offset = findIntervalCdf(cdf.data(), (int)cdf.size(), u);
    if (off) *off = offset;
    float du = u - cdf[offset];
    if ((cdf[offset + 1] - cdf[offset]) > 0) du /= (cdf[offset + 1] - cdf[offset]);
    if (pdf) *pdf = (funcInt > 0) ? func[offset] / funcInt : 0;
    return (offset + du) / count();
  }
};

// Envmap with an image (envmap.cpp:9-44): texels times L, ImageTexture
// lookups with the default wrap filter (texture.cpp:3-27), Distribution2D
// (sampling.h:127-151, sampling.cpp:63-76) over intensity x sin(theta).
struct EnvImage {
  int w = 0, h = 0;
  std::vector<V> tex;
  std::vector<std::unique_ptr<Distribution1D>> cond;
  std::unique_ptr<Distribution1D> marg;
  V ave{0.f};
  V sample(int x, int y) const {
    x = x >= 0 ? x % w : w - (-x) % w;
    y = y >= 0 ? y % h : h - (-y) % h;
    return tex[(size_t)y * w + x];
  }
  V sample(float u, float v) const { return sample((int)(u * w), (int)(v * h)); }
  void build(const orion_image& im, V L) {
    w = im.width;
    h = im.height;
    tex.resize((size_t)w * h);
    for (size_t i = 0; i < tex.size(); ++i) tex[i] = mul(V(im.rgb[3 * i], im.rgb[3 * i + 1], im.rgb[3 * i + 2]), L);
    std::vector<float> img((size_t)w * h);
    for (int j = 0; j < h; ++j) {
      float v = (j + 0.5f) / (float)h;
      float sinTheta = std::sin(kPi * v);
      for (int i = 0; i < w; ++i) {
        V sp = sample(i, j);
        img[i + (size_t)j * w] = intensity(sp) * sinTheta;
        ave = ave + sp;
      }
    }
    ave = V(ave.x / (w * h), ave.y / (w * h), ave.z / (w * h));
    for (int v = 0; v < h; ++v) cond.emplace_back(new Distribution1D(&img[(size_t)v * w], w));
    std::vector<float> mf;
    for (int v = 0; v < h; ++v) mf.push_back(cond[v]->funcInt);
    marg.reset(new Distribution1D(mf.data(), h));
  }
  void sampleContinuous(float u0, float u1, float* su, float* sv, float* pdf) const {
    float p0, p1;
    int v;
    *sv = marg->sampleContinuous(u1, &p1, &v);
    *su = cond[v]->sampleContinuous(u0, &p0, nullptr);
    *pdf = p0 * p1;
  }
  float pdf(float pu, float pv) const {
    int iu = std::max(0, std::min(int(pu * cond[0]->count()), cond[0]->count() - 1));
    int iv = std::max(0, std::min(int(pv * marg->count()), marg->count() - 1));
    return cond[iv]->func[iu] / marg->funcInt;
  }
};

struct Light {
  int type;
  int prim;
  V L, p, dir;
  float area = 0;
  float l2w[12], w2l[12];
  float cosTotal = 0, cosFalloff = 0;
  float envInt = 0;
  std::shared_ptr<EnvImage> image;  // image environment map, or null (constant map)
};

struct Isect {
  V p, ng, ns, u, v;
  int prim = -1;
  float t = 0;
  float uvx = 0, uvy = 0;  // texture coordinates (kernel.cpp:138-142)
};

// ImageTexture with the wrap filter (src/core/texture.cpp:8-29,
// src/texture/imagetexture.cpp:4-12).
struct Tex {
  int w = 0, h = 0;
  std::vector<float> rgb;
  V eval(float u, float v) const {
    int x = (int)(u * w), y = (int)(v * h);
    // _coordFilter, FILTER_WRAP; a negative multiple of the size wraps to the
    // size itself, which reads the texel that follows in memory; past the
    // last texel (undefined in the reference) the last texel is read.
    x = x >= 0 ? x % w : w - (int)((0u - (unsigned)x) % (unsigned)w);
    y = y >= 0 ? y % h : h - (int)((0u - (unsigned)y) % (unsigned)h);
    int64_t off = (int64_t)y * w + x;
    const int64_t last = (int64_t)w * h - 1;
    if (off > last) off = last;
    return ld(&rgb[3 * off]);
  }
};

struct Scene {
  oracle_bvh::BVH bvh;
  std::vector<float> pos, nrm;
  std::vector<int> matOf, lightOf;
  std::vector<Mat> mats;
  std::vector<Light> lights;
  std::vector<int> envs;
  std::vector<float> func, cdf;
  float funcInt = 0;
  float worldRadius = 0;
  V worldCenter{0.f};
  orion_camera cam;
  float tanHalf = 0, aspect = 1;
  int spp = 1, maxDepth = 5;
  // Image textures: per material its record and whether an input is an
  // image; per primitive its corner texture coordinates.
  std::vector<orion_material> matSrc;
  std::vector<char> textured;
  std::vector<Tex> images;
  std::vector<float> uv;

  // Material::getBSDF of material `mi` at the hit (textures evaluated there).
  Mat material(int mi, const Isect& it) const {
    orion_material m = matSrc[mi];
    float* dst[ORION_TEX_SLOTS] = {m.Kd, m.Ks, m.Kr, m.Kt, m.opacity, m.eta_rgb, m.k};
    for (int t = 0; t < ORION_TEX_SLOTS; ++t) {
      if (m.tex[t] == 0) continue;
      V c = images[m.tex[t] - 1].eval(it.uvx, it.uvy);
      dst[t][0] = c.x, dst[t][1] = c.y, dst[t][2] = c.z;
    }
    return makeMat(m);
  }

  // Scene::intersect -> EmbreeKernel::intersect post-hit (kernel.cpp:127-169)
  bool intersect(V o, V d, float tnear, float tfar, Isect* is) const {
    float oo[3] = {o.x, o.y, o.z}, dd[3] = {d.x, d.y, d.z};
    oracle_bvh::Hit h;
    if (!bvh.closest(oo, dd, tnear, tfar, &h)) return false;
    const float* q = &pos[9 * (size_t)h.prim];
    const float* n = &nrm[9 * (size_t)h.prim];
    V p0 = ld(q), p1 = ld(q + 3), p2 = ld(q + 6);
    float w = 1 - h.u - h.v;
    is->p = w * p0 + h.u * p1 + h.v * p2;
    is->ns = ld(n) * w + ld(n + 3) * h.u + ld(n + 6) * h.v;
    is->ng = normalize(cross(p1 - p0, p2 - p0));
    is->t = h.t;
    V su = normalize(p1 - p0);
    is->v = normalize(cross(is->ns, su));
    is->u = normalize(cross(is->v, is->ns));
    is->prim = h.prim;
    if (!uv.empty()) {
      const float* q2 = &uv[6 * (size_t)h.prim];
      is->uvx = w * q2[0] + h.u * q2[2] + h.v * q2[4];
      is->uvy = w * q2[1] + h.u * q2[3] + h.v * q2[5];
    }
    return true;
  }
  bool occluded(V o, V d, float tmax) const {  // ShadowTester::unoccluded, light.h:26-29 (closest hit)
    Isect is;
    return intersect(o, d, 0, tmax, &is);
  }
};

V mat3(const float* m, V v) {  // Transform applied to a vector (rows of a 3x4)
  return V(m[0] * v.x + m[1] * v.y + m[2] * v.z, m[4] * v.x + m[5] * v.y + m[6] * v.z,
           m[8] * v.x + m[9] * v.y + m[10] * v.z);
}

// sphericalTheta / sphericalPhi (sampling.h:61-69)
float sphericalTheta(V v) { return std::acos(clampf(v.z, -1.0f, 1.0f)); }
float sphericalPhi(V v) {
  float p = std::atan2(v.y, v.x);
  return (p < 0) ? (p + 2 * kPi) : p;
}

// Envmap::Le (envmap.cpp:44-49)
V envLe(const Light& L, V d) {
  if (!L.image) return L.L;
  V w = normalize(mat3(L.w2l, d));
  return L.image->sample(sphericalPhi(w) * kInv2Pi, sphericalTheta(w) * kInvPi);
}

// Distribution1D::sampleDiscrete with findInterval (sampling.h:113-121, geometry.h:877-889)
int sampleDiscrete(const Scene& s, float u, float* pdf) {
  int size = (int)s.cdf.size(), first = 0, len = size;
  while (len > 0) {
    int half = len >> 1, mid = first + half;
    if (s.cdf[mid] <= u) {
      first = mid + 1;
      len -= half + 1;
    } else {
      len = half;
    }
  }
  int off = std::max(0, std::min(first - 1, size - 2));
  int n = (int)s.func.size();
  *pdf = s.funcInt > 0 ? s.func[off] / (s.funcInt * n) : 0;
  return off;
}

struct LS {
  V Li, wi, pLight;
  float pdf = 0;
};

// Light::sample_Li (src/light/*.cpp)
LS sampleLi(const Scene& s, const Light& L, const Isect& it, float u0, float u1) {
  LS r;
  r.pLight = it.p;
  switch (L.type) {
    case ORION_LIGHT_AREA: {  // diffuse.cpp:12-26, triangle.cpp:85-121
      const float* q = &s.pos[9 * (size_t)L.prim];
      const float* n = &s.nrm[9 * (size_t)L.prim];
      float su0 = std::sqrt(u0);
      float b0 = 1 - su0, b1 = u1 * su0;
      V p0 = ld(q), p1 = ld(q + 3), p2 = ld(q + 6);
      V p = b0 * p0 + b1 * p1 + (1 - b0 - b1) * p2;
      V ng = normalize(cross(p1 - p0, p2 - p0));
      V ns = ld(n) * b0 + ld(n + 3) * b1 + ld(n + 6) * (1.0f - b0 - b1);
      ng = faceforward(ng, ns);
      float pdf = 1.0f / L.area;
      V w = p - it.p;
      if (len_sq(w) == 0)
        pdf = 0;
      else {
        w = normalize(w);
        pdf *= len_sq(it.p - p) / absdot(ng, -w);
        if (std::isinf(pdf)) pdf = 0;
      }
      r.pLight = p;
      if (pdf == 0 || len_sq(p - it.p) == 0) {
        r.pdf = 0;
        return r;
      }
      r.wi = normalize(p - it.p);
      r.pdf = pdf;
      r.Li = dot(ng, -r.wi) > 0 ? L.L : V(0.f);
      return r;
    }
    case ORION_LIGHT_POINT:  // point.cpp:10-19
      r.wi = normalize(L.p - it.p);
      r.pdf = 1.0f;
      r.pLight = L.p;
      r.Li = sdiv(L.L, len_sq(L.p - it.p));
      return r;
    case ORION_LIGHT_SPOT: {  // spot.cpp:10-29
      r.wi = normalize(L.p - it.p);
      r.pdf = 1.f;
      r.pLight = L.p;
      V wl = normalize(mat3(L.w2l, -r.wi));
      float c = wl.z, f;
      if (c < L.cosTotal)
        f = 0;
      else if (c > L.cosFalloff)
        f = 1;
      else {
        float d = (c - L.cosTotal) / (L.cosFalloff - L.cosTotal);
        f = (d * d) * (d * d);
      }
      r.Li = sdiv(L.L * f, len_sq(L.p - it.p));
      return r;
    }
    case ORION_LIGHT_DISTANT:  // distant.cpp:15-25
      r.wi = L.dir;
      r.pdf = 1;
      r.pLight = it.p + L.dir * (2 * s.worldRadius);
      r.Li = L.L;
      return r;
    case ORION_LIGHT_ENV: {  // envmap.cpp:50-68
      if (L.image) {
        float su, sv, mapPdf;
        L.image->sampleContinuous(u0, u1, &su, &sv, &mapPdf);
        if (mapPdf == 0) return r;
        float theta = sv * kPi, phi = su * 2 * kPi;
        float ct = std::cos(theta), st = std::sin(theta), sp = std::sin(phi), cp = std::cos(phi);
        r.wi = mat3(L.l2w, V(st * cp, st * sp, ct));
        r.pdf = mapPdf / (2 * kPi * kPi * st);
        if (st == 0) r.pdf = 0;
        r.pLight = it.p + r.wi * (2 * s.worldRadius);
        r.Li = L.image->sample(su, sv);
        return r;
      }
      // constant map (1x1 distribution: uv = u, mapPdf = 1)
      if (L.envInt == 0) return r;
      float theta = u1 * kPi, phi = u0 * 2 * kPi;
      float ct = std::cos(theta), st = std::sin(theta), sp = std::sin(phi), cp = std::cos(phi);
      r.wi = mat3(L.l2w, V(st * cp, st * sp, ct));
      r.pdf = 1 / (2 * kPi * kPi * st);
      if (st == 0) r.pdf = 0;
      r.pLight = it.p + r.wi * (2 * s.worldRadius);
      r.Li = L.L;
      return r;
    }
  }
  return r;
}

bool isDelta(int type) { return type == ORION_LIGHT_POINT || type == ORION_LIGHT_SPOT || type == ORION_LIGHT_DISTANT; }

constexpr int NONSPEC = ALL & ~SPEC;

// estimateDirect (src/core/integrator.cpp:29-90)
V estimateDirect(const Scene& s, V rayD, const Isect& it, const Mat& m, const Frame& fr, float bu0, float bu1,
                 const Light& L, int li, float lu0, float lu1, int64_t* rays) {
  V Ld(0.f);
  V wo = normalize(-rayD);
  LS ls = sampleLi(s, L, it, lu0, lu1);
  float bsdfPdfv = 0;
  if (ls.pdf > 0 && !black(ls.Li)) {
    V f = bsdfF(m, fr, ls.wi, wo, NONSPEC) * absdot(ls.wi, it.ns);
    bsdfPdfv = bsdfPdf(m, fr, ls.wi, wo, NONSPEC);
    if (!black(f)) {
      V so = offsetRayOrigin(it.p, it.ng, ls.pLight - it.p);  // Intersection::spawnRay(Intersection), intersection.h:40-44
      ++*rays;
      V Li = ls.Li;
      if (s.occluded(so, ls.pLight - so, 1 - kShadowEpsilon)) Li = V(0.f);
      if (!black(Li)) {
        if (isDelta(L.type))
          Ld = Ld + sdiv(mul(f, Li), ls.pdf);
        else
          Ld = Ld + sdiv(mul(f, Li) * powerHeuristic(ls.pdf, bsdfPdfv), ls.pdf);
      }
    }
  }
  if (!isDelta(L.type)) {
    V wi;
    int st;
    V f = bsdfSample(m, fr, wo, bu0, bu1, NONSPEC, &wi, &bsdfPdfv, &st);
    f = f * absdot(wi, it.ns);
    if (!black(f) && bsdfPdfv > 0) {
      V ro = offsetRayOrigin(it.p, it.ng, wi);
      float lightPdf;
      Isect in;
      bool hit;
      if (L.type == ORION_LIGHT_AREA) {  // Triangle::pdf, triangle.cpp:123-135 (the same ray is traced twice there)
        ++*rays;
        hit = s.intersect(ro, wi, 0, kInfinity, &in);
        if (!hit || in.prim != L.prim) return Ld;
        lightPdf = len_sq(it.p - in.p) / (absdot(in.ng, -wi) * L.area);
        if (std::isinf(lightPdf)) lightPdf = 0;
      } else {  // Envmap::pdf_Li (envmap.cpp:70-80)
        // v = theta / (2 pi) and no early return at sin(theta) == 0, as written there.
        V w = mat3(L.w2l, wi);
        float theta = std::acos(clampf(w.z, -1.0f, 1.0f));
        float mapPdf = L.image ? L.image->pdf(sphericalPhi(w) * kInv2Pi, theta * kInv2Pi) : 1.0f;
        lightPdf = mapPdf / (2 * kPi * kPi * std::sin(theta));
      }
      if (lightPdf == 0) return Ld;
      float weight = powerHeuristic(bsdfPdfv, lightPdf);
      ++*rays;
      hit = s.intersect(ro, wi, 0, kInfinity, &in);
      V Li(0.f);
      if (hit) {
        if (s.lightOf[in.prim] == li) Li = dot(in.ng, -wi) > 0 ? L.L : V(0.f);
      } else {
        if (L.type == ORION_LIGHT_ENV) Li = envLe(L, wi);
      }
      if (!black(Li)) Ld = Ld + sdiv(mul(f, Li) * weight, bsdfPdfv);
    }
  }
  return Ld;
}

// Pinhole::generateRay (src/camera/pinhole.cpp:8-33)
// Sampler::next2() is Point2f(next(), next()) (src/core/sampler.h:29); its two
// calls are unsequenced and the compiled reference evaluates the second one
// first, so .x receives the later dimension. Every 2-D sample here follows that.
void cameraRay(const Scene& s, Sampler& smp, int i, int j, V* o, V* d) {
  float s0 = smp.next(), s1 = smp.next();
  float rx = (float)i + s1;
  float ry = (float)j + s0;
  float xx = (2 * rx / (float)s.cam.width - 1) * s.aspect * s.tanHalf;
  float yy = (1 - 2 * ry / (float)s.cam.height) * s.tanHalf;
  V dir = normalize(V(xx, yy, -1.0f));
  V org(0.f);
  if (s.cam.lens_radius > 0) {
    V target = org + dir * s.cam.focal_distance;
    float a = smp.next(), b = smp.next(), lx, ly;
    concentricSampleDisk(b, a, &lx, &ly);
    org = V(lx * s.cam.lens_radius, ly * s.cam.lens_radius, 0);
    dir = normalize(target - org);
  }
  const float* m = s.cam.c2w;
  float xp = m[0] * org.x + m[1] * org.y + m[2] * org.z + m[3];
  float yp = m[4] * org.x + m[5] * org.y + m[6] * org.z + m[7];
  float zp = m[8] * org.x + m[9] * org.y + m[10] * org.z + m[11];
  float wp = m[12] * org.x + m[13] * org.y + m[14] * org.z + m[15];
  if (wp == 1)
    *o = V(xp, yp, zp);
  else {
    float inv = 1.f / wp;
    *o = V(inv * xp, inv * yp, inv * zp);
  }
  *d = V(m[0] * dir.x + m[1] * dir.y + m[2] * dir.z, m[4] * dir.x + m[5] * dir.y + m[6] * dir.z,
         m[8] * dir.x + m[9] * dir.y + m[10] * dir.z);
}

// PathTracing::Li (src/integrator/path.cpp:50-99) with the roulette depth as a parameter (3 there).
V Li(const Scene& s, V ro, V rd, Sampler& smp, int maxDepth, int rrDepth, int64_t* rays) {
  V L(0.f), beta(1.0f);
  bool specular = false;
  for (int bounces = 0;; ++bounces) {
    Isect it;
    ++*rays;
    bool found = s.intersect(ro, rd, 0, kInfinity, &it);
    if (bounces == 0 || specular) {
      if (found) {
        int li = s.lightOf[it.prim];
        if (li >= 0 && dot(it.ng, -rd) > 0) L = L + mul(beta, s.lights[li].L);
      } else {
        for (int e : s.envs) L = L + mul(beta, envLe(s.lights[e], rd));
      }
    }
    if (!found || bounces >= maxDepth) break;
    const int mi = s.matOf[it.prim];
    Mat tm;
    if (s.textured[mi]) tm = s.material(mi, it);
    const Mat& m = s.textured[mi] ? tm : s.mats[mi];
    Frame fr{it.ng, it.ns, it.u, it.v};
    if (numMatching(m, NONSPEC) > 0 && !s.lights.empty()) {  // uniformSampleOneLight, integrator.cpp:8-27
      float sel;
      int li = sampleDiscrete(s, smp.next(), &sel);
      if (sel != 0) {
        float a = smp.next(), b = smp.next(), c = smp.next(), d = smp.next();
        V ld = estimateDirect(s, rd, it, m, fr, d, c, s.lights[li], li, b, a, rays);
        L = L + mul(beta, sdiv(ld, sel));
      }
    }
    V wo = -rd, wi;
    float pdf;
    int st;
    float u0 = smp.next(), u1 = smp.next();
    V f = bsdfSample(m, fr, wo, u1, u0, ALL, &wi, &pdf, &st);
    if (black(f) || pdf == 0) break;
    beta = mul(beta, sdiv(f * absdot(wi, it.ns), pdf));
    specular = (st & SPEC) != 0;
    ro = offsetRayOrigin(it.p, it.ng, wi);  // Intersection::spawnRay(Vector3f), intersection.h:45-48
    rd = wi;
    if (bounces > rrDepth) {
      float q = std::max((float)0.05, 1 - maxc(beta));
      if (smp.next() < q) break;
      beta = sdiv(beta, 1 - q);
    }
  }
  return L;
}

// ------------------------------------------------------------------ SPPM
// SPPM::render (src/integrator/sppm.cpp:58-322), restated one thread at a
// time: the photon contributions add in photon order and each grid cell
// lists its visible points most recent first, as the reference's
// single-threaded run builds and walks them.

// coordinateSystem (src/core/geometry.h:902-909)
inline void coordinateSystem(V z, V* x, V* y) {
  if (std::abs(z.x) > std::abs(z.y))
    *y = vdiv(V(-z.z, 0, z.x), std::sqrt(z.x * z.x + z.z * z.z));
  else
    *y = vdiv(V(0, z.z, -z.y), std::sqrt(z.y * z.y + z.z * z.z));
  *x = cross(*y, z);
}

// Material at a hit in the given transport mode (Intersection::calculateBSDF).
Mat materialAt(const Scene& s, const Isect& it, bool photon) {
  const int mi = s.matOf[it.prim];
  Mat m = s.textured[mi] ? s.material(mi, it) : s.mats[mi];
  if (photon)
    for (Lobe& l : m.lobes) l.photon = true;
  return m;
}

// Light::sample_Le (src/light/{diffuse,point,spot,distant,envmap}.cpp);
// rand0 / rand1 as the reference's Point2f (x = the later dimension).
V sampleLe(const Scene& s, const Light& L, float r0x, float r0y, float r1x, float r1y, V* ro, V* rd, V* nLight,
           float* pdfPos, float* pdfDir) {
  *pdfPos = *pdfDir = 0;
  switch (L.type) {
    case ORION_LIGHT_AREA: {  // diffuse.cpp:32-44, triangle.cpp:85-106
      const float* q = &s.pos[9 * (size_t)L.prim];
      const float* n = &s.nrm[9 * (size_t)L.prim];
      float su0 = std::sqrt(r0x);
      float b0 = 1 - su0, b1 = r0y * su0;
      V p0 = ld(q), p1 = ld(q + 3), p2 = ld(q + 6);
      V p = b0 * p0 + b1 * p1 + (1 - b0 - b1) * p2;
      V ng = normalize(cross(p1 - p0, p2 - p0));
      V ns = ld(n) * b0 + ld(n + 3) * b1 + ld(n + 6) * (1.0f - b0 - b1);
      ng = faceforward(ng, ns);
      *pdfPos = 1.0f / L.area;
      *nLight = ng;
      V w = cosineSampleHemisphere(r1x, r1y);
      *pdfDir = w.z * kInvPi;
      V x, y;
      coordinateSystem(ng, &x, &y);
      w = w.x * x + w.y * y + w.z * ng;
      *ro = offsetRayOrigin(p, ng, w);
      *rd = w;
      return dot(ng, w) > 0 ? L.L : V(0.f);
    }
    case ORION_LIGHT_POINT: {  // point.cpp:20-27
      float z = 1 - 2 * r0x;
      float r = std::sqrt(std::max((float)0, (float)1 - z * z));
      float phi = 2 * kPi * r0y;
      *ro = L.p;
      *rd = V(r * std::cos(phi), r * std::sin(phi), z);
      *nLight = *rd;
      *pdfPos = 1;
      *pdfDir = kInv4Pi;
      return L.L;
    }
    case ORION_LIGHT_SPOT: {  // spot.cpp:30-38
      float cosTheta = ((float)1 - r0x) + r0x * L.cosTotal;
      float sinTheta = std::sqrt((float)1 - cosTheta * cosTheta);
      float phi = r0y * 2 * kPi;
      V w(std::cos(phi) * sinTheta, std::sin(phi) * sinTheta, cosTheta);
      *ro = L.p;
      *rd = mat3(L.l2w, w);
      *nLight = *rd;
      *pdfPos = 1;
      *pdfDir = 1 / (2 * kPi * (1 - L.cosTotal));
      V wl = normalize(mat3(L.w2l, *rd));
      float c = wl.z, f;
      if (c < L.cosTotal)
        f = 0;
      else if (c > L.cosFalloff)
        f = 1;
      else {
        float d = (c - L.cosTotal) / (L.cosFalloff - L.cosTotal);
        f = (d * d) * (d * d);
      }
      return L.L * f;
    }
    case ORION_LIGHT_DISTANT: {  // distant.cpp:28-41
      V v1, v2;
      coordinateSystem(L.dir, &v1, &v2);
      float cx, cy;
      concentricSampleDisk(r0x, r0y, &cx, &cy);
      V pDisk = s.worldCenter + s.worldRadius * (cx * v1 + cy * v2);
      *ro = pDisk + s.worldRadius * L.dir;
      *rd = -L.dir;
      *nLight = *rd;
      *pdfPos = 1 / (kPi * s.worldRadius * s.worldRadius);
      *pdfDir = 1;
      return L.L;
    }
    case ORION_LIGHT_ENV: {  // envmap.cpp:82-104
      float su, sv, mapPdf;
      if (L.image) {
        L.image->sampleContinuous(r0x, r0y, &su, &sv, &mapPdf);
      } else {  // 1x1 distribution: uv = u, mapPdf = 1 (0 for a black map)
        su = r0x, sv = r0y;
        mapPdf = L.envInt == 0 ? 0.f : 1.f;
      }
      if (mapPdf == 0) return V(0.f);
      float theta = sv * kPi, phi = su * 2.f * kPi;
      float ct = std::cos(theta), st = std::sin(theta), sp = std::sin(phi), cp = std::cos(phi);
      V d = -mat3(L.l2w, V(st * cp, st * sp, ct));
      *nLight = d;
      V v1, v2;
      coordinateSystem(-d, &v1, &v2);
      float cx, cy;
      concentricSampleDisk(r1x, r1y, &cx, &cy);
      V pDisk = s.worldCenter + s.worldRadius * (cx * v1 + cy * v2);
      *ro = pDisk + s.worldRadius * -d;
      *rd = d;
      *pdfDir = st == 0 ? 0 : mapPdf / (2 * kPi * kPi * st);
      *pdfPos = 1 / (kPi * s.worldRadius * s.worldRadius);
      return L.image ? L.image->sample(su, sv) : L.L;
    }
  }
  return V(0.f);
}

struct SppmPixel {
  float radius = 0;
  V Ld{0.f};
  bool vp = false;  // a visible point this iteration (the reference: vp.beta non-black)
  V vpP{0.f}, vpWo{0.f}, vpBeta{0.f};
  Mat vpMat;
  Frame vpFr;
  V phi{0.f};
  int M = 0;
  float N = 0;
  V tau{0.f};
};

struct SppmGrid {
  V lo{kInfinity}, hi{-kInfinity};  // Bounds3f(): pMin = max, pMax = lowest
  int res[3] = {1, 1, 1};
  // offset() then the truncated cell index, clamped (sppm.cpp:41-51)
  bool toGrid(V p, int* c) const {
    V o = p - lo;
    if (hi.x > lo.x) o.x = o.x / (hi.x - lo.x);
    if (hi.y > lo.y) o.y = o.y / (hi.y - lo.y);
    if (hi.z > lo.z) o.z = o.z / (hi.z - lo.z);
    float pg[3] = {o.x, o.y, o.z};
    bool in = true;
    for (int i = 0; i < 3; ++i) {
      c[i] = (int)(res[i] * pg[i]);
      in &= c[i] >= 0 && c[i] < res[i];
      c[i] = std::min(std::max(c[i], 0), res[i] - 1);
    }
    return in;
  }
};

// hash (sppm.cpp:53-57), products taken modulo 2^32
inline unsigned sppmHash(const int* c, int size) {
  return (((unsigned)c[0] * 73856093u) ^ ((unsigned)c[1] * 19349663u) ^ ((unsigned)c[2] * 83492791u)) %
         (unsigned)size;
}

// film: W*H*3 sums of each iteration's estimate (RenderTarget::acumulate).
// threads == 1: the reference's single-thread order (the parity oracle);
// otherwise the camera and photon passes run on OpenMP threads with atomic
// photon sums, as the reference runs them (a timing baseline).
void renderSppm(const Scene& s, int nIter, int photons, float radius0, int maxDepth, float* film, int64_t* rays,
                int threads) {
  const int W = s.cam.width, H = s.cam.height, nPix = W * H;
  std::vector<SppmPixel> px(nPix);
  for (SppmPixel& p : px) p.radius = radius0;
  const int nL = (int)s.lights.size();
  const bool par = threads != 1;
  if (threads > 1) omp_set_num_threads(threads);
  int64_t nrays = 0;
  for (int iter = 0; iter < nIter; ++iter) {
    // Visible points (sppm.cpp:78-140).
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : nrays) if (par)
    for (int j = 0; j < H; ++j)
      for (int i = 0; i < W; ++i) {
        int64_t* rays = &nrays;
        Sampler smp{(uint64_t)iter * nPix + (uint64_t)W * j + i};
        V ro, rd;
        cameraRay(s, smp, i, j, &ro, &rd);
        V beta(1.0f);
        SppmPixel& pixel = px[(size_t)W * j + i];
        bool specular = false;
        for (int depth = 0; depth < maxDepth; ++depth) {
          Isect it;
          ++*rays;
          if (!s.intersect(ro, rd, 0, kInfinity, &it)) {
            for (int e : s.envs) pixel.Ld = pixel.Ld + mul(beta, envLe(s.lights[e], rd));
            break;
          }
          Mat m = materialAt(s, it, false);
          Frame fr{it.ng, it.ns, it.u, it.v};
          V wo = -rd;
          if (depth == 0 || specular) {
            int li = s.lightOf[it.prim];
            V Le = (li >= 0 && dot(it.ng, wo) > 0) ? s.lights[li].L : V(0.f);
            pixel.Ld = pixel.Ld + mul(beta, Le);
          }
          V direct(0.f);  // uniformSampleOneLight without a light distribution (integrator.cpp:8-27)
          if (nL > 0) {
            int li = std::min((int)(smp.next() * nL), nL - 1);
            float lightPdf = 1.0f / nL;
            float a = smp.next(), b = smp.next(), c = smp.next(), d = smp.next();
            direct = sdiv(estimateDirect(s, rd, it, m, fr, d, c, s.lights[li], li, b, a, rays), lightPdf);
          }
          pixel.Ld = pixel.Ld + mul(beta, direct);
          bool isDiffuse = numMatching(m, DIFF | REFL | TRANS) > 0;
          bool isGlossy = numMatching(m, GLOSSY | REFL | TRANS) > 0;
          if (isDiffuse || (isGlossy && depth == maxDepth - 1)) {
            pixel.vp = !black(beta);
            pixel.vpP = it.p;
            pixel.vpWo = wo;
            pixel.vpBeta = beta;
            pixel.vpMat = m;
            pixel.vpFr = fr;
            break;
          }
          if (depth < maxDepth - 1) {
            float u0 = smp.next(), u1 = smp.next();
            V wi;
            float pdf;
            int st;
            V f = bsdfSample(m, fr, wo, u1, u0, ALL, &wi, &pdf, &st);
            if (pdf == 0 || black(f)) break;
            specular = (st & SPEC) != 0;
            beta = mul(beta, sdiv(f * absdot(wi, it.ns), pdf));
            if (intensity(beta) < 0.25f) {
              float continueProb = std::min((float)1, intensity(beta));
              if (smp.next() > continueProb) break;
              beta = sdiv(beta, continueProb);
            }
            ro = offsetRayOrigin(it.p, it.ng, wi);
            rd = wi;
          }
        }
      }
    // Visible-point grid (sppm.cpp:142-195).
    SppmGrid g;
    float maxRadius = 0;
    bool any = false;
    for (const SppmPixel& p : px) {
      if (!p.vp) continue;
      any = true;
      V r(p.radius);
      V lo = p.vpP - r, hi = p.vpP + r;
      g.lo = V(std::min(g.lo.x, lo.x), std::min(g.lo.y, lo.y), std::min(g.lo.z, lo.z));
      g.hi = V(std::max(g.hi.x, hi.x), std::max(g.hi.y, hi.y), std::max(g.hi.z, hi.z));
      maxRadius = std::max(maxRadius, p.radius);
    }
    std::vector<std::vector<int>> cells(nPix);  // each list most recent first
    if (any) {
      V diag = g.hi - g.lo;
      float maxDiag = maxc(diag);
      int base = (int)(maxDiag / maxRadius);
      float dg[3] = {diag.x, diag.y, diag.z};
      for (int i = 0; i < 3; ++i) g.res[i] = std::max((int)(base * dg[i] / maxDiag), 1);
      for (int pi = 0; pi < nPix; ++pi) {
        const SppmPixel& p = px[pi];
        if (!p.vp) continue;
        V r(p.radius);
        int lo[3], hi[3];
        g.toGrid(p.vpP - r, lo);
        g.toGrid(p.vpP + r, hi);
        for (int z = lo[2]; z <= hi[2]; ++z)
          for (int y = lo[1]; y <= hi[1]; ++y)
            for (int x = lo[0]; x <= hi[0]; ++x) {
              int c[3] = {x, y, z};
              cells[sppmHash(c, nPix)].push_back(pi);
            }
      }
    }
    // Photons (sppm.cpp:197-270).
#pragma omp parallel for schedule(dynamic, 64) reduction(+ : nrays) if (par)
    for (int k = 0; k < photons; ++k) {
      if (!any) continue;
      int64_t* rays = &nrays;
      Sampler smp{(uint64_t)nIter * nPix + (uint64_t)iter * photons + k};
      float lightPdf;
      int ln = sampleDiscrete(s, smp.next(), &lightPdf);
      const Light& L = s.lights[ln];
      float a = smp.next(), b = smp.next(), c = smp.next(), d = smp.next();
      V ro, rd, nLight;
      float pdfPos, pdfDir;
      V Le = sampleLe(s, L, b, a, d, c, &ro, &rd, &nLight, &pdfPos, &pdfDir);
      if (pdfPos == 0 || pdfDir == 0 || black(Le)) continue;
      V beta = sdiv(absdot(nLight, rd) * Le, lightPdf * pdfPos * pdfDir);
      if (black(beta)) continue;
      for (int depth = 0; depth < maxDepth; ++depth) {
        Isect it;
        ++*rays;
        if (!s.intersect(ro, rd, 0, kInfinity, &it)) break;
        if (depth > 0) {
          int cell[3];
          if (g.toGrid(it.p, cell)) {
            const std::vector<int>& list = cells[sppmHash(cell, nPix)];
            for (size_t e = list.size(); e-- > 0;) {
              SppmPixel& p = px[list[e]];
              if (len_sq(p.vpP - it.p) > p.radius * p.radius) continue;
              V wi = -rd;
              V Phi = mul(beta, bsdfF(p.vpMat, p.vpFr, wi, p.vpWo, ALL));
              if (par) {
#pragma omp atomic
                p.phi.x += Phi.x;
#pragma omp atomic
                p.phi.y += Phi.y;
#pragma omp atomic
                p.phi.z += Phi.z;
#pragma omp atomic
                ++p.M;
              } else {
                p.phi = p.phi + Phi;
                ++p.M;
              }
            }
          }
        }
        Mat m = materialAt(s, it, true);
        Frame fr{it.ng, it.ns, it.u, it.v};
        V wo = -rd, wi;
        float pdf;
        int st;
        float u0 = smp.next(), u1 = smp.next();
        V f = bsdfSample(m, fr, wo, u1, u0, ALL, &wi, &pdf, &st);
        if (black(f) || pdf == 0) break;
        V bnew = sdiv(mul(beta, f) * absdot(wi, it.ns), pdf);
        float q = std::max((float)0, 1 - intensity(bnew) / intensity(beta));
        if (smp.next() < q) break;
        beta = sdiv(bnew, 1 - q);
        ro = offsetRayOrigin(it.p, it.ng, wi);
        rd = wi;
      }
    }
    // Pixel update (sppm.cpp:285-312).
    for (SppmPixel& p : px) {
      if (p.M > 0) {
        float gamma = (float)2 / (float)3;
        float Nnew = p.N + gamma * p.M;
        float Rnew = p.radius * std::sqrt(Nnew / (p.N + p.M));
        p.tau = sdiv((p.tau + mul(p.vpBeta, p.phi)) * (Rnew * Rnew), p.radius * p.radius);
        p.N = Nnew;
        p.radius = Rnew;
        p.M = 0;
        p.phi = V(0.f);
      }
      p.vp = false;
      p.vpBeta = V(0.f);
    }
    // Film (sppm.cpp:314-320).
    const uint64_t Np = (uint64_t)nIter * (uint64_t)photons;
    for (int pi = 0; pi < nPix; ++pi) {
      const SppmPixel& p = px[pi];
      V L = sdiv(p.Ld, (float)nIter);
      L = L + sdiv(p.tau, Np * kPi * p.radius * p.radius);
      film[3 * pi] += L.x;
      film[3 * pi + 1] += L.y;
      film[3 * pi + 2] += L.z;
    }
  }
  *rays += nrays;
}

// Scene setup: Scene::Scene + light preprocess + PathTracing::preprocess.
Scene* makeScene(const orion_scene_desc* d) {
  Scene* s = new Scene();
  size_t T = (size_t)d->num_prims;
  s->pos.assign(d->positions, d->positions + 9 * T);
  s->nrm.assign(d->normals, d->normals + 9 * T);
  s->matOf.assign(d->material_of_prim, d->material_of_prim + T);
  if (d->light_of_prim)
    s->lightOf.assign(d->light_of_prim, d->light_of_prim + T);
  else
    s->lightOf.assign(T, -1);
  s->bvh.build(s->pos.data(), (int)T);
  for (int i = 0; i < d->num_materials; ++i) {
    const orion_material& m = d->materials[i];
    s->mats.push_back(makeMat(m));
    s->matSrc.push_back(m);
    bool tex = false;
    for (int t = 0; t < ORION_TEX_SLOTS; ++t) {
      if (m.tex[t] < 0 || m.tex[t] > d->num_images) {
        delete s;
        return nullptr;
      }
      tex = tex || m.tex[t] != 0;
    }
    s->textured.push_back(tex);
    if (tex && s->uv.empty() && d->uvs) s->uv.assign(d->uvs, d->uvs + 6 * T);
  }
  for (int i = 0; i < d->num_images; ++i) {
    Tex t;
    t.w = d->images[i].width;
    t.h = d->images[i].height;
    t.rgb.assign(d->images[i].rgb, d->images[i].rgb + 3 * (size_t)t.w * t.h);
    s->images.push_back(std::move(t));
  }
  // worldbound + boundingSphere (kernel.cpp:44-50, geometry.h:551-554)
  float lo[3] = {kInfinity, kInfinity, kInfinity}, hi[3] = {-kInfinity, -kInfinity, -kInfinity};
  for (size_t i = 0; i < 9 * T; ++i) {
    int k = (int)(i % 3);
    lo[k] = std::min(lo[k], s->pos[i]);
    hi[k] = std::max(hi[k], s->pos[i]);
  }
  V c = (V(lo[0], lo[1], lo[2]) + V(hi[0], hi[1], hi[2])) * 0.5f;
  bool in = T > 0 && c.x >= lo[0] && c.x <= hi[0] && c.y >= lo[1] && c.y <= hi[1] && c.z >= lo[2] && c.z <= hi[2];
  s->worldRadius = in ? std::sqrt(len_sq(c - V(hi[0], hi[1], hi[2]))) : 0;
  s->worldCenter = c;
  const float r = s->worldRadius;
  std::vector<float> power;
  for (int i = 0; i < d->num_lights; ++i) {
    const orion_light& o = d->lights[i];
    Light L;
    L.type = o.type;
    L.prim = o.prim;
    L.L = ld(o.L);
    L.p = ld(o.p);
    L.dir = ld(o.dir);
    std::memcpy(L.l2w, o.l2w, sizeof(L.l2w));
    std::memcpy(L.w2l, o.w2l, sizeof(L.w2l));
    L.cosTotal = o.cos_total;
    L.cosFalloff = o.cos_falloff;
    V pw;
    switch (o.type) {
      case ORION_LIGHT_AREA: {  // diffuse.cpp:8-11, triangle.cpp:77-83
        const float* q = &s->pos[9 * (size_t)o.prim];
        L.area = 0.5f * std::sqrt(len_sq(cross(ld(q + 3) - ld(q), ld(q + 6) - ld(q))));
        pw = L.L * L.area * kPi;
        break;
      }
      case ORION_LIGHT_POINT:
        pw = L.L * (4 * kPi);
        break;
      case ORION_LIGHT_SPOT:
        pw = L.L * 2 * kPi * (1 - .5f * (L.cosFalloff + L.cosTotal));
        break;
      case ORION_LIGHT_DISTANT:
        pw = L.L * kPi * r * r;
        break;
      case ORION_LIGHT_ENV:
        L.envInt = intensity(L.L) * std::sin(kPi * 0.5f);
        if (o.image > 0) {
          L.image = std::make_shared<EnvImage>();
          L.image->build(d->images[o.image - 1], L.L);
          pw = L.image->ave * (kPi * r * r);
        } else {
          pw = L.L * (kPi * r * r);
        }
        s->envs.push_back(i);
        break;
    }
    s->lights.push_back(L);
    power.push_back(intensity(pw));
  }
  // Distribution1D (sampling.h:75-90)
  int n = (int)power.size();
  s->func = power;
  s->cdf.assign(n + 1, 0.f);
  for (int i = 1; i < n + 1; ++i) s->cdf[i] = s->cdf[i - 1] + power[i - 1] / n;
  s->funcInt = n ? s->cdf[n] : 0;
  if (n) {
    if (s->funcInt == 0)
      for (int i = 1; i < n + 1; ++i) s->cdf[i] = float(i) / float(n);
    else
      for (int i = 1; i < n + 1; ++i) s->cdf[i] /= s->funcInt;
  }
  s->cam = d->camera;
  s->tanHalf = std::tan(d->camera.fov * 0.5f * static_cast<float>(0.01745329251994329576923690768489));
  s->aspect = (float)d->camera.width / d->camera.height;
  s->spp = d->spp;
  s->maxDepth = d->max_depth;
  return s;
}

}  // namespace port

using namespace port;

extern "C" {

int port_load_sobol(const char* path) {
  FILE* f = std::fopen(path, "rb");
  if (!f) return -2;
  g_sobol.assign((size_t)1024 * 52, 0);
  size_t n = std::fread(g_sobol.data(), 4, g_sobol.size(), f);
  std::fclose(f);
  return n == g_sobol.size() ? 0 : -2;
}

int port_sobol(const uint64_t* index, const uint32_t* dim, int64_t n, float* out) {
  if (g_sobol.empty()) return -1;
  for (int64_t i = 0; i < n; ++i) out[i] = sobolSample(index[i], dim[i]);
  return 0;
}

int port_bsdf_eval(const orion_material* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                   const float* rnd, int32_t type, float* f, float* pdf, float* sf, float* swi, float* spdf,
                   int32_t* stype, int32_t* nbxdf) {
  Mat m = makeMat(*mat);
  for (int64_t i = 0; i < n; ++i) {
    const float* q = frame + 12 * i;
    Frame fr{ld(q), ld(q + 3), ld(q + 6), ld(q + 9)};
    V o = ld(wo + 3 * i), w = ld(wi + 3 * i);
    V fv = bsdfF(m, fr, w, o, type);
    f[3 * i] = fv.x;
    f[3 * i + 1] = fv.y;
    f[3 * i + 2] = fv.z;
    pdf[i] = bsdfPdf(m, fr, w, o, type);
    V sw(0.f);
    float p = 0;
    int st = 0;
    V s = bsdfSample(m, fr, o, rnd[2 * i], rnd[2 * i + 1], type, &sw, &p, &st);
    sf[3 * i] = s.x;
    sf[3 * i + 1] = s.y;
    sf[3 * i + 2] = s.z;
    swi[3 * i] = sw.x;
    swi[3 * i + 1] = sw.y;
    swi[3 * i + 2] = sw.z;
    spdf[i] = p;
    stype[i] = st;
    nbxdf[i] = numMatching(m, NONSPEC);
  }
  return 0;
}

void* port_scene_create(const orion_scene_desc* desc) { return makeScene(desc); }
void port_scene_free(void* h) { delete static_cast<Scene*>(h); }

int port_trace(void* h, int64_t n, const float* rays, int32_t brute_force, float* t, float* u, float* v,
               int32_t* prim) {
  const Scene& s = *static_cast<Scene*>(h);
#pragma omp parallel for schedule(dynamic, 256)
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 8 * i;
    oracle_bvh::Hit hh;
    bool ok = brute_force ? s.bvh.brute_force_closest(r, r + 3, r[6], r[7], &hh) : s.bvh.closest(r, r + 3, r[6], r[7], &hh);
    t[i] = ok ? hh.t : 0.f;
    u[i] = ok ? hh.u : 0.f;
    v[i] = ok ? hh.v : 0.f;
    prim[i] = ok ? hh.prim : -1;
  }
  return 0;
}

int port_camera_rays(void* h, int64_t n, const int64_t* index, float* rays) {
  const Scene& s = *static_cast<Scene*>(h);
  const int64_t wh = (int64_t)s.cam.width * s.cam.height;
  for (int64_t q = 0; q < n; ++q) {
    int64_t pix = index[q] % wh;
    Sampler smp{(uint64_t)index[q]};
    V o, d;
    cameraRay(s, smp, (int)(pix % s.cam.width), (int)(pix / s.cam.width), &o, &d);
    float* r = rays + 6 * q;
    r[0] = o.x, r[1] = o.y, r[2] = o.z, r[3] = d.x, r[4] = d.y, r[5] = d.z;
  }
  return 0;
}

// PathTracing::render (path.cpp:15-37): passes k in [k0, k0 + spp), OpenMP over
// rows, FP32 film sums in sample order. Only the `nrows` rows listed in `rows`
// (the CPU baseline renders a bounded sample of the image's rows); the film is
// the whole W x H x 3 image. Returns traced rays.
int64_t port_render_rows(void* h, int32_t spp, int64_t k0, int32_t max_depth, int32_t rr_depth, int32_t nrows,
                         const int32_t* rows, float* film, int32_t threads) {
  const Scene& s = *static_cast<Scene*>(h);
  const int W = s.cam.width, H = s.cam.height;
  for (int q = 0; q < nrows; ++q)
    if (rows[q] < 0 || rows[q] >= H) return -1;
  const int64_t wh = (int64_t)W * H;
  if (threads > 0) omp_set_num_threads(threads);
  int64_t rays = 0;
  for (int64_t k = k0; k < k0 + spp; ++k) {
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : rays)
    for (int q = 0; q < nrows; ++q)
      for (int i = 0, j = rows[q]; i < W; ++i) {
        Sampler smp{(uint64_t)(k * wh + (int64_t)j * W + i)};
        V o, d;
        cameraRay(s, smp, i, j, &o, &d);
        int64_t r = 0;
        V L = Li(s, o, d, smp, max_depth, rr_depth, &r);
        rays += r;
        float* px = film + 3 * ((size_t)j * W + i);
        px[0] += L.x;
        px[1] += L.y;
        px[2] += L.z;
      }
  }
  return rays;
}

// Rows [row0, row1) of port_render_rows.
int64_t port_render(void* h, int32_t spp, int64_t k0, int32_t max_depth, int32_t rr_depth, int32_t row0,
                    int32_t row1, float* film, int32_t threads) {
  const int H = static_cast<Scene*>(h)->cam.height;
  if (row1 > H) row1 = H;
  std::vector<int32_t> rows;
  for (int j = row0; j < row1; ++j) rows.push_back(j);
  return port_render_rows(h, spp, k0, max_depth, rr_depth, (int32_t)rows.size(), rows.data(), film, threads);
}

// FP64 per-pixel sums and sums of squares over passes [k0, k0 + spp).
int port_render_pixels(void* h, int64_t npix, const int32_t* pix, int64_t k0, int32_t spp, int32_t max_depth,
                       int32_t rr_depth, double* sum, double* sumsq, int32_t threads) {
  const Scene& s = *static_cast<Scene*>(h);
  const int64_t wh = (int64_t)s.cam.width * s.cam.height;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t q = 0; q < npix; ++q) {
    int i = pix[2 * q], j = pix[2 * q + 1];
    double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int64_t k = k0; k < k0 + spp; ++k) {
      Sampler smp{(uint64_t)(k * wh + (int64_t)j * s.cam.width + i)};
      V o, d;
      cameraRay(s, smp, i, j, &o, &d);
      int64_t r = 0;
      V L = Li(s, o, d, smp, max_depth, rr_depth, &r);
      double c[3] = {L.x, L.y, L.z};
      for (int ch = 0; ch < 3; ++ch) {
        a[ch] += c[ch];
        b[ch] += c[ch] * c[ch];
      }
    }
    for (int ch = 0; ch < 3; ++ch) {
      sum[3 * q + ch] = a[ch];
      sumsq[3 * q + ch] = b[ch];
    }
  }
  return 0;
}

// SPPM::render with the given parameters; film: W*H*3 floats, zeroed by the caller;
// threads 1 = the deterministic single-thread order, 0 = all cores.
int64_t port_render_sppm(void* h, int32_t iterations, int32_t photons, float radius, int32_t max_depth, float* film,
                         int32_t threads) {
  int64_t rays = 0;
  renderSppm(*static_cast<Scene*>(h), iterations, photons, radius, max_depth, film, &rays, threads);
  return rays;
}

int port_scene_info(void* h, int32_t* info) {
  const Scene& s = *static_cast<Scene*>(h);
  info[0] = s.cam.width;
  info[1] = s.cam.height;
  info[2] = s.spp;
  info[3] = s.maxDepth;
  info[4] = (int32_t)s.lights.size();
  return 0;
}

}  // extern "C"
