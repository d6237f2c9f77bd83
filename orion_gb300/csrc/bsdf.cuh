// Device BSDFs: the reference's BxDF set evaluated from a material's fixed
// lobe list (no per-hit allocation).
//
// Lobe semantics, quirks included, follow:
//   BSDF::f / sample_f / pdf            src/core/bsdf.cpp:16-106
//   default cosine sample_f / pdf       src/core/bsdf.cpp:109-121
//   frConductor / frDielectric          src/core/bsdf.cpp:124-170
//   Lambert, Oren-Nayar                 src/bsdf/lambert.cpp:5-8, src/bsdf/orennayar.cpp:5-37
//   GGX D / lambda / sample_wh          src/bsdf/microfacet.cpp:9-40
//   MicrofacetReflection (G(wi, wi))    src/bsdf/microfacet.cpp:42-74
//   MicrofacetTransmission (sample_f leaves pdf at 0) src/bsdf/microfacet.cpp:76-120
//   Specular R/T, FresnelSpecular       src/bsdf/specular.cpp:4-54
// Beckmann (not in the reference) follows the published isotropic Beckmann
// model with the rational Smith-lambda approximation (Walter et al. 2007, as
// in pbrt-v3) and the same roughness-to-alpha map.
#pragma once
#include "device_types.h"
#include "dmath.cuh"

namespace orion_gb300 {

struct Frame {
  V3 ng, ns, u, v;
};

__device__ __forceinline__ V3 world_to_local(const Frame& f, V3 w) { return V3{dot(w, f.u), dot(w, f.v), dot(w, f.ns)}; }
__device__ __forceinline__ V3 local_to_world(const Frame& f, V3 w) {
  return V3{f.u.x * w.x + f.v.x * w.y + f.ns.x * w.z, f.u.y * w.x + f.v.y * w.y + f.ns.y * w.z,
            f.u.z * w.x + f.v.z * w.y + f.ns.z * w.z};
}

// ---------------------------------------------------------------- Fresnel

__device__ __forceinline__ float fr_dielectric(float cos_i, float eta_i, float eta_t) {
  cos_i = clampf(cos_i, -1.f, 1.f);
  if (!(cos_i > 0.f)) {
    float t = eta_i;
    eta_i = eta_t;
    eta_t = t;
    cos_i = fabsf(cos_i);
  }
  float sin_i = sqrtf(fmaxf(0.f, 1.f - cos_i * cos_i));
  float sin_t = eta_i / eta_t * sin_i;
  if (sin_t >= 1.f) return 1.f;
  float cos_t = sqrtf(fmaxf(0.f, 1.f - sin_t * sin_t));
  float r_parl = ((eta_t * cos_i) - (eta_i * cos_t)) / ((eta_t * cos_i) + (eta_i * cos_t));
  float r_perp = ((eta_i * cos_i) - (eta_t * cos_t)) / ((eta_i * cos_i) + (eta_t * cos_t));
  return (r_parl * r_parl + r_perp * r_perp) / 2.f;
}

// Conductor Fresnel with etaI = 1 (the only use, src/material/metal.cpp:13).
__device__ __forceinline__ V3 fr_conductor(float cos_i, V3 eta, V3 k) {
  cos_i = clampf(cos_i, -1.f, 1.f);
  float c2 = cos_i * cos_i;
  float s2 = 1.f - c2;
  V3 eta2 = mul(eta, eta), k2 = mul(k, k);
  V3 t0 = (eta2 - k2) - v3(s2, s2, s2);
  V3 q = mul(t0, t0) + mul(eta2 * 4.f, k2);
  V3 a2b2 = V3{sqrtf(q.x), sqrtf(q.y), sqrtf(q.z)};
  V3 t1 = a2b2 + v3(c2, c2, c2);
  V3 h = (a2b2 + t0) * 0.5f;
  V3 a = V3{sqrtf(h.x), sqrtf(h.y), sqrtf(h.z)};
  V3 t2 = a * (2.f * cos_i);
  V3 rs = V3{(t1.x - t2.x) / (t1.x + t2.x), (t1.y - t2.y) / (t1.y + t2.y), (t1.z - t2.z) / (t1.z + t2.z)};
  V3 t3 = a2b2 * c2 + v3(s2 * s2, s2 * s2, s2 * s2);
  V3 t4 = t2 * s2;
  V3 rp = V3{rs.x * (t3.x - t4.x) / (t3.x + t4.x), rs.y * (t3.y - t4.y) / (t3.y + t4.y),
             rs.z * (t3.z - t4.z) / (t3.z + t4.z)};
  return (rp + rs) * 0.5f;
}

__device__ __forceinline__ V3 fresnel_eval(const DevLobe& l, float cos_i) {
  if (l.fresnel == FRESNEL_CONDUCTOR) return fr_conductor(fabsf(cos_i), ld3(l.fr_eta), ld3(l.fr_k));
  if (l.fresnel == FRESNEL_DIELECTRIC) {
    float f = fr_dielectric(fabsf(cos_i), l.etaA, l.etaB);
    return V3{f, f, f};
  }
  return V3{1.f, 1.f, 1.f};
}

// src/core/bsdf.h:101-115
__device__ __forceinline__ V3 reflect(V3 wo, V3 n) { return -wo + n * (2.f * dot(wo, n)); }
__device__ __forceinline__ bool refract(V3 wi, V3 n, float eta, V3* wt) {
  float cos_i = dot(n, wi);
  float sin2_i = fmaxf(0.f, 1.f - cos_i * cos_i);
  float sin2_t = eta * eta * sin2_i;
  if (sin2_t >= 1.f) return false;
  float cos_t = sqrtf(1.f - sin2_t);
  *wt = (-wi) * eta + n * (eta * cos_i - cos_t);
  return true;
}

// ------------------------------------------------------ microfacet models

__device__ __forceinline__ float md_D(int dist, float alpha, V3 wh) {
  float t2 = tan2_theta(wh);
  if (isinf(t2)) return 0.f;
  float c4 = cos2_theta(wh) * cos2_theta(wh);
  float a2 = alpha * alpha;
  if (dist == DIST_BECKMANN) return expf(-t2 / a2) / (kPi * a2 * c4);
  float e = t2 / a2;
  return 1.f / (kPi * a2 * c4 * (1.f + e) * (1.f + e));
}

__device__ __forceinline__ float md_lambda(int dist, float alpha, V3 w) {
  float at = fabsf(tan_theta(w));
  if (isinf(at)) return 0.f;
  if (dist == DIST_BECKMANN) {
    float a = 1.f / (alpha * at);
    if (a >= 1.6f) return 0.f;
    return (1.f - 1.259f * a + 0.396f * a * a) / (3.535f * a + 2.181f * a * a);
  }
  float a2t2 = (alpha * at) * (alpha * at);
  return (-1.f + sqrtf(1.f + a2t2)) / 2.f;
}

__device__ __forceinline__ float md_G(int dist, float alpha, V3 wi, V3 wo) {
  return 1.f / (1.f + md_lambda(dist, alpha, wi) + md_lambda(dist, alpha, wo));
}

__device__ __forceinline__ V3 md_sample_wh(int dist, float alpha, V3 wo, float u0, float u1) {
  float tan2;
  if (dist == DIST_BECKMANN) {
    float ls = logf(1.f - u0);
    if (isinf(ls)) ls = 0.f;
    tan2 = -alpha * alpha * ls;
  } else {
    tan2 = alpha * alpha * u0 / (1.f - u0);
  }
  float c = 1.f / sqrtf(1.f + tan2);
  float s = sqrtf(fmaxf(0.f, 1.f - c * c));
  float phi = (2.f * kPi) * u1;
  V3 wh = V3{s * cosf(phi), s * sinf(phi), c};
  if (!same_hemisphere(wo, wh)) wh = -wh;
  return wh;
}

__device__ __forceinline__ float md_pdf(int dist, float alpha, V3 wh) { return md_D(dist, alpha, wh) * abs_cos_theta(wh); }

// -------------------------------------------------------------- one lobe
//
// Every lobe and BSDF function is a template over KM, the set of lobe kinds
// (bit k = LobeKind k) its material may contain. The shading kernel of a
// shading class instantiates them with that class's kinds only, so its code
// holds just those lobes' arithmetic; KM = kLobeAll is the general form,
// whose lobe evaluators stay out of line (inlining every copy of every kind
// overflows the instruction cache).

constexpr unsigned kLobeAll = 0x7fu;

template <unsigned KM>
__device__ __forceinline__ constexpr bool has_kind(int kind) {
  return ((KM >> kind) & 1u) != 0u;
}

template <unsigned KM>
__device__ __forceinline__ V3 lobe_f_t(const DevLobe& l, V3 wi, V3 wo) {
  switch (l.kind) {
    case LOBE_LAMBERT_R:
      if constexpr (has_kind<KM>(LOBE_LAMBERT_R)) return ld3(l.c) * kInvPi;
      break;
    case LOBE_OREN_NAYAR:
      if constexpr (has_kind<KM>(LOBE_OREN_NAYAR)) {
        float si = sin_theta(wi), so = sin_theta(wo);
        float cos_term = 0.f;
        if (si > 1e-4f && so > 1e-4f) {
          float d = cos_phi(wi) * cos_phi(wo) + sin_phi(wi) * sin_phi(wo);
          cos_term = fmaxf(0.f, d);
        }
        float sin_a, tan_b;
        if (abs_cos_theta(wi) > abs_cos_theta(wo)) {
          sin_a = so;
          tan_b = si / abs_cos_theta(wi);
        } else {
          sin_a = si;
          tan_b = so / abs_cos_theta(wo);
        }
        return (ld3(l.c) * kInvPi) * (l.on_a + l.on_b * cos_term * sin_a * tan_b);
      }
      break;
    case LOBE_MICROFACET_R:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_R)) {
        float co = abs_cos_theta(wo), ci = abs_cos_theta(wi);
        if (ci == 0.f || co == 0.f) return V3{0, 0, 0};
        V3 wh = wi + wo;
        if (wh.x == 0.f && wh.y == 0.f && wh.z == 0.f) return V3{0, 0, 0};
        wh = normalize(wh);
        V3 F = fresnel_eval(l, dot(wi, wh));
        float dg = md_D(l.dist, l.alpha, wh);
        float g = md_G(l.dist, l.alpha, wi, wi);  // the reference passes wi twice
        return sdiv(mul((ld3(l.c) * dg) * g, F), 4.f * ci * co);
      }
      break;
    case LOBE_MICROFACET_T:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_T)) {
        if (same_hemisphere(wi, wo)) return V3{0, 0, 0};
        float co = cos_theta(wo), ci = cos_theta(wi);
        if (ci == 0.f || co == 0.f) return V3{0, 0, 0};
        float eta = cos_theta(wo) > 0.f ? (l.etaB / l.etaA) : (l.etaA / l.etaB);
        V3 wh = normalize(wo + wi * eta);
        if (wh.z < 0.f) wh = -wh;
        float F = fr_dielectric(fabsf(dot(wo, wh)), l.etaA, l.etaB);
        float sd = dot(wo, wh) + eta * dot(wi, wh);
        float factor = l.photon ? 1.f : 1.f / eta;  // TransportMode (microfacet.cpp:102)
        float v = fabsf(md_D(l.dist, l.alpha, wh) * md_G(l.dist, l.alpha, wi, wo) * eta * eta * absdot(wi, wh) *
                        absdot(wo, wh) * factor * factor / (ci * co * sd * sd));
        return mul(V3{1.f - F, 1.f - F, 1.f - F}, ld3(l.c)) * v;
      }
      break;
    default:  // specular lobes are delta distributions
      break;
  }
  return V3{0, 0, 0};
}

template <unsigned KM>
__device__ __forceinline__ float lobe_pdf_t(const DevLobe& l, V3 wi, V3 wo) {
  switch (l.kind) {
    case LOBE_LAMBERT_R:
    case LOBE_OREN_NAYAR:
      if constexpr (has_kind<KM>(LOBE_LAMBERT_R) || has_kind<KM>(LOBE_OREN_NAYAR))
        return same_hemisphere(wi, wo) ? abs_cos_theta(wi) * kInvPi : 0.f;
      break;
    case LOBE_MICROFACET_R:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_R)) {
        if (!same_hemisphere(wi, wo)) return 0.f;
        V3 wh = normalize(wi + wo);
        return md_pdf(l.dist, l.alpha, wh) / (4.f * dot(wo, wh));
      }
      break;
    case LOBE_MICROFACET_T:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_T)) {
        if (same_hemisphere(wo, wi)) return 0.f;
        float eta = cos_theta(wo) > 0.f ? (l.etaB / l.etaA) : (l.etaA / l.etaB);
        V3 wh = normalize(wo + wi * eta);
        float sd = dot(wo, wh) + eta * dot(wi, wh);
        float dwh = fabsf((eta * eta * dot(wi, wh)) / (sd * sd));
        return md_pdf(l.dist, l.alpha, wh) * dwh;
      }
      break;
    default:
      break;
  }
  return 0.f;
}

static __device__ __noinline__ V3 lobe_f_all(const DevLobe& l, V3 wi, V3 wo) { return lobe_f_t<kLobeAll>(l, wi, wo); }
static __device__ __noinline__ float lobe_pdf_all(const DevLobe& l, V3 wi, V3 wo) {
  return lobe_pdf_t<kLobeAll>(l, wi, wo);
}

template <unsigned KM>
__device__ __forceinline__ V3 lobe_f(const DevLobe& l, V3 wi, V3 wo) {
  if constexpr (KM == kLobeAll)
    return lobe_f_all(l, wi, wo);
  else
    return lobe_f_t<KM>(l, wi, wo);
}

template <unsigned KM>
__device__ __forceinline__ float lobe_pdf(const DevLobe& l, V3 wi, V3 wo) {
  if constexpr (KM == kLobeAll)
    return lobe_pdf_all(l, wi, wo);
  else
    return lobe_pdf_t<KM>(l, wi, wo);
}

// Samples one lobe; *pdf is left untouched (0) on the reference's early exits.
template <unsigned KM>
__device__ __forceinline__ V3 lobe_sample_f_t(const DevLobe& l, V3 wo, float u0, float u1, V3* wi, float* pdf,
                                              int* stype) {
  switch (l.kind) {
    case LOBE_LAMBERT_R:
    case LOBE_OREN_NAYAR:
      if constexpr (has_kind<KM>(LOBE_LAMBERT_R) || has_kind<KM>(LOBE_OREN_NAYAR)) {
        *wi = cosine_sample_hemisphere(u0, u1);
        if (wo.z < 0.f) wi->z *= -1.f;
        *pdf = lobe_pdf<KM>(l, *wi, wo);
        return lobe_f<KM>(l, *wi, wo);
      }
      break;
    case LOBE_MICROFACET_R:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_R)) {
        if (wo.z == 0.f) return V3{0, 0, 0};
        V3 wh = md_sample_wh(l.dist, l.alpha, wo, u0, u1);
        *wi = reflect(wo, wh);
        if (!same_hemisphere(*wi, wo)) return V3{0, 0, 0};
        *pdf = md_pdf(l.dist, l.alpha, wh) / (4.f * dot(wo, wh));
        return lobe_f<KM>(l, *wi, wo);
      }
      break;
    case LOBE_MICROFACET_T:
      if constexpr (has_kind<KM>(LOBE_MICROFACET_T)) {
        if (wo.z == 0.f) return V3{0, 0, 0};
        V3 wh = md_sample_wh(l.dist, l.alpha, wo, u0, u1);
        float eta = cos_theta(wo) > 0.f ? (l.etaA / l.etaB) : (l.etaB / l.etaA);
        if (!refract(wo, wh, eta, wi)) return V3{0, 0, 0};
        return lobe_f<KM>(l, *wi, wo);  // pdf is never set (src/bsdf/microfacet.cpp:76-85)
      }
      break;
    case LOBE_SPECULAR_R:
      if constexpr (has_kind<KM>(LOBE_SPECULAR_R)) {
        *wi = V3{-wo.x, -wo.y, wo.z};
        *pdf = 1.f;
        return sdiv(mul(fresnel_eval(l, cos_theta(*wi)), ld3(l.c)), abs_cos_theta(*wi));
      }
      break;
    case LOBE_SPECULAR_T:
      if constexpr (has_kind<KM>(LOBE_SPECULAR_T)) {
        bool entering = cos_theta(wo) > 0.f;
        float ei = entering ? l.etaA : l.etaB;
        float et = entering ? l.etaB : l.etaA;
        if (!refract(wo, faceforward(V3{0, 0, 1}, wo), ei / et, wi)) return V3{0, 0, 0};
        *pdf = 1.f;
        float F = fr_dielectric(fabsf(cos_theta(*wi)), l.etaA, l.etaB);
        V3 ft = mul(ld3(l.c), V3{1.f - F, 1.f - F, 1.f - F});
        if (!l.photon) ft = ft * ((ei * ei) / (et * et));
        return sdiv(ft, abs_cos_theta(*wi));
      }
      break;
    case LOBE_FRESNEL_SPECULAR:
      if constexpr (has_kind<KM>(LOBE_FRESNEL_SPECULAR)) {
        float F = fr_dielectric(cos_theta(wo), l.etaA, l.etaB);
        if (u0 < F) {
          *wi = V3{-wo.x, -wo.y, wo.z};
          *stype = BXDF_SPECULAR | BXDF_REFLECTION;
          *pdf = F;
          return sdiv(ld3(l.c) * F, abs_cos_theta(*wi));
        }
        bool entering = cos_theta(wo) > 0.f;
        float ei = entering ? l.etaA : l.etaB;
        float et = entering ? l.etaB : l.etaA;
        if (!refract(wo, faceforward(V3{0, 0, 1}, wo), ei / et, wi)) return V3{0, 0, 0};
        V3 ft = ld3(l.c2) * (1.f - F);
        if (!l.photon) ft = ft * ((ei * ei) / (et * et));
        *stype = BXDF_SPECULAR | BXDF_TRANSMISSION;
        *pdf = 1.f - F;
        return sdiv(ft, abs_cos_theta(*wi));
      }
      break;
    default:
      break;
  }
  return V3{0, 0, 0};
}

static __device__ __noinline__ V3 lobe_sample_f_all(const DevLobe& l, V3 wo, float u0, float u1, V3* wi, float* pdf,
                                                    int* stype) {
  return lobe_sample_f_t<kLobeAll>(l, wo, u0, u1, wi, pdf, stype);
}

template <unsigned KM>
__device__ __forceinline__ V3 lobe_sample_f(const DevLobe& l, V3 wo, float u0, float u1, V3* wi, float* pdf,
                                            int* stype) {
  if constexpr (KM == kLobeAll)
    return lobe_sample_f_all(l, wo, u0, u1, wi, pdf, stype);
  else
    return lobe_sample_f_t<KM>(l, wo, u0, u1, wi, pdf, stype);
}

__device__ __forceinline__ bool lobe_matches(const DevLobe& l, int type) { return (l.type & type) == l.type; }

// ------------------------------------------------------------- full BSDF

__device__ __forceinline__ int bsdf_num_matching(const DevMaterial& m, int type) {
  int n = 0;
  for (int i = 0; i < m.num_lobes; ++i) n += lobe_matches(m.lobes[i], type);
  return n;
}

template <unsigned KM = kLobeAll>
__device__ __forceinline__ V3 bsdf_f(const DevMaterial& m, const Frame& fr, V3 wi_w, V3 wo_w, int type) {
  V3 wi = world_to_local(fr, wi_w), wo = world_to_local(fr, wo_w);
  V3 r{0, 0, 0};
  for (int i = 0; i < m.num_lobes; ++i)
    if (lobe_matches(m.lobes[i], type)) r = r + lobe_f<KM>(m.lobes[i], wi, wo);
  return r;
}

template <unsigned KM = kLobeAll>
__device__ __forceinline__ float bsdf_pdf(const DevMaterial& m, const Frame& fr, V3 wi_w, V3 wo_w, int type) {
  if (m.num_lobes == 0) return 0.f;
  V3 wi = world_to_local(fr, wi_w), wo = world_to_local(fr, wo_w);
  if (wo.z == 0.f) return 0.f;
  float pdf = 0.f;
  int n = 0;
  for (int i = 0; i < m.num_lobes; ++i)
    if (lobe_matches(m.lobes[i], type)) {
      ++n;
      pdf += lobe_pdf<KM>(m.lobes[i], wi, wo);
    }
  return n > 0 ? pdf / n : 0.f;
}

// Returns f; *pdf = 0 and *stype = 0 on failure. *wi is written only on success.
template <unsigned KM>
__device__ __forceinline__ V3 bsdf_sample_f_t(const DevMaterial& m, const Frame& fr, V3 wo_w, float u0, float u1,
                                              int type, V3* wi_w, float* pdf, int* stype) {
  int n = bsdf_num_matching(m, type);
  *pdf = 0.f;
  *stype = 0;
  if (n == 0) return V3{0, 0, 0};
  int pos = min((int)floorf(u0 * n), n - 1);
  int sel = -1, count = pos;
  for (int i = 0; i < m.num_lobes; ++i)
    if (lobe_matches(m.lobes[i], type) && count-- == 0) {
      sel = i;
      break;
    }
  const DevLobe& lb = m.lobes[sel];
  float nu0 = fminf(u0 * n - pos, kOneMinusEpsilon);
  V3 wo = world_to_local(fr, wo_w);
  if (wo.z == 0.f) return V3{0, 0, 0};
  *stype = lb.type;
  V3 wi;
  V3 f = lobe_sample_f<KM>(lb, wo, nu0, u1, &wi, pdf, stype);
  if (*pdf == 0.f) {
    *stype = 0;
    return V3{0, 0, 0};
  }
  *wi_w = local_to_world(fr, wi);
  bool specular = (lb.type & BXDF_SPECULAR) != 0;
  if (!specular && n > 1)
    for (int i = 0; i < m.num_lobes; ++i)
      if (i != sel && lobe_matches(m.lobes[i], type)) *pdf += lobe_pdf<KM>(m.lobes[i], wi, wo);
  if (n > 1) *pdf /= n;
  if (!specular && n > 1) {
    bool refl = dot(*wi_w, fr.ng) * dot(wo_w, fr.ng) > 0.f;
    f = V3{0, 0, 0};
    for (int i = 0; i < m.num_lobes; ++i) {
      const DevLobe& l = m.lobes[i];
      bool has_r = (l.type & BXDF_REFLECTION) != 0, has_t = (l.type & BXDF_TRANSMISSION) != 0;
      if (lobe_matches(l, type) && ((refl && has_r) || (!refl && has_t))) f = f + lobe_f<KM>(l, wi, wo);
    }
  }
  return f;
}

static __device__ __noinline__ V3 bsdf_sample_f_all(const DevMaterial& m, const Frame& fr, V3 wo_w, float u0,
                                                    float u1, int type, V3* wi_w, float* pdf, int* stype) {
  return bsdf_sample_f_t<kLobeAll>(m, fr, wo_w, u0, u1, type, wi_w, pdf, stype);
}

template <unsigned KM = kLobeAll>
__device__ __forceinline__ V3 bsdf_sample_f(const DevMaterial& m, const Frame& fr, V3 wo_w, float u0, float u1,
                                            int type, V3* wi_w, float* pdf, int* stype) {
  if constexpr (KM == kLobeAll)
    return bsdf_sample_f_all(m, fr, wo_w, u0, u1, type, wi_w, pdf, stype);
  else
    return bsdf_sample_f_t<KM>(m, fr, wo_w, u0, u1, type, wi_w, pdf, stype);
}

}  // namespace orion_gb300
