// Lobe lists of the reference's materials (Material::getBSDF,
// src/material/*.cpp), built from evaluated inputs. The host builds every
// material once from its constants; the textured shading kernel builds a
// material per hit from the texels under the hit. Both run this code, so a
// textured material whose texels equal its constants gets the same lobes.
//
// No transcendental function is evaluated here (alpha and the Oren-Nayar
// constants arrive precomputed) and no product feeds a sum, so host and
// device arithmetic agree bit for bit.
#pragma once
#include "../../include/orion_gpu.h"
#include "device_types.h"

namespace orion_gb300 {

namespace mb {

ORION_HD inline bool black3(const float* c) { return c[0] == 0.f && c[1] == 0.f && c[2] == 0.f; }
ORION_HD inline void clamp0(const float* in, float* out) {
  for (int k = 0; k < 3; ++k) out[k] = in[k] < 0.f ? 0.f : in[k];
}
ORION_HD inline void set3(float* d, const float* s) {
  d[0] = s[0];
  d[1] = s[1];
  d[2] = s[2];
}
ORION_HD inline DevLobe lobe(int kind, int type) {
  DevLobe l{};
  l.kind = kind;
  l.type = type;
  l.fresnel = FRESNEL_NOOP;
  l.dist = DIST_GGX;
  return l;
}
ORION_HD inline void add(DevMaterial* m, const DevLobe& l) {
  if (m->num_lobes < kMaxLobes) m->lobes[m->num_lobes++] = l;
}
ORION_HD inline DevLobe microfacet_r(const float* R, int dist, float alpha) {
  DevLobe l = lobe(LOBE_MICROFACET_R, BXDF_REFLECTION | BXDF_GLOSSY);
  set3(l.c, R);
  l.dist = dist;
  l.alpha = alpha;
  return l;
}
ORION_HD inline DevLobe dielectric_fresnel(DevLobe l, float eta_i, float eta_t) {
  l.fresnel = FRESNEL_DIELECTRIC;
  l.etaA = eta_i;
  l.etaB = eta_t;
  return l;
}
// c = clamp(a) * op, componentwise (uber.cpp:18-37).
ORION_HD inline void clamp_times(const float* a, const float* op, float* c) {
  float t[3];
  clamp0(a, t);
  for (int k = 0; k < 3; ++k) c[k] = t[k] * op[k];
}

}  // namespace mb

// Material::getBSDF for the material `mt` (constants and evaluated textures).
// Fills lobes, num_lobes and num_nonspecular; shade_class is left as is.
ORION_HD inline void build_material(const MaterialInputs& mt, DevMaterial* m) {
  using namespace mb;
  m->num_lobes = 0;
  m->num_nonspecular = 0;
  const int dist = mt.dist;
  switch (mt.type) {
    case ORION_MAT_MATTE: {  // src/material/matte.cpp:9-21
      float r[3];
      clamp0(mt.Kd, r);
      if (!black3(r)) {
        if (mt.sigma == 0.f) {
          DevLobe l = lobe(LOBE_LAMBERT_R, BXDF_REFLECTION | BXDF_DIFFUSE);
          set3(l.c, r);
          add(m, l);
        } else {  // src/bsdf/orennayar.cpp:5-12
          DevLobe l = lobe(LOBE_OREN_NAYAR, BXDF_REFLECTION | BXDF_DIFFUSE);
          set3(l.c, r);
          l.on_a = mt.on_a;
          l.on_b = mt.on_b;
          add(m, l);
        }
      }
      break;
    }
    case ORION_MAT_METAL: {  // src/material/metal.cpp:8-17
      const float one[3] = {1.f, 1.f, 1.f};
      DevLobe l = microfacet_r(one, dist, mt.alpha);
      l.fresnel = FRESNEL_CONDUCTOR;
      set3(l.fr_eta, mt.eta_rgb);
      set3(l.fr_k, mt.k);
      add(m, l);
      break;
    }
    case ORION_MAT_MIRROR: {  // src/material/mirror.cpp:6-13
      float r[3];
      clamp0(mt.Kr, r);
      if (!black3(r)) {
        DevLobe l = lobe(LOBE_SPECULAR_R, BXDF_REFLECTION | BXDF_SPECULAR);
        set3(l.c, r);
        add(m, l);
      }
      break;
    }
    case ORION_MAT_GLASS: {  // src/material/glass.cpp:9-37
      const float e = mt.eta;
      if (black3(mt.Kr) && black3(mt.Kt)) break;
      if (mt.roughness == 0.f) {
        DevLobe l = lobe(LOBE_FRESNEL_SPECULAR, BXDF_REFLECTION | BXDF_TRANSMISSION | BXDF_SPECULAR);
        set3(l.c, mt.Kr);
        set3(l.c2, mt.Kt);
        l.etaA = 1.f;
        l.etaB = e;
        add(m, l);
      } else {
        if (!black3(mt.Kr)) add(m, dielectric_fresnel(microfacet_r(mt.Kr, dist, mt.alpha), 1.f, e));
        if (!black3(mt.Kt)) {
          DevLobe l = lobe(LOBE_MICROFACET_T, BXDF_TRANSMISSION | BXDF_GLOSSY);
          set3(l.c, mt.Kt);
          l.dist = dist;
          l.alpha = mt.alpha;
          l.etaA = 1.f;
          l.etaB = e;
          add(m, l);
        }
      }
      break;
    }
    case ORION_MAT_PLASTIC: {  // src/material/plastic.cpp:8-24
      float kd[3], ks[3];
      clamp0(mt.Kd, kd);
      if (!black3(kd)) {
        DevLobe l = lobe(LOBE_LAMBERT_R, BXDF_REFLECTION | BXDF_DIFFUSE);
        set3(l.c, kd);
        add(m, l);
      }
      clamp0(mt.Ks, ks);
      if (!black3(ks))  // the reference's fixed Fresnel has the etas reversed (plastic.cpp:17)
        add(m, dielectric_fresnel(microfacet_r(ks, dist, mt.alpha), 1.5f, 1.0f));
      break;
    }
    case ORION_MAT_UBER: {  // src/material/uber.cpp:9-42
      const float* op = mt.opacity;
      const float e = mt.eta;
      float one_minus[3] = {1.f - op[0], 1.f - op[1], 1.f - op[2]}, t[3], c[3];
      clamp0(one_minus, t);
      if (!black3(t)) {
        DevLobe l = lobe(LOBE_SPECULAR_T, BXDF_TRANSMISSION | BXDF_SPECULAR);
        set3(l.c, t);
        l.etaA = 1.f;
        l.etaB = 1.f;
        add(m, l);
      }
      clamp_times(mt.Kd, op, c);
      if (!black3(c)) {
        DevLobe l = lobe(LOBE_LAMBERT_R, BXDF_REFLECTION | BXDF_DIFFUSE);
        set3(l.c, c);
        add(m, l);
      }
      clamp_times(mt.Ks, op, c);
      if (!black3(c)) add(m, dielectric_fresnel(microfacet_r(c, dist, mt.alpha), 1.f, e));
      clamp_times(mt.Kr, op, c);
      if (!black3(c)) {
        DevLobe l = lobe(LOBE_SPECULAR_R, BXDF_REFLECTION | BXDF_SPECULAR);
        set3(l.c, c);
        add(m, dielectric_fresnel(l, 1.f, e));
      }
      clamp_times(mt.Kt, op, c);
      if (!black3(c)) {
        DevLobe l = lobe(LOBE_SPECULAR_T, BXDF_TRANSMISSION | BXDF_SPECULAR);
        set3(l.c, c);
        l.etaA = 1.f;
        l.etaB = e;
        add(m, l);
      }
      break;
    }
    default:
      break;
  }
  for (int i = 0; i < m->num_lobes; ++i) {
    const int t = m->lobes[i].type;
    const int ns = BXDF_ALL & ~BXDF_SPECULAR;
    if ((t & ns) == t) ++m->num_nonspecular;
  }
}

}  // namespace orion_gb300
