// Device scene records from a HostScene.
//
// All host-side float arithmetic here restates the reference's operation
// order (compiled without FP contraction), so lobe constants, light powers
// and the light-selection CDF are bit-identical to the values the reference
// computes per hit or at preprocess time.
#include "scene_prep.h"

#include "material_build.h"

#include <cmath>
#include <cstring>
#include <limits>

namespace orion_gb300 {

namespace {
constexpr float kPiF = 3.14159265358979323846f;

void set3(float* d, const float* s) {
  d[0] = s[0];
  d[1] = s[1];
  d[2] = s[2];
}
}  // namespace

float roughness_to_alpha(float roughness) {
  roughness = std::max(roughness, 1e-3f);
  float x = std::log(roughness);
  return 1.62142f + 0.819955f * x + 0.1734f * x * x + 0.0171201f * x * x * x + 0.000640711f * x * x * x * x;
}

float spectrum_intensity(const float c[3]) { return 0.212671f * c[0] + 0.715160f * c[1] + 0.072169f * c[2]; }

MaterialInputs material_inputs(const orion_material& mt) {
  MaterialInputs in;
  std::memset(&in, 0, sizeof(in));
  in.type = mt.type;
  in.dist = mt.distribution == ORION_DIST_BECKMANN ? DIST_BECKMANN : DIST_GGX;
  set3(in.Kd, mt.Kd);
  set3(in.Ks, mt.Ks);
  set3(in.Kr, mt.Kr);
  set3(in.Kt, mt.Kt);
  set3(in.opacity, mt.opacity);
  set3(in.eta_rgb, mt.eta_rgb);
  set3(in.k, mt.k);
  in.sigma = mt.has_sigma ? (mt.sigma < 0.f ? 0.f : mt.sigma) : 0.f;
  in.roughness = mt.roughness;
  in.eta = mt.eta;
  in.alpha = roughness_to_alpha(mt.roughness);
  if (in.sigma != 0.f) {  // src/bsdf/orennayar.cpp:5-12
    float s = in.sigma * static_cast<float>(0.01745329251994329576923690768489);
    float s2 = s * s;
    in.on_a = 1.f - (s2 / (2.f * (s2 + 0.33f)));
    in.on_b = 0.45f * s2 / (s2 + 0.09f);
  }
  return in;
}

bool material_textured(const orion_material& mt) {
  for (int t = 0; t < kTexSlots; ++t)
    if (mt.tex[t] != 0) return true;
  return false;
}

DevMaterial prepare_material(const orion_material& mt) {
  DevMaterial m;
  std::memset(&m, 0, sizeof(m));
  build_material(material_inputs(mt), &m);
  unsigned kinds = 0;
  for (int i = 0; i < m.num_lobes; ++i) {
    int t = m.lobes[i].type;
    const int ns = BXDF_ALL & ~BXDF_SPECULAR;
    if ((t & ns) == t) ++m.num_nonspecular;
    kinds |= 1u << m.lobes[i].kind;
  }
  const unsigned spec = (1u << LOBE_SPECULAR_R) | (1u << LOBE_SPECULAR_T) | (1u << LOBE_FRESNEL_SPECULAR);
  if (kinds == (1u << LOBE_LAMBERT_R))
    m.shade_class = SC_DIFFUSE;
  else if (kinds == (1u << LOBE_MICROFACET_R))
    m.shade_class = SC_CONDUCTOR;
  else if (kinds != 0 && (kinds & ~spec) == 0)
    m.shade_class = SC_SPECULAR;
  else if (kinds == ((1u << LOBE_MICROFACET_R) | (1u << LOBE_MICROFACET_T)))
    m.shade_class = SC_DIELECTRIC;
  else if (kinds == ((1u << LOBE_LAMBERT_R) | (1u << LOBE_MICROFACET_R)))
    m.shade_class = SC_PLASTIC;
  else
    m.shade_class = SC_GENERAL;
  if (material_textured(mt)) m.shade_class = SC_TEXTURED;
  return m;
}

namespace {

// Distribution1D (src/sampler/sampling.h:71-90): func, cdf (n + 1), funcInt.
float dist1d(const float* f, int n, float* func, float* cdf) {
  for (int i = 0; i < n; ++i) func[i] = f[i];
  cdf[0] = 0.f;
  for (int i = 1; i < n + 1; ++i) cdf[i] = cdf[i - 1] + func[i - 1] / n;
  const float func_int = cdf[n];
  if (func_int == 0.f) {
    for (int i = 1; i < n + 1; ++i) cdf[i] = float(i) / float(n);
  } else {
    for (int i = 1; i < n + 1; ++i) cdf[i] /= func_int;
  }
  return func_int;
}

// Envmap::Envmap for an image (src/light/envmap.cpp:9-44): texels times L,
// the sampling function intensity(texel) * sin(theta) per texel, and the
// Distribution2D over it (sampling.cpp:63-76). Returns the average texel.
void prepare_envmap(const HostImage& im, const float L[3], PreparedScene* out, float ave[3]) {
  const int w = im.width, h = im.height;
  const size_t n = (size_t)w * h;
  PreparedScene::EnvMapLayout lay;
  lay.width = w;
  lay.height = h;
  std::vector<float>& d = out->env_data;
  lay.texels = d.size();
  d.resize(d.size() + 3 * n);
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) d[lay.texels + 3 * i + k] = im.rgb[3 * i + k] * L[k];
  std::vector<float> img(n);
  float sum[3] = {0.f, 0.f, 0.f};
  for (int j = 0; j < h; ++j) {
    const float v = (j + 0.5f) / (float)h;
    const float sin_theta = std::sin(kPiF * v);
    for (int i = 0; i < w; ++i) {
      const float* t = &d[lay.texels + 3 * ((size_t)j * w + i)];
      img[i + (size_t)j * w] = spectrum_intensity(t) * sin_theta;
      for (int k = 0; k < 3; ++k) sum[k] += t[k];
    }
  }
  for (int k = 0; k < 3; ++k) ave[k] = sum[k] / (float)(w * h);
  lay.cond_func = d.size();
  d.resize(d.size() + n);
  lay.cond_cdf = d.size();
  d.resize(d.size() + (size_t)h * (w + 1));
  lay.cond_int = d.size();
  d.resize(d.size() + h);
  for (int j = 0; j < h; ++j)
    d[lay.cond_int + j] = dist1d(&img[(size_t)j * w], w, &d[lay.cond_func + (size_t)j * w],
                                 &d[lay.cond_cdf + (size_t)j * (w + 1)]);
  std::vector<float> marginal(d.begin() + lay.cond_int, d.begin() + lay.cond_int + h);
  lay.marg_func = d.size();
  d.resize(d.size() + h);
  lay.marg_cdf = d.size();
  d.resize(d.size() + h + 1);
  lay.marg_int = dist1d(marginal.data(), h, &d[lay.marg_func], &d[lay.marg_cdf]);
  out->envmaps.push_back(lay);
}

}  // namespace

bool prepare_scene(const HostScene& s, PreparedScene* out, std::string* err) {
  const int64_t T = s.num_prims();
  out->prims.resize(T);
  float lo[3] = {std::numeric_limits<float>::max(), std::numeric_limits<float>::max(),
                 std::numeric_limits<float>::max()};
  float hi[3] = {std::numeric_limits<float>::lowest(), std::numeric_limits<float>::lowest(),
                 std::numeric_limits<float>::lowest()};
  for (int64_t i = 0; i < T; ++i) {
    PrimShade& p = out->prims[i];
    std::memset(&p, 0, sizeof(p));
    std::memcpy(p.p, &s.positions[9 * i], 9 * sizeof(float));
    std::memcpy(p.n, &s.normals[9 * i], 9 * sizeof(float));
    p.material = s.material_of_prim[i];
    p.light = s.light_of_prim[i];
    for (int c = 0; c < 3; ++c)
      for (int k = 0; k < 3; ++k) {
        lo[k] = std::min(lo[k], p.p[3 * c + k]);
        hi[k] = std::max(hi[k], p.p[3 * c + k]);
      }
  }
  // Bounds3::boundingSphere (src/core/geometry.h:551-554).
  for (int k = 0; k < 3; ++k) out->world_center[k] = (lo[k] + hi[k]) * 0.5f;
  bool inside = T > 0;
  for (int k = 0; k < 3; ++k) inside = inside && out->world_center[k] >= lo[k] && out->world_center[k] <= hi[k];
  if (inside) {
    float d[3] = {out->world_center[0] - hi[0], out->world_center[1] - hi[1], out->world_center[2] - hi[2]};
    out->world_radius = std::sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
  } else {
    out->world_radius = 0.f;
  }

  out->mats.clear();
  for (const orion_material& m : s.materials) out->mats.push_back(prepare_material(m));

  const float pi = kPiF, r = out->world_radius;
  out->lights.clear();
  out->env_idx.clear();
  out->env_data.clear();
  out->envmaps.clear();
  out->textures.clear();
  out->mat_src.clear();
  out->prim_uv.clear();
  // Image textures (src/util/parser.cpp:433-461): one DevTexture per image
  // that a material input reads, texels as loaded (no scaling).
  std::vector<int> tex_of_image(s.images.size(), -1);
  bool any_textured = false;
  for (const orion_material& m : s.materials) {
    DevMaterialSrc src;
    std::memset(&src, 0, sizeof(src));
    src.in = material_inputs(m);
    for (int t = 0; t < 8; ++t) src.tex[t] = -1;
    for (int t = 0; t < kTexSlots; ++t) {
      if (m.tex[t] == 0) continue;
      if (m.tex[t] < 0 || m.tex[t] > (int)s.images.size()) {
        *err = "material references a missing image";
        return false;
      }
      const int ii = m.tex[t] - 1;
      if (tex_of_image[ii] < 0) {
        const HostImage& im = s.images[ii];
        PreparedScene::TextureLayout lay{im.width, im.height, out->env_data.size()};
        out->env_data.insert(out->env_data.end(), im.rgb.begin(), im.rgb.begin() + 3 * (size_t)im.width * im.height);
        tex_of_image[ii] = (int)out->textures.size();
        out->textures.push_back(lay);
      }
      src.tex[t] = tex_of_image[ii];
      any_textured = true;
    }
    out->mat_src.push_back(src);
  }
  if (any_textured) {
    if (s.uvs.size() != 6 * (size_t)T) {
      *err = "textured materials need texture coordinates for every primitive";
      return false;
    }
    out->prim_uv = s.uvs;
  }
  std::vector<float> power;
  for (size_t i = 0; i < s.lights.size(); ++i) {
    const orion_light& l = s.lights[i];
    DevLight d;
    std::memset(&d, 0, sizeof(d));
    set3(d.L, l.L);
    float pw[3];
    switch (l.type) {
      case ORION_LIGHT_AREA: {  // src/light/diffuse.cpp:8-11, src/core/triangle.cpp:77-83
        if (l.prim < 0 || l.prim >= T) {
          *err = "area light references a missing primitive";
          return false;
        }
        d.kind = DL_AREA;
        d.prim = l.prim;
        const float* p = &s.positions[9 * (size_t)l.prim];
        float e1[3] = {p[3] - p[0], p[4] - p[1], p[5] - p[2]};
        float e2[3] = {p[6] - p[0], p[7] - p[1], p[8] - p[2]};
        float c[3] = {e1[1] * e2[2] - e1[2] * e2[1], e1[2] * e2[0] - e1[0] * e2[2], e1[0] * e2[1] - e1[1] * e2[0]};
        d.area = 0.5f * std::sqrt(c[0] * c[0] + c[1] * c[1] + c[2] * c[2]);
        for (int k = 0; k < 3; ++k) pw[k] = l.L[k] * d.area * pi;
        break;
      }
      case ORION_LIGHT_POINT: {  // src/light/point.cpp:6-9
        d.kind = DL_POINT;
        set3(d.p, l.p);
        float s4 = 4 * pi;
        for (int k = 0; k < 3; ++k) pw[k] = l.L[k] * s4;
        break;
      }
      case ORION_LIGHT_SPOT: {  // src/light/spot.cpp:6-9
        d.kind = DL_SPOT;
        set3(d.p, l.p);
        for (int rr = 0; rr < 3; ++rr)
          for (int c = 0; c < 3; ++c) {
            d.m[3 * rr + c] = l.w2l[4 * rr + c];
            d.minv[3 * rr + c] = l.l2w[4 * rr + c];
          }
        d.cos_total = l.cos_total;
        d.cos_falloff = l.cos_falloff;
        float f = 1 - .5f * (l.cos_falloff + l.cos_total);
        for (int k = 0; k < 3; ++k) pw[k] = l.L[k] * 2 * pi * f;
        break;
      }
      case ORION_LIGHT_DISTANT: {  // src/light/distant.cpp:11-14
        d.kind = DL_DISTANT;
        set3(d.p, l.dir);
        for (int k = 0; k < 3; ++k) pw[k] = l.L[k] * pi * r * r;
        break;
      }
      case ORION_LIGHT_ENV: {  // src/light/envmap.cpp:9-44, 62-65
        d.kind = DL_ENV;
        for (int rr = 0; rr < 3; ++rr)
          for (int c = 0; c < 3; ++c) {
            d.m[3 * rr + c] = l.l2w[4 * rr + c];
            d.minv[3 * rr + c] = l.w2l[4 * rr + c];
          }
        float ave[3] = {l.L[0], l.L[1], l.L[2]};  // constant map: the one texel is L
        d.image = -1;
        if (l.image > 0) {
          if (l.image > (int)s.images.size()) {
            *err = "environment light references a missing image";
            return false;
          }
          d.image = (int)out->envmaps.size();
          prepare_envmap(s.images[l.image - 1], l.L, out, ave);
        }
        d.area = spectrum_intensity(l.L) * std::sin(pi * 0.5f);
        float f = pi * r * r;
        for (int k = 0; k < 3; ++k) pw[k] = ave[k] * f;
        out->env_idx.push_back((int)i);
        break;
      }
      default:
        *err = "unknown light type";
        return false;
    }
    out->lights.push_back(d);
    power.push_back(spectrum_intensity(pw));
  }
  // Distribution1D (src/sampler/sampling.h:71-90).
  const int n = (int)power.size();
  out->light_func = power;
  out->light_cdf.assign(n + 1, 0.f);
  for (int i = 1; i < n + 1; ++i) out->light_cdf[i] = out->light_cdf[i - 1] + power[i - 1] / n;
  out->light_func_int = n > 0 ? out->light_cdf[n] : 0.f;
  if (n > 0) {
    if (out->light_func_int == 0.f) {
      for (int i = 1; i < n + 1; ++i) out->light_cdf[i] = float(i) / float(n);
    } else {
      for (int i = 1; i < n + 1; ++i) out->light_cdf[i] /= out->light_func_int;
    }
  }
  if (out->light_func.empty()) {  // keep device pointers valid
    out->light_func.push_back(0.f);
  }

  out->cam = prepare_camera(s.camera);
  return true;
}

// Pinhole (src/camera/pinhole.h:22-26, src/core/camera.h:24-25).
DevCamera prepare_camera(const orion_camera& cam) {
  DevCamera c;
  std::memset(&c, 0, sizeof(c));
  std::memcpy(c.c2w, cam.c2w, sizeof(c.c2w));
  c.tan_half_fov = std::tan(cam.fov * 0.5f * static_cast<float>(0.01745329251994329576923690768489));
  c.aspect = (float)cam.width / cam.height;
  c.lens_radius = cam.lens_radius;
  c.focal_distance = cam.focal_distance;
  c.width = cam.width;
  c.height = cam.height;
  return c;
}

}  // namespace orion_gb300
