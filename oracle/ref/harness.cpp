// Test infrastructure: a C ABI over the reference renderer compiled here.
//
// Built only in this development container (the reference sources are not on
// the GPU machines) into oracle/_ref/liborion_ref.so by oracle/ref/Makefile.
// The golden-fixture script and the CPU tests load it with ctypes to
//   * pin the C++ restatement in oracle/port against the reference itself,
//   * generate the small golden vectors committed under tests/golden/.
// Every entry point drives the reference's own classes; nothing here
// re-implements their arithmetic.
#include <core/bsdf.h>
#include <core/camera.h>
#include <core/integrator.h>
#include <core/light.h>
#include <core/primitive.h>
#include <core/sampler.h>
#include <core/scene.h>
#include <material/glass.h>
#include <material/matte.h>
#include <material/metal.h>
#include <material/mirror.h>
#include <material/plastic.h>
#include <material/uber.h>
#include <sampler/sobol.h>
#include <texture/constant.h>
#include <texture/floattexture.h>
#include <texture/rendertarget.h>
#include <util/param.h>
#include <util/parser.h>

#include <omp.h>

#include <cstdint>
#include <memory>
#include <string>
#include <unordered_map>

#include "../../include/orion_gpu.h"
#include "../cpu_bvh.h"

namespace orion {
struct ShimKernelState {
  oracle_bvh::BVH bvh;
  std::vector<std::shared_ptr<Primitive>> prims;
  std::unordered_map<const Primitive*, int> index;
};
extern ShimKernelState* g_last_kernel;
}  // namespace orion

extern "C" void oracle_set_scene_dir(const char* dir);

using namespace orion;

namespace {

std::shared_ptr<Texture> tex(const float* rgb) { return std::make_shared<ConstantTexture>(Spectrum(rgb[0], rgb[1], rgb[2])); }
std::shared_ptr<FloatTexture> ftex(float v) { return std::make_shared<FloatTexture>(v); }

std::shared_ptr<Material> make_material(const orion_material* m) {
  switch (m->type) {
    case ORION_MAT_MATTE:
      return createMatteMaterial(tex(m->Kd), m->has_sigma ? ftex(m->sigma) : nullptr);
    case ORION_MAT_METAL:
      return createMetalMaterial(tex(m->eta_rgb), tex(m->k), ftex(m->roughness), ParamSet());
    case ORION_MAT_MIRROR:
      return createMirrorMaterial(tex(m->Kr));
    case ORION_MAT_GLASS:
      return createGlassMaterial(tex(m->Kr), tex(m->Kt), ftex(m->roughness), ftex(m->eta));
    case ORION_MAT_PLASTIC:
      return createPlasticMaterial(tex(m->Kd), tex(m->Ks), ftex(m->roughness));
    case ORION_MAT_UBER:
      return createUberMaterial(tex(m->Kd), tex(m->Ks), tex(m->Kr), tex(m->Kt), tex(m->opacity), ftex(m->roughness),
                                ftex(m->eta));
    default:
      return nullptr;
  }
}

struct RefScene {
  std::unique_ptr<Parser> parser;
  ShimKernelState* kernel = nullptr;
  int width = 0, height = 0;
};

}  // namespace

extern "C" {

int ref_sobol(const uint64_t* index, const uint32_t* dim, int64_t n, float* out) {
  for (int64_t i = 0; i < n; ++i) out[i] = sobol::sample(index[i], dim[i]);
  return 0;
}

// BSDF at a synthetic hit with frame (ng, ns, u, v): f/pdf for (wi, wo) and
// sample_f for (wo, rnd). `type` is a BxDFType mask (31 = BxDF_ALL).
int ref_bsdf_eval(const orion_material* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                  const float* rnd, int32_t type, float* f_out, float* pdf_out, float* sf_out, float* swi_out,
                  float* spdf_out, int32_t* stype_out, int32_t* nbxdf_out) {
  std::shared_ptr<Material> material = make_material(mat);
  if (!material) return -1;
  for (int64_t i = 0; i < n; ++i) {
    const float* fr = frame + 12 * i;
    Intersection isec;
    isec.ng = Normal3f(fr[0], fr[1], fr[2]);
    isec.ns = Normal3f(fr[3], fr[4], fr[5]);
    isec.u = Vector3f(fr[6], fr[7], fr[8]);
    isec.v = Vector3f(fr[9], fr[10], fr[11]);
    isec.uv = Point2f(0, 0);
    std::shared_ptr<BSDF> bsdf = material->getBSDF(isec, TransportMode::Path);
    Vector3f vo(wo[3 * i], wo[3 * i + 1], wo[3 * i + 2]);
    Vector3f vi(wi[3 * i], wi[3 * i + 1], wi[3 * i + 2]);
    BxDFType t = BxDFType(type);
    Spectrum f = bsdf->f(vi, vo, t);
    f_out[3 * i] = f.r;
    f_out[3 * i + 1] = f.g;
    f_out[3 * i + 2] = f.b;
    pdf_out[i] = bsdf->pdf(vi, vo, t);
    Vector3f swi(0, 0, 0);
    Float spdf = 0;
    BxDFType st = BxDFType(0);
    Spectrum sf = bsdf->sample_f(&swi, vo, Point2f(rnd[2 * i], rnd[2 * i + 1]), &spdf, t, &st);
    sf_out[3 * i] = sf.r;
    sf_out[3 * i + 1] = sf.g;
    sf_out[3 * i + 2] = sf.b;
    swi_out[3 * i] = swi.x;
    swi_out[3 * i + 1] = swi.y;
    swi_out[3 * i + 2] = swi.z;
    spdf_out[i] = spdf;
    stype_out[i] = (int32_t)st;
    nbxdf_out[i] = bsdf->numBxDF(BxDFType(BxDF_ALL & ~BxDF_SPECULAR));
  }
  return 0;
}

void* ref_scene_load(const char* path) {
  std::string p(path);
  size_t slash = p.find_last_of('/');
  std::string dir = slash == std::string::npos ? std::string("./") : p.substr(0, slash + 1);
  oracle_set_scene_dir(dir.c_str());
  RefScene* s = new RefScene();
  s->parser.reset(new Parser(p));
  s->kernel = g_last_kernel;
  auto film = s->parser->getRenderOption()->camera->getFilm();
  s->width = film->getWidth();
  s->height = film->getHeight();
  return s;
}

void ref_scene_free(void* h) { delete static_cast<RefScene*>(h); }

// OpenMP threads of the reference's own parallel loops (1: SPPM's photon
// sums and cell lists in their single-thread order).
void ref_set_threads(int32_t n) { omp_set_num_threads(n > 0 ? n : omp_get_num_procs()); }

// info: width, height, num_prims, num_lights, num_envmaps
int ref_scene_info(void* h, int32_t* info) {
  RefScene* s = static_cast<RefScene*>(h);
  const auto& ro = s->parser->getRenderOption();
  info[0] = s->width;
  info[1] = s->height;
  info[2] = (int32_t)s->kernel->prims.size();
  info[3] = (int32_t)ro->scene->lights.size();
  info[4] = (int32_t)ro->scene->envmaps.size();
  return 0;
}

// World-space corner data per primitive, in primID order, plus the index of
// each primitive's area light in scene.lights (-1 if none) and each light's
// power intensity (the light-selection weight, src/integrator/path.cpp:39-48).
int ref_scene_geometry(void* h, float* p, float* n, float* uv, int32_t* light_of_prim, float* light_power) {
  RefScene* s = static_cast<RefScene*>(h);
  const auto& lights = s->parser->getRenderOption()->scene->lights;
  std::unordered_map<const Light*, int> lid;
  for (size_t i = 0; i < lights.size(); ++i) {
    lid[lights[i].get()] = (int)i;
    light_power[i] = lights[i]->power().intensity();
  }
  const auto& prims = s->kernel->prims;
  for (size_t i = 0; i < prims.size(); ++i) {
    const Triangle& tri = *prims[i]->triangle;
    for (int k = 0; k < 3; ++k) {
      const Point3f& pp = tri.mesh->p[tri.triNumber * 3 + k];
      const Normal3f& nn = tri.mesh->n[tri.triNumber * 3 + k];
      p[9 * i + 3 * k] = pp.x;
      p[9 * i + 3 * k + 1] = pp.y;
      p[9 * i + 3 * k + 2] = pp.z;
      n[9 * i + 3 * k] = nn.x;
      n[9 * i + 3 * k + 1] = nn.y;
      n[9 * i + 3 * k + 2] = nn.z;
      if (tri.mesh->uv.size() > (size_t)(tri.triNumber * 3 + k)) {
        const Point2f& tt = tri.mesh->uv[tri.triNumber * 3 + k];
        uv[6 * i + 2 * k] = tt.x;
        uv[6 * i + 2 * k + 1] = tt.y;
      } else {
        uv[6 * i + 2 * k] = uv[6 * i + 2 * k + 1] = 0.f;
      }
    }
    const AreaLight* al = prims[i]->getAreaLight();
    light_of_prim[i] = al ? lid[al] : -1;
  }
  return 0;
}

// Closest hit through Scene::intersect. rays: n x 8 (o, d, tnear, tfar).
int ref_scene_trace(void* h, int64_t n, const float* rays, float* t, int32_t* prim, float* p, float* ng, float* ns) {
  RefScene* s = static_cast<RefScene*>(h);
  const Scene& scene = *s->parser->getRenderOption()->scene;
#pragma omp parallel for schedule(dynamic, 1024)
  for (int64_t i = 0; i < n; ++i) {
    const float* r = rays + 8 * i;
    Ray ray(Point3f(r[0], r[1], r[2]), Vector3f(r[3], r[4], r[5]), r[6], r[7]);
    Intersection isec;
    if (scene.intersect(ray, &isec)) {
      t[i] = isec.t;
      prim[i] = s->kernel->index.at(isec.primitive);
      p[3 * i] = isec.p.x;
      p[3 * i + 1] = isec.p.y;
      p[3 * i + 2] = isec.p.z;
      ng[3 * i] = isec.ng.x;
      ng[3 * i + 1] = isec.ng.y;
      ng[3 * i + 2] = isec.ng.z;
      ns[3 * i] = isec.ns.x;
      ns[3 * i + 1] = isec.ns.y;
      ns[3 * i + 2] = isec.ns.z;
    } else {
      t[i] = 0.f;
      prim[i] = -1;
    }
  }
  return 0;
}

// The reference's own Integrator::render() (src/integrator/path.cpp:15-37)
// with the scene's XML spp; returns the film's FP32 per-pixel sums.
int ref_scene_render(void* h, float* rgb_sum) {
  RefScene* s = static_cast<RefScene*>(h);
  const auto& ro = s->parser->getRenderOption();
  ro->integrator->render(*ro->scene);
  auto film = ro->camera->getFilm();
  for (int j = 0; j < s->height; ++j)
    for (int i = 0; i < s->width; ++i) {
      Spectrum v = film->sample(i, j);
      size_t o = 3 * ((size_t)j * s->width + i);
      rgb_sum[o] = v.r;
      rgb_sum[o + 1] = v.g;
      rgb_sum[o + 2] = v.b;
    }
  return 0;
}

// Per-pixel estimates with the reference's camera, sampler and Li over the
// sample indices k*W*H + j*W + i for k in [k0, k0+spp) (src/integrator/path.cpp:22-29),
// accumulated in FP64: sum and sum of squares per channel.
int ref_scene_render_pixels(void* h, int64_t npix, const int32_t* pix, int32_t k0, int32_t spp, double* sum,
                            double* sumsq, int32_t threads) {
  RefScene* s = static_cast<RefScene*>(h);
  const auto& ro = s->parser->getRenderOption();
  ro->integrator->preprocess(*ro->scene, *ro->sampler);
  const int64_t WH = (int64_t)s->width * s->height;
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1)
  for (int64_t q = 0; q < npix; ++q) {
    int i = pix[2 * q], j = pix[2 * q + 1];
    double a[3] = {0, 0, 0}, b[3] = {0, 0, 0};
    for (int k = k0; k < k0 + spp; ++k) {
      std::unique_ptr<Sampler> smp = ro->sampler->clone((int64_t)k * WH + (int64_t)j * s->width + i);
      Ray ray = ro->camera->generateRay(Point2f((Float)i, (Float)j), *smp);
      Spectrum L = ro->integrator->Li(ray, *ro->scene, *smp);
      double c[3] = {L.r, L.g, L.b};
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

// Camera rays for sample indices (src/camera/pinhole.cpp:8-33): rays n x 6.
int ref_scene_camera_rays(void* h, int64_t n, const int64_t* sample_index, float* rays) {
  RefScene* s = static_cast<RefScene*>(h);
  const auto& ro = s->parser->getRenderOption();
  const int64_t WH = (int64_t)s->width * s->height;
  for (int64_t q = 0; q < n; ++q) {
    int64_t idx = sample_index[q];
    int64_t pixel = idx % WH;
    int i = (int)(pixel % s->width), j = (int)(pixel / s->width);
    std::unique_ptr<Sampler> smp = ro->sampler->clone(idx);
    Ray ray = ro->camera->generateRay(Point2f((Float)i, (Float)j), *smp);
    float* r = rays + 6 * q;
    r[0] = ray.o.x;
    r[1] = ray.o.y;
    r[2] = ray.o.z;
    r[3] = ray.d.x;
    r[4] = ray.d.y;
    r[5] = ray.d.z;
  }
  return 0;
}

}  // extern "C"
