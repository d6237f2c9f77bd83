// GpuPathTracing: the integrator a maintainer adds to the reference renderer
// so that `integrator->render(*scene)` (src/main.cpp:15) renders on the GB300
// library through its C ABI (include/orion_gpu.h). It is the adapter
// INTEGRATION.md describes, compiled here against the reference's own headers
// and linked with the reference's objects and liborion_gb300.so, which proves
// that it builds; it is not part of the oracle's checks.
//
// It stands in for PathTracing (src/integrator/path.h:16-36): same
// constructor inputs (camera, sampler, maxDepth, nSamplesPerPixel from the
// <Integrator> ParamSet, src/integrator/path.cpp:108-113) plus the scene
// file's path, which the GPU library loads with its own parser
// (orion_scene_load_ori reproduces the reference parser's primitives,
// materials, lights and camera). The reference-side edits that select it:
//   src/util/parser.h      RenderOption gains `std::string path;`
//   src/util/parser.cpp    Parser::Parser stores the path in renderOption->path;
//                          _makeIntegrator: `else if (inte == "gpupath")
//                          renderOption->integrator = createGpuPathTracingIntegrator(
//                              renderOption->camera, renderOption->sampler, ps,
//                              renderOption->path);`
// Errors follow the reference's convention (CHECK_INFO prints and continues,
// src/orion.h:33-37); ok() tells a caller whether the device path is usable.
#include <core/camera.h>
#include <core/integrator.h>
#include <texture/rendertarget.h>
#include <util/param.h>
#include <util/strutil.h>

#include <memory>
#include <string>
#include <vector>

#include "../../include/orion_gpu.h"

ORION_NAMESPACE_BEGIN

class GpuPathTracing : public Integrator {
 public:
  GpuPathTracing(const std::shared_ptr<Camera>& camera, const std::shared_ptr<Sampler>& sampler,
                 const std::string& scenePath, int maxDepth, int nSamples)
      : Integrator(camera, sampler), maxDepth_(maxDepth), nSamples_(nSamples) {
    orion_gpu_opts opts = {0, 0, 0, nullptr};
    ok_ = check(orion_gpu_create(&opts, &ctx_), "orion_gpu_create") &&
          check(orion_scene_load_ori(scenePath.c_str(), &host_), "orion_scene_load_ori") &&
          check(orion_gpu_scene_upload(ctx_, host_, &id_), "orion_gpu_scene_upload");
  }
  ~GpuPathTracing() override {
    if (ctx_) orion_gpu_destroy(ctx_);
    if (host_) orion_scene_free(host_);
  }

  bool ok() const { return ok_; }

  // PathTracing::render (src/integrator/path.cpp:15-37) on the device: the
  // film sums of all nSamples passes, in sample order, then one accumulate
  // of sum / nSamples per pixel, so getAveraged() (rendertarget.cpp:28-37)
  // returns the same sum / nSamples the CPU path's film gives.
  void render(const Scene&) override {
    if (!ok_) return;
    std::shared_ptr<RenderTarget> film = camera->getFilm();
    const int W = film->getWidth(), H = film->getHeight();
    std::vector<float> sum(3 * (size_t)W * H);
    orion_render_params p = {};
    p.spp = nSamples_;
    p.max_depth = maxDepth_;
    p.rr_depth = 3;  // `bounces > 3` (src/integrator/path.cpp:91)
    if (!check(orion_gpu_render(ctx_, id_, &p, sum.data(), nullptr), "orion_gpu_render")) return;
    for (int j = 0; j < H; ++j)
      for (int i = 0; i < W; ++i) {
        const float* s = &sum[3 * ((size_t)j * W + i)];
        film->acumulate(i, j, Spectrum(s[0], s[1], s[2]) / nSamples_);
      }
  }

 private:
  static bool check(int rc, const char* what) {
    CHECK_INFO(rc == ORION_OK, std::string(what) + ": " + orion_last_error());
    return rc == ORION_OK;
  }

  orion_gpu_ctx* ctx_ = nullptr;
  orion_host_scene* host_ = nullptr;
  orion_scene_id id_ = 0;
  int maxDepth_, nSamples_;
  bool ok_ = false;
};

// Factory in the shape of createPathTracingIntegrator (src/integrator/path.cpp:108-113).
std::shared_ptr<Integrator> createGpuPathTracingIntegrator(const std::shared_ptr<Camera>& camera,
                                                           const std::shared_ptr<Sampler>& sampler,
                                                           const ParamSet& param, const std::string& scenePath) {
  return std::make_shared<GpuPathTracing>(camera, sampler, scenePath, parseInt(param.getParam("maxDepth")),
                                          parseInt(param.getParam("nSamplesPerPixel")));
}

bool gpuPathTracingReady(const Integrator& integrator) {
  const GpuPathTracing* g = dynamic_cast<const GpuPathTracing*>(&integrator);
  return g != nullptr && g->ok();
}

ORION_NAMESPACE_END
