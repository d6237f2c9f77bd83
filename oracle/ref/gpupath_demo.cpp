// The reference's main() (src/main.cpp) with the GPU integrator in place of
// the parser's: parse a scene file with the reference Parser, build
// GpuPathTracing from the same camera, sampler and <Integrator> parameters,
// render, and write the averaged film with the reference's saveAsBmp.
//   gpupath_demo scene.ori out.bmp
// Exit status: 0 rendered; 3 the GPU library could not start (its message is
// printed), e.g. on a machine without a CUDA device.
#include <core/camera.h>
#include <core/texture.h>
#include <texture/rendertarget.h>
#include <util/param.h>
#include <util/parser.h>

#include <cstdio>
#include <string>

ORION_NAMESPACE_BEGIN
std::shared_ptr<Integrator> createGpuPathTracingIntegrator(const std::shared_ptr<Camera>& camera,
                                                           const std::shared_ptr<Sampler>& sampler,
                                                           const ParamSet& param, const std::string& scenePath);
bool gpuPathTracingReady(const Integrator& integrator);
ORION_NAMESPACE_END

using namespace orion;

int main(int argc, char** argv) {
  if (argc != 5) {
    std::fprintf(stderr, "usage: gpupath_demo scene.ori maxDepth nSamplesPerPixel out.bmp\n");
    return 2;
  }
  Parser parser(argv[1]);
  auto& option = parser.getRenderOption();
  ParamSet ps;
  ps.setParam("maxDepth", argv[2]);
  ps.setParam("nSamplesPerPixel", argv[3]);
  auto integrator = createGpuPathTracingIntegrator(option->camera, option->sampler, ps, argv[1]);
  if (!gpuPathTracingReady(*integrator)) return 3;
  integrator->render(*option->scene);
  auto film = option->camera->getFilm()->getAveraged();
  return saveAsBmp(film.get(), argv[4]) ? 0 : 1;
}
