// C ABI, stochastic progressive photon mapping (include/orion_gpu.h:
// orion_gpu_render_sppm). Follows SPPMIntegrator::render
// (src/integrator/sppm.cpp); the kernels are in sppm.cu.
#include <cuda_runtime.h>

#include <algorithm>
#include <string>

#include "context.h"

using namespace orion_gb300;

extern "C" int orion_gpu_render_sppm(orion_gpu_ctx* ctx, orion_scene_id id, const orion_sppm_params* params,
                                     float* film_rgb_sum, uint32_t* film_count) {
  if (!ctx || !film_rgb_sum) return fail(ORION_ERR_INVALID, "null argument");
  NvtxRange range("orion_gpu_render_sppm");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  const DeviceScene& d = *it->second;
  const orion_sppm_params p = params ? *params : d.sppm;
  if (p.iterations <= 0) return fail(ORION_ERR_INVALID, "sppm: iterations must be positive");
  if (p.max_depth < 0 || p.max_depth > 1024) return fail(ORION_ERR_INVALID, "sppm: max_depth out of range");
  if (!(p.initial_radius > 0.f)) return fail(ORION_ERR_INVALID, "sppm: initial radius must be positive");
  // SPPM::render requires a light (CHECK_INFO, src/integrator/sppm.cpp:72-73).
  if (d.view.num_lights == 0) return fail(ORION_ERR_INVALID, "sppm: the scene has no light");
  const int W = d.view.cam.width, H = d.view.cam.height;
  const int64_t npix = (int64_t)W * H;
  const int64_t photons = p.photons_per_iter < 0 ? npix : p.photons_per_iter;
  const int64_t hits_cap = photons * std::max(1, p.max_depth - 1);  // hits after each photon's first
  if (npix <= 0 || npix > (1 << 28) || hits_cap > INT32_MAX) return fail(ORION_ERR_INVALID, "sppm: size out of range");
  if ((int64_t)p.iterations * (npix + photons) >= (1LL << 52))
    return fail(ORION_ERR_INVALID, "sppm: sample indices exceed the Sobol matrices");
  cudaStream_t st = ctx->stream;

  // Per-pixel state, 16-byte aligned pieces of one allocation.
  const int nparts = kSppmBoundsBlocks;
  const int nscan = (int)((npix + 1 + kScanBlock - 1) / kScanBlock);
  struct Piece {
    void** dst;
    size_t bytes;
  };
  SppmView v{};
  float4* f4s[9];
  std::vector<Piece> pieces;
  for (int k = 0; k < 9; ++k) pieces.push_back({(void**)&f4s[k], sizeof(float4) * (size_t)npix});
  pieces.push_back({(void**)&v.phi, sizeof(float) * 3 * (size_t)npix});
  pieces.push_back({(void**)&v.m, sizeof(int) * (size_t)npix});
  pieces.push_back({(void**)&v.cell_start, sizeof(int) * ((size_t)npix + 1)});
  pieces.push_back({(void**)&v.cell_fill, sizeof(int) * (size_t)npix});
  pieces.push_back({(void**)&v.scan_part, sizeof(int) * (size_t)nscan});
  pieces.push_back({(void**)&v.part_lo, sizeof(float4) * (size_t)nparts});
  pieces.push_back({(void**)&v.part_hi, sizeof(float4) * (size_t)nparts});
  pieces.push_back({(void**)&v.grid, sizeof(SppmGrid)});
  pieces.push_back({(void**)&v.film, sizeof(float) * 3 * (size_t)npix});
  pieces.push_back({(void**)&v.film_count, sizeof(unsigned) * (size_t)npix});
  pieces.push_back({(void**)&v.rays, sizeof(unsigned long long)});
  pieces.push_back({(void**)&v.hit_count, sizeof(int)});
  size_t total = 0;
  for (const Piece& pc : pieces) total += (pc.bytes + 255) & ~(size_t)255;
  if (ctx->sppm_block.bytes < total) RC(ctx->sppm_block.alloc(total));
  {
    char* base = static_cast<char*>(ctx->sppm_block.p);
    for (const Piece& pc : pieces) {
      *pc.dst = base;
      base += (pc.bytes + 255) & ~(size_t)255;
    }
  }
  v.vp_pr = f4s[0], v.vp_wo = f4s[1], v.vp_beta = f4s[2], v.vp_ns = f4s[3], v.vp_ng = f4s[4];
  v.vp_su = f4s[5], v.vp_sv = f4s[6], v.ld = f4s[7], v.tau = f4s[8];
  v.width = W;
  v.height = H;
  v.npix = (int)npix;
  v.max_depth = p.max_depth;
  v.iterations = p.iterations;
  v.photons = (int)photons;
  v.sobol = ctx->sobol.as<uint32_t>();
  // Photon hits (3 float4) as recorded and in hash-cell order, one block.
  const size_t hit_bytes = ((size_t)hits_cap * 3 * sizeof(float4) + 255) & ~(size_t)255;
  if (ctx->sppm_hits.bytes < 2 * hit_bytes) RC(ctx->sppm_hits.alloc(2 * hit_bytes));
  v.hits = ctx->sppm_hits.as<float4>();
  v.by_cell = reinterpret_cast<float4*>(static_cast<char*>(ctx->sppm_hits.p) + hit_bytes);
  v.hits_cap = (int)hits_cap;

  launch_sppm_init(v, p.initial_radius, st);
  CUDA_TRY(cudaMemsetAsync(v.rays, 0, sizeof(unsigned long long), st));
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaEventRecord(ctx->ev0, st));
  int64_t launches = 1;
  for (int iter = 0; iter < p.iterations; ++iter) {
    launch_sppm_visible_points(d.view, v, iter, st);
    launch_sppm_photons(d.view, v, iter, st);
    CUDA_TRY(cudaGetLastError());
    launches += 10;
  }
  CUDA_TRY(cudaEventRecord(ctx->ev1, st));
  unsigned long long rays = 0;
  CUDA_TRY(cudaMemcpyAsync(film_rgb_sum, v.film, sizeof(float) * 3 * (size_t)npix, cudaMemcpyDeviceToHost, st));
  if (film_count)
    CUDA_TRY(cudaMemcpyAsync(film_count, v.film_count, sizeof(uint32_t) * (size_t)npix, cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaMemcpyAsync(&rays, v.rays, sizeof(rays), cudaMemcpyDeviceToHost, st));
  CUDA_TRY(cudaStreamSynchronize(st));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->last = orion_render_stats{};
  ctx->last.paths = npix * p.iterations + photons * p.iterations;
  ctx->last.rays = (int64_t)rays;
  ctx->last.ext_rays = (int64_t)rays;
  ctx->last.kernel_launches = launches;
  ctx->last.device_ms = ms;
  return ORION_OK;
}
