// Internal hooks between the C ABI implementation (capi.cpp) and the
// serving loop (server.cpp). Not part of the public ABI.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>

#include "../../include/orion_gpu.h"

namespace orion_gb300 {

// A render job whose film lives in device memory owned by the caller.
struct DeviceFilmJob {
  orion_scene_id scene;
  orion_render_params params;   // spp, max_depth, rr_depth, first_pass
  const orion_camera* camera;   // or NULL
  double* sum;                  // device W*H*3, accumulated into (not cleared)
  double* sumsq;                // device W*H*3
  unsigned int* count;          // device W*H
};

// One batched launch over `jobs`, adding into their device films.
int ctx_run_device_jobs(orion_gpu_ctx* ctx, const DeviceFilmJob* jobs, int njobs, double* device_ms, int64_t* paths);
int ctx_device(orion_gpu_ctx* ctx);
cudaStream_t ctx_stream(orion_gpu_ctx* ctx);
// Film size, spp and depth of a resident scene.
int ctx_scene_info(orion_gpu_ctx* ctx, orion_scene_id id, int* width, int* height, int* spp, int* max_depth);
// Bytes of the shared path-slot pool currently allocated.
int64_t ctx_pool_bytes(orion_gpu_ctx* ctx);
// Device -> host copy ordered after all work queued on the context's stream.
int ctx_copy_to_host(orion_gpu_ctx* ctx, void* dst, const void* src, size_t bytes);
// 8-bit preview (B, G, R, 255 per pixel) of a device film laid out as sums
// (W*H*3 doubles), sums of squares, counts (W*H uint32), into host `bgra`.
int ctx_film_preview(orion_gpu_ctx* ctx, const void* film, int width, int height, int bottom_up, uint8_t* bgra);
// Records an error message for orion_last_error() and returns `code`.
int ctx_fail(int code, const char* msg);

// Fixed trace scratch of orion_gpu_trace_noalloc (noalloc.cu): the device's
// array address (looked up once per device; returns a cudaError_t) and its
// sections.
int noalloc_trace_scratch(int device, unsigned char** out, std::string* err);
void noalloc_trace_layout(unsigned char* base, float** rays, float** t, float** u, float** v, int** prim);

}  // namespace orion_gb300
