// Host-callable launchers for the wavefront kernels (kernels.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "device_types.h"

namespace orion_gb300 {

// A resident scene, as the kernels see it.
struct SceneView {
  const float4* nodes;
  const float4* woop;
  const int* tri_prim;
  const PrimShade* prims;
  const DevMaterial* mats;
  const DevLight* lights;
  const float* light_func;
  const float* light_cdf;
  float light_func_int;
  int num_lights;
  int env_idx[8];
  int num_env;
  float world_radius;
  DevCamera cam;
};

// Device path state for one wave of `capacity` paths (structure of arrays).
struct WaveView {
  float4* ray_o;     // o.xyz
  float4* ray_d;     // d.xyz
  float4* beta;      // beta.rgb, w = 1 after a specular bounce
  float4* L;         // radiance so far
  int* dim;          // Sobol dimension counter
  float4* hit;       // t, u, v, leaf triangle (int bits; -1 miss)
  float4* nee_p;     // shading point xyz, light-selection pdf
  float4* nee_beta;  // beta before the bounce, w = flags | light << 8 (int bits)
  float4* nee_ld;    // light-sample contribution rgb, w = BSDF-sample pdf
  float4* nee_f;     // BSDF-sample f * |cos| rgb, w = MIS weight for environment lights
  float4* sh_o;      // shadow ray origin, w = tmax
  float4* sh_d;
  float4* mis_o;
  float4* mis_d;
  float4* mis_hit;
  int* occluded;
  int* q_ext[2];     // extension-ray queues (current / next bounce)
  int* q_nee;        // paths that sampled a light this bounce
  int* q_sh;         // shadow rays
  int* q_mis;        // BSDF-sampled rays towards a non-delta light
  int* counters;     // kCounterSlots ints
  unsigned long long* ray_stats;  // ext, shadow, mis
  int* error_word;
  int capacity;
};

enum CounterSlot { CNT_EXT0 = 0, CNT_EXT1 = 1, CNT_NEE = 2, CNT_SH = 3, CNT_MIS = 4, kCounterSlots = 8 };

struct WaveArgs {
  const uint32_t* sobol;
  int64_t base_index;  // sample index of path slot 0
  int n_paths;
  int width, height;
  int max_depth;
  int rr_depth;
};

struct FilmView {
  float* sum;        // W*H*3
  uint32_t* count;   // W*H
  double* sum64;     // W*H*3 or null
  double* sumsq64;   // W*H*3 or null
};

struct LaunchConfig {
  int num_sms;
  int trace_block;   // threads per block of the trace kernels
  int shade_block;
  int blocks_per_sm; // persistent grid size factor
  int smem_stack;    // shared-memory stack entries per thread (0, 8, 16, 24, 32)
};

enum Stage { ST_CAMERA = 0, ST_TRACE_EXT, ST_SHADE, ST_TRACE_SHADOW, ST_TRACE_MIS, ST_RESOLVE, ST_FILM, ST_OTHER,
             kNumStages };

// Optional per-kernel timing: event pairs recorded around every launch.
struct StageTimer {
  cudaEvent_t* events;  // 2 * capacity events
  int* stage;           // capacity
  int capacity;
  int used;
  void begin(int st, cudaStream_t s) {
    if (used < capacity) {
      stage[used] = st;
      cudaEventRecord(events[2 * used], s);
    }
  }
  void end(cudaStream_t s) {
    if (used < capacity) cudaEventRecord(events[2 * used + 1], s);
    ++used;
  }
};

// One full wave: camera rays, then (trace, shade, shadow/MIS trace,
// resolve) per bounce, then film accumulation. All on `stream`, no host sync.
void launch_wave(const SceneView& s, const WaveView& w, const WaveArgs& a, const FilmView& film,
                 const LaunchConfig& cfg, cudaStream_t stream, int* launches, StageTimer* timer = nullptr);

// Component hooks for the parity tests.
void launch_sobol(const uint32_t* sobol, int64_t n, const uint64_t* index, const uint32_t* dim, float* out,
                  cudaStream_t stream);
void launch_trace(const SceneView& s, int64_t n, const float* rays, int any_hit, float* t, float* u, float* v,
                  int* prim, const LaunchConfig& cfg, cudaStream_t stream);
void launch_camera_rays(const SceneView& s, const uint32_t* sobol, int64_t n, const int64_t* index, float* rays,
                        cudaStream_t stream);
void launch_bsdf_eval(const DevMaterial* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                      const float* rnd, int type, float* f, float* pdf, float* sf, float* swi, float* spdf,
                      int* stype, int* nbxdf, cudaStream_t stream);

}  // namespace orion_gb300
