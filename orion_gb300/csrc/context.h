// Internal to the C-ABI sources (capi*.cpp): the host scene handle, the
// device context and the helpers they share. Not part of the ABI.
#pragma once
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <vector>

#include "../../include/orion_gpu.h"
#include "bvh_build.h"
#include "internal.h"
#include "kernels.h"
#include "scene_host.h"
#include "scene_prep.h"

struct orion_host_scene {
  orion_gb300::HostScene s;
  // Host BVH and device records, built on the first upload and reused by
  // later uploads of the same scene (resident-scene serving, re-uploads).
  std::unique_ptr<orion_gb300::BvhBuild> bvh;
  std::unique_ptr<orion_gb300::PreparedScene> prep;
  std::vector<uint8_t> tri_class;  // leaf order -> shading class
  unsigned class_mask = 0;
  // The upload arrays above are page-locked once (portable across contexts)
  // so every upload copies at DMA speed; unlocked when the scene is freed.
  std::vector<void*> pinned;
  std::mutex mu;
  ~orion_host_scene() {
    for (void* p : pinned) cudaHostUnregister(p);
  }
};

namespace orion_gb300 {

// Records `msg` as this thread's last error (orion_last_error) and returns `code`.
int fail(int code, const std::string& msg);

// Returns the unused memory every context's scene pool keeps (released scenes)
// to the device, so that a cudaMalloc that ran out of memory can be retried.
void trim_scene_pools();

#define CUDA_TRY(call)                                                                                 \
  do {                                                                                                 \
    cudaError_t e_ = (call);                                                                           \
    if (e_ != cudaSuccess) return fail(ORION_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

// A named NVTX range over a scope: the entry points mark their host work so a
// timeline profiler shows renders, uploads and batches beside the kernels
// (header-only NVTX: a no-op unless a profiler is attached).
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

#define RC(x)                        \
  do {                               \
    int rc_ = (x);                   \
    if (rc_ != ORION_OK) return rc_; \
  } while (0)

struct DevBuf {
  void* p = nullptr;
  size_t bytes = 0;
  // Non-null: p came from a memory pool in this stream's order (alloc_pooled)
  // and goes back to it in the same order, without a device-wide sync.
  cudaStream_t pool_stream = nullptr;
  ~DevBuf() { release(); }
  void release() {
    if (p) {
      if (pool_stream)
        cudaFreeAsync(p, pool_stream);
      else
        cudaFree(p);
    }
    p = nullptr;
    bytes = 0;
    pool_stream = nullptr;
  }
  int alloc(size_t n) {
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMalloc(&p, n);
    if (e == cudaErrorMemoryAllocation) {  // memory of released scenes may still sit in a pool
      cudaGetLastError();
      trim_scene_pools();
      e = cudaMalloc(&p, n);
    }
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(e == cudaErrorMemoryAllocation ? ORION_ERR_NOMEM : ORION_ERR_CUDA,
                  std::string("cudaMalloc(") + std::to_string(n) + "): " + cudaGetErrorString(e));
    }
    bytes = n;
    return ORION_OK;
  }
  // From `pool`, in the order of stream `s` (usable by work later on `s`).
  int alloc_pooled(size_t n, cudaMemPool_t pool, cudaStream_t s) {
    release();
    if (n == 0) n = 16;
    cudaError_t e = cudaMallocFromPoolAsync(&p, n, pool, s);
    if (e != cudaSuccess) {
      p = nullptr;
      return fail(e == cudaErrorMemoryAllocation ? ORION_ERR_NOMEM : ORION_ERR_CUDA,
                  std::string("cudaMallocFromPoolAsync(") + std::to_string(n) + "): " + cudaGetErrorString(e));
    }
    bytes = n;
    pool_stream = s;
    return ORION_OK;
  }
  template <class T>
  T* as() const {
    return static_cast<T*>(p);
  }
};

struct DeviceScene {
  DevBuf nodes, woop, tri_prim, tri_class, prims, mats, lights, lfunc, lcdf, env_data, envmaps;
  DevBuf mat_src, textures, prim_uv;  // image textures (empty when no material is textured)
  SceneView view{};
  int64_t bytes = 0;
  int64_t num_prims = 0;
  int width = 0, height = 0, spp = 1, max_depth = 5;
  int bvh_depth = 0;
  unsigned class_mask = 1u << SC_MISS;  // shading classes of the scene's triangles, and misses
  orion_sppm_params sppm{0, 0, 0.f, 0};  // the scene's <Integrator type="sppm"> parameters
};

constexpr int kMaxWaveStreams = 4;  // plain-render waves in flight at once

// A captured device-side loop of one batch mode (pooled or waves).
struct BatchGraph {
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  const void* key[4] = {nullptr, nullptr, nullptr, nullptr};  // buffers the graph was captured with
  LaunchConfig cfg{};
  int slots = 0;
  unsigned mask = 0;  // shading classes the captured loop launches
  void drop() {
    if (exec) cudaGraphExecDestroy(exec);
    if (graph) cudaGraphDestroy(graph);
    exec = nullptr;
    graph = nullptr;
  }
};

// One batch engine: its free and retire lists, control block, job table and
// captured device-side loops (the path slots are a Wave).
struct BatchEngine {
  DevBuf retire, free_list, ctl, jobs;
  int slots_alloc = 0, jobs_alloc = 0;
  BatchGraph loop[2];  // [ORION_BATCH_POOLED], [ORION_BATCH_WAVES]
  void drop_graph() {
    for (BatchGraph& g : loop) g.drop();
  }
};

struct Wave {
  int capacity = 0;
  DevBuf block;  // all per-path arrays in one allocation
  WaveView view{};
};

}  // namespace orion_gb300

struct orion_gpu_ctx {
  using DevBuf = orion_gb300::DevBuf;
  using Wave = orion_gb300::Wave;
  using BatchEngine = orion_gb300::BatchEngine;
  using DeviceScene = orion_gb300::DeviceScene;
  int device = 0;
  cudaStream_t stream = nullptr;
  int num_sms = 0;
  // Resident scenes' arrays come from this pool in the order of `stream`:
  // uploading and releasing scenes (serving evicts and re-uploads them) then
  // reuses the memory with no cudaMalloc or device-wide cudaFree sync.
  cudaMemPool_t scene_pool = nullptr;
  DevBuf sobol;  // Sobol tables: per dimension and index byte, the XOR of every byte value's direction numbers
  std::map<int, std::unique_ptr<DeviceScene>> scenes;
  int next_id = 1;
  Wave wave;
  // Plain renders overlap consecutive waves on up to kWaveStreams streams:
  // per extra stream its wave state, the stream, its join event; the events
  // that order the film writes wave after wave.
  static constexpr int kWaveStreams = orion_gb300::kMaxWaveStreams;
  // Four: the eight-sphere 1080p render (eight waves) 2583 -> 2822 Mpaths/s
  // against two. Renders of fewer than two full waves are split two ways
  // only (render_impl).
  int wave_streams = 4;
  // Pooled or wave-mode batch engines running at once (at most kBatchEngines):
  // orion_gpu_set_config sets min(streams, kBatchEngines), the batch
  // autotuner tunes it alone, so tuning batches leaves plain renders' waves be.
  int batch_engines = 2;
  Wave xwave[kWaveStreams - 1];
  cudaStream_t xstream[kWaveStreams - 1] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[kWaveStreams - 1] = {}, ev_film[kWaveStreams] = {};
  DevBuf film_sum, film_count, film64, filmsq64;
  int64_t film_pixels = 0;
  int64_t budget = 0;
  orion_render_stats last{};
  orion_gb300::LaunchConfig cfg{};
  // Large waves amortise each bounce's kernel tails over more paths, and two
  // waves in flight fill the tails that remain (1024x1024 x 64 spp displaced
  // sphere: 449 Mpaths/s with one stream of 4M-path waves, 708 with two
  // streams of 32M, same traversal).
  int default_wave = 1 << 25;
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  bool profiling = false;
  bool count_work = false;  // plain renders count BVH node visits and triangle tests
  orion_traversal_work last_work{};
  std::vector<cudaEvent_t> prof_events;
  std::vector<int> prof_stage;
  orion_stage_times stage_times{};
  // batched mode
  int default_batch_slots = 1 << 24;  // pooled: path slots; waves: paths per wave
  DevBuf b_films;
  DevBuf b_films32;  // FP32 copies of batch films for read-back (orion_job.sum32)
  // Pooled batch engines: a batch's jobs are split between as many as the
  // `streams` knob allows (at most kBatchEngines) and they run concurrently,
  // engine e on the wave state and stream of wave slot e.
  static constexpr int kBatchEngines = 2;
  BatchEngine beng[kBatchEngines];
  int batch_mode = ORION_BATCH_WAVES;
  // SPPM: per-pixel state in one block, the grid's cell lists apart
  DevBuf sppm_block, sppm_hits;
  DevBuf preview;  // 8-bit previews of server films
  int smem_limit = 48 * 1024;  // opt-in dynamic shared memory per block
  orion_gb300::KernelLimits limits{1024, 1024};
  std::mutex mu;
};

namespace orion_gb300 {

// Why a launch configuration cannot run on this context ("" if it can).
std::string config_problem(const orion_gpu_ctx* ctx, const LaunchConfig& c);
// Path-state block of `capacity` slots (grows only).
int alloc_wave(Wave& wave, int capacity);

}  // namespace orion_gb300
