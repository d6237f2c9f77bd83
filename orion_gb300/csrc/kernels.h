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
  const uint8_t* tri_class;  // leaf order -> ShadeClass of the triangle's material
  const PrimShade* prims;
  const DevMaterial* mats;
  const DevLight* lights;
  const DevEnvMap* envmaps;  // image environment maps (DevLight::image)
  const DevTexture* textures;      // image textures (DevMaterialSrc::tex)
  const DevMaterialSrc* mat_src;   // builder inputs per material (null when nothing is textured)
  const float* prim_uv;            // texture coordinates, 6 per primitive (null when nothing is textured)
  const float* light_func;
  const float* light_cdf;
  float light_func_int;
  int num_lights;
  int env_idx[8];
  int num_env;
  int num_area_lights;
  float world_radius;
  float world_center[3];  // Bounds3::boundingSphere (distant and environment photons)
  unsigned class_mask;  // shading classes of the scene's triangles (bit ShadeClass), SC_MISS always
  DevCamera cam;
};

// One field of an array of per-path records, seen as an array of its own
// (STRIDE: record size in units of T).
template <class T, int STRIDE>
struct FieldView {
  T* p;
  ORION_HD inline T& operator[](int64_t i) const { return p[i * STRIDE]; }
};

// Per-path state, one 96-byte record (three 32-byte sectors) per path slot,
// so a kernel that reaches a path through a scattered slot index moves whole
// sectors: [o, d] (what a trace reads), [beta, L], [hit, meta].
struct PathRec {
  float4 o;     // ray origin; w unused
  float4 d;     // ray direction; w unused
  float4 beta;  // throughput; w = 1 after a specular bounce
  float4 L;     // radiance so far; w = batched mode: sample index, low 32 bits
  float4 hit;   // t, u, v, primitive (int bits; -1 miss)
  int4 meta;    // Sobol dimension counter; batched mode: job, bounce, sample index high 32 bits
};
static_assert(sizeof(PathRec) == 96, "PathRec is three sectors");

// Next-event-estimation record of a path, 128 bytes: written whole by the
// shading kernel; the shadow trace reads [sh_o, sh_d], the MIS trace
// [mis_o, mis_d], the resolve kernel the first two sectors.
struct NeeRec {
  float4 p;      // shading point xyz, light-selection pdf
  float4 beta;   // beta before the bounce, w = flags | light << 8 (int bits)
  float4 ld;     // light-sample contribution rgb, w = BSDF-sample pdf
  float4 f;      // BSDF-sample f * |cos| rgb, w = MIS weight for environment lights
  float4 sh_o;   // shadow ray origin, w = tmax
  float4 sh_d;
  float4 mis_o;
  float4 mis_d;
};
static_assert(sizeof(NeeRec) == 128, "NeeRec is four sectors");

using RecF4 = FieldView<float4, sizeof(PathRec) / sizeof(float4)>;
using RecI = FieldView<int, sizeof(PathRec) / sizeof(int)>;
using NeeF4 = FieldView<float4, sizeof(NeeRec) / sizeof(float4)>;
using F4 = FieldView<float4, 1>;

// Device path state for one wave of `capacity` paths.
struct WaveView {
  PathRec* rec;
  NeeRec* nee;
  RecF4 ray_o, ray_d, beta, L, hit;                          // fields of rec
  RecI dim, job, bounce, index_hi;                           // rec.meta
  NeeF4 nee_p, nee_beta, nee_ld, nee_f, sh_o, sh_d, mis_o, mis_d;  // fields of nee
  float4* mis_hit;   // MIS ray hit: t, u, v, primitive
  int* occluded;
  int* mis_occluded;  // MIS ray towards an environment light: anything hit
  int* q_mis_env;     // MIS rays towards an environment light (occlusion queries)
  int* q_ext[2];     // extension-ray queues (current / next bounce)
  int* q_nee;        // paths that sampled a light this bounce
  int* q_sh;         // shadow rays
  int* q_mis;        // BSDF-sampled rays towards a non-delta light
  int* q_cls;        // extension hits by shading class: kShadeClasses queues of `capacity`
  int* counters;     // kCounterSlots ints
  unsigned long long* ray_stats;  // ext, shadow, mis
  // Null, or (a counting render) 6 counters the trace kernels add to: node
  // visits of the extension, shadow and MIS rays, then their triangle tests.
  unsigned long long* trace_work;
  int* error_word;
  // Plain renders: per slot, the queues its shading appended it to this
  // bounce (kQueueFlag* bits); k_compact_queues turns them into the queues,
  // in slot order, and clears them.
  uint8_t* qflags;
  int capacity;
};

// Bits of WaveView::qflags: the queues a shaded path goes to.
enum QueueFlag { kQfExt = 1, kQfNee = 2, kQfShadow = 4, kQfMis = 8, kQfMisEnv = 16 };

// Bits of a launch's error word (plain renders: WaveView::error_word; batches: BatchCtl::error).
constexpr int kErrIterationCap = 1;    // a batch loop reached its iteration bound
constexpr int kErrTraversalStack = 2;  // a traversal needed more stack entries than its capacity
// Stack capacity of the test-only trace kernels (orion_gpu_set_test_limits).
constexpr int kTestStackEntries = 2;

enum CounterSlot { CNT_EXT0 = 0, CNT_EXT1 = 1, CNT_NEE = 2, CNT_SH = 3, CNT_MIS = 4, CNT_RETIRE = 5, CNT_FREE = 6,
                   CNT_FETCH_EXT = 8, CNT_FETCH_SH = 9, CNT_FETCH_MIS = 10, CNT_MIS_ENV = 11,
                   CNT_FETCH_MIS_ENV = 12, CNT_CLS0 = 16, kCounterSlots = 32 };

// ------------------------------------------------------------ batched mode
//
// Many render jobs (scenes, views, resolutions, spp, depths) share one pool
// of path slots. Each loop iteration refills free slots from the global work
// list (job by job, sample index by sample index), runs one bounce for every
// live path, and retires finished paths into their job's FP64 film.

struct DevJob {
  SceneView scene;
  int width, height;
  int max_depth, rr_depth;
  long long first_index;  // sample index of the job's first path: k0 * W * H
  long long num_paths;    // W * H * spp
  long long work_begin;   // offset of the job in the global work list
  double* sum;            // W*H*3
  double* sumsq;          // W*H*3
  unsigned int* count;    // W*H
};

struct BatchCtl {
  unsigned long long cursor;     // next work item
  unsigned long long total;      // total work items
  unsigned long long take_base;  // first work item taken this iteration
  int take;                      // slots refilled this iteration
  int cur;                       // parity of the current extension queue
  int counters[kCounterSlots];
  int njobs;
  int iterations;
  int max_iterations;
  int error;                     // kErr* bits
  unsigned long long rays[3];    // ext, shadow, mis
  unsigned long long paths_done;
  int more;                      // host-driven loop: 1 while another iteration is needed
};

struct BatchView {
  DevJob* jobs;
  BatchCtl* ctl;
  int* q_retire;
  int* q_free;
};

#ifdef __CUDACC__
// Sample index of a batched path slot (kept in L.w and meta.w).
__device__ __forceinline__ long long slot_index(const WaveView& w, int pid) {
  return (long long)(((unsigned long long)(unsigned)w.index_hi[pid] << 32) |
                     (unsigned long long)__float_as_uint(w.L[pid].w));
}
#endif

struct WaveArgs {
  const uint32_t* sobol;          // Sobol tables (sobol_sample, dmath.cuh)
  int64_t base_index;  // sample index of path slot 0
  int n_paths;
  int width, height;
  int max_depth;
  int rr_depth;
  unsigned class_mask;  // shading classes present in the scene (bit ShadeClass), SC_MISS always
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
  int refill_below;  // a traversal warp refills idle lanes when fewer lanes than this hold a ray (1..32)
  // Test knobs (orion_gpu_set_test_limits), 0 in normal operation:
  int test_stack_entries;   // plain renders trace with kernels whose stack holds kTestStackEntries entries
  int test_batch_iterations;  // batch loops stop (with an error) after this many iterations
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
// The film kernel first waits for `film_wait` (the previous wave's film
// write, when waves run on two streams) and then records `film_done`.
void launch_wave(const SceneView& s, const WaveView& w, const WaveArgs& a, const FilmView& film,
                 const LaunchConfig& cfg, cudaStream_t stream, int* launches, StageTimer* timer = nullptr,
                 cudaEvent_t film_wait = nullptr, cudaEvent_t film_done = nullptr);

// Launch limits of the kernel families, and the dynamic shared-memory
// allowance of the traversal kernels (raised to `smem_bytes`, the device's
// opt-in maximum, so any accepted stack depth x block size can launch).
struct KernelLimits {
  int max_trace_block;  // threads per block the traversal kernels can launch with
  int max_shade_block;  // same for the shade / resolve / retire kernels
};
cudaError_t configure_kernels(int smem_bytes, KernelLimits* lim);
cudaError_t configure_batch_kernels(int smem_bytes, KernelLimits* lim);

// Batched mode: builds the body of the device-side loop (one iteration)
// into `body` by stream capture on `stream`. The loop keeps running while
// work or live paths remain; `cond` is the graph's while-condition handle.
// Shading kernels are launched for the classes in `class_mask` only.
// waves: the iteration of wave mode (no refills, no per-iteration film).
cudaError_t capture_batch_iteration(const WaveView& w, const BatchView& b, const uint32_t* sobol,
                                    const LaunchConfig& cfg, unsigned class_mask, bool waves,
                                    cudaGraphConditionalHandle cond, cudaStream_t stream, cudaGraph_t body);
// The same iteration launched directly (a host-driven loop reading ctl->more),
// each stage timed by `timer`: the profiling path of the batched engine.
void launch_batch_iteration(const WaveView& w, const BatchView& b, const uint32_t* sobol, const LaunchConfig& cfg,
                            unsigned class_mask, bool waves, cudaStream_t stream, StageTimer* timer);
// Wave mode: starts a wave of work items [base, base + n) on slots 0..n-1
// (at most `iteration_cap` more loop iterations), and after its loop adds
// the n paths' radiance to their jobs' films.
void launch_batch_wave_begin(const WaveView& w, const BatchView& b, const uint32_t* sobol,
                             unsigned long long base, int n, int iteration_cap, int num_sms, cudaStream_t stream);
void launch_batch_wave_film(const WaveView& w, const BatchView& b, int n, int num_sms, cudaStream_t stream);
// dst[i] = (float)src[i] for i < n.
void launch_film_to_f32(const double* src, float* dst, long long n, int num_sms, cudaStream_t stream);
// Resets the batch control block and the free-slot list for `capacity` slots.
void launch_batch_init(const WaveView& w, const BatchView& b, int capacity, cudaStream_t stream);

// ------------------------------------------------------------------ SPPM
//
// Stochastic progressive photon mapping (src/integrator/sppm.cpp:58-322):
// per iteration a camera pass leaves one visible point per pixel, a hash
// grid over the visible points is built, a photon pass adds photon
// contributions to the visible points near each photon hit, and a per-pixel
// update shrinks the radii and adds the iteration's estimate to the film.

struct SppmGrid {
  float lo[3], hi[3];  // bounds of the visible points' spheres
  int res[3];
  float max_radius;
  int any;             // some pixel has a visible point
};

struct SppmView {
  int width, height, npix;
  int max_depth, iterations, photons;  // photons per iteration
  const uint32_t* sobol;               // Sobol tables (sobol_sample, dmath.cuh)
  // per pixel
  float4* vp_pr;    // visible point p, search radius (kept across iterations)
  float4* vp_wo;    // wo, material index (int bits; -1: no visible point)
  float4* vp_beta;  // beta, texture u
  float4* vp_ns;    // shading normal, texture v
  float4* vp_ng;    // geometric normal
  float4* vp_su;    // shading frame s
  float4* vp_sv;    // shading frame t
  float4* ld;       // direct light sum Ld, photon count N
  float4* tau;      // tau
  float* phi;       // 3 per pixel, photon flux of this iteration
  int* m;           // photons gathered this iteration
  SppmGrid* grid;
  float4* part_lo;  // per block of the bounds pass: lo, max radius
  float4* part_hi;  // hi, any
  // photon hits of this iteration: 3 float4 each (point + hash cell, wi, beta)
  float4* hits;
  int hits_cap;     // photons x (max depth - 1): every hit after a photon's first
  int* hit_count;
  // hash cell -> photon hits: cell h holds records [cell_start[h], cell_start[h + 1]) of by_cell
  int* cell_start;  // npix + 1 (counts, then their exclusive scan)
  int* cell_fill;   // npix
  int* scan_part;   // per scan block
  float4* by_cell;  // the hits in hash-cell order, 3 float4 each (hits_cap)
  float* film;      // W*H*3 sums of the iterations' estimates
  unsigned* film_count;
  unsigned long long* rays;
};

constexpr int kSppmBoundsBlocks = 1024;  // blocks of the bounds pass (part_lo / part_hi entries)
constexpr int kScanBlock = 1024;         // elements per block of the cell-count scan

// Resets per-pixel state (radius r0, no visible point) and the film.
void launch_sppm_init(const SppmView& v, float radius0, cudaStream_t stream);
// Camera pass and the grid over the visible points of iteration `iter`.
void launch_sppm_visible_points(const SceneView& s, const SppmView& v, int iter, cudaStream_t stream);
// Exclusive scan of the cell counts (cell_start).
void launch_sppm_scan(const SppmView& v, cudaStream_t stream);
// Photon pass, photon lists by cell, gather at the visible points, pixel
// update and film. No host synchronisation between iterations.
void launch_sppm_photons(const SceneView& s, const SppmView& v, int iter, cudaStream_t stream);

// Averaged FP64 film (W*H*3 sums, W*H counts) -> W*H pixels of bytes B, G,
// R, 255 as saveAsBmp writes them; rows bottom-up when `bottom_up`.
void launch_film_preview(const double* sum, const uint32_t* count, int width, int height, int bottom_up,
                         uint8_t* bgra, cudaStream_t stream);

// Component hooks for the parity tests.
void launch_sobol(const uint32_t* sobol, int64_t n, const uint64_t* index, const uint32_t* dim, float* out,
                  cudaStream_t stream);
void launch_trace(const SceneView& s, int64_t n, const float* rays, int any_hit, float* t, float* u, float* v,
                  int* prim, const LaunchConfig& cfg, cudaStream_t stream);
// The same queries through the renderer's persistent trace kernels: the rays
// become wave `w`'s extension rays (closest hit) or shadow rays (any hit).
void launch_trace_wave(const SceneView& s, const WaveView& w, int n, const float* rays, int any_hit, float* t,
                       float* u, float* v, int* prim, const LaunchConfig& cfg, cudaStream_t stream);
void launch_camera_rays(const SceneView& s, const uint32_t* sobol, int64_t n, const int64_t* index, float* rays,
                        cudaStream_t stream);
void launch_bsdf_eval(const DevMaterial* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                      const float* rnd, int type, float* f, float* pdf, float* sf, float* swi, float* spdf,
                      int* stype, int* nbxdf, cudaStream_t stream);

}  // namespace orion_gb300
