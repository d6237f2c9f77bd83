/*
 * orion_gpu.h -- C ABI of the GB300 wavefront path tracer.
 *
 * This is the whole boundary between a host application and the CUDA path
 * tracer: plain C types, caller-owned buffers, status-code returns, opaque
 * handles, no exceptions or C++ types across it. It replaces the reference's
 * path-tracing hot path:
 *
 *   Integrator::render(const Scene&)      src/core/integrator.h:26
 *   PathTracing::render / Li              src/integrator/path.cpp:15-37, 50-99
 *   Scene::intersect -> EmbreeKernel      src/core/scene.cpp:16-19, src/core/kernel.cpp:111-174
 *   Parser(path).getRenderOption()        src/util/parser.cpp:45-56, 463-471
 *
 * Every entry point returns ORION_OK (0) or a negative ORION_ERR_* code; the
 * message for the last failure on the calling thread is available from
 * orion_last_error().
 */
#ifndef ORION_GPU_H_
#define ORION_GPU_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
enum {
  ORION_OK = 0,
  ORION_ERR_INVALID = -1,     /* bad argument or handle */
  ORION_ERR_IO = -2,          /* file missing or unreadable */
  ORION_ERR_PARSE = -3,       /* malformed scene XML or OBJ */
  ORION_ERR_CUDA = -4,        /* CUDA runtime failure */
  ORION_ERR_NOMEM = -5,       /* allocation failed or device budget exceeded */
  ORION_ERR_UNSUPPORTED = -6, /* scene feature outside this library */
  ORION_ERR_DEVICE = -7,      /* a kernel raised its error word (overflow / iteration cap) */
  ORION_ERR_NOT_READY = -8,   /* serving: job still running */
  ORION_ERR_CANCELLED = -9    /* serving: job cancelled */
};

/* Message of the last failure on this thread ("" if none). */
const char* orion_last_error(void);

/* ------------------------------------------------------------- materials */
/* One record per <Material>; fields unused by a type are ignored.
 * Types follow src/material/{matte,metal,mirror,glass,plastic,uber}.cpp. */
enum {
  ORION_MAT_MATTE = 0,   /* Kd, sigma (src/material/matte.cpp:9-21) */
  ORION_MAT_METAL = 1,   /* eta_rgb, k, roughness (src/material/metal.cpp:8-17) */
  ORION_MAT_MIRROR = 2,  /* Kr (src/material/mirror.cpp:6-13) */
  ORION_MAT_GLASS = 3,   /* Kr, Kt, roughness, eta (src/material/glass.cpp:9-37) */
  ORION_MAT_PLASTIC = 4, /* Kd, Ks, roughness (src/material/plastic.cpp:8-24) */
  ORION_MAT_UBER = 5     /* Kd, Ks, Kr, Kt, opacity, roughness, eta (src/material/uber.cpp:9-42) */
};
/* Microfacet distribution. The reference has GGX only (src/bsdf/microfacet.cpp:9-40);
 * Beckmann is an extension selected by <Param distribution="beckmann"/>. */
enum { ORION_DIST_GGX = 0, ORION_DIST_BECKMANN = 1 };

/* Spectrum inputs a material can take from an image texture
 * (<Kd><Param type="image"/><Param filename="..."/></Kd>, src/util/parser.cpp:433-461):
 * index into orion_material.tex. */
enum {
  ORION_TEX_KD = 0,
  ORION_TEX_KS = 1,
  ORION_TEX_KR = 2,
  ORION_TEX_KT = 3,
  ORION_TEX_OPACITY = 4,
  ORION_TEX_ETA = 5, /* metal eta_rgb */
  ORION_TEX_K = 6,   /* metal k */
  ORION_TEX_SLOTS = 7
};

typedef struct orion_material {
  int32_t type;
  int32_t distribution;
  int32_t has_sigma; /* matte: 0 = no <sigma> (Lambert) */
  int32_t reserved;
  float Kd[3], Ks[3], Kr[3], Kt[3], opacity[3];
  float eta_rgb[3], k[3]; /* metal */
  float sigma, roughness, eta;
  /* tex[ORION_TEX_*]: 0 = the constant above; k = the scene's image k - 1,
   * looked up at the hit's texture coordinates (Texture::evaluate,
   * src/core/texture.cpp:8-11, wrap filter). tex[7] is reserved (0). */
  int32_t tex[8];
} orion_material;

/* ---------------------------------------------------------------- lights */
/* Order in a scene is the reference's scene.lights order: area lights (one
 * per emissive triangle, in primitive order), then <Light> elements, then
 * <Envmap> elements (src/util/parser.cpp:45-56). */
enum {
  ORION_LIGHT_AREA = 0,    /* src/light/diffuse.cpp:8-56 */
  ORION_LIGHT_POINT = 1,   /* src/light/point.cpp:6-19 */
  ORION_LIGHT_SPOT = 2,    /* src/light/spot.cpp:6-29 */
  ORION_LIGHT_DISTANT = 3, /* src/light/distant.cpp:6-26 */
  ORION_LIGHT_ENV = 4      /* constant environment, src/light/envmap.cpp:9-81 */
};

typedef struct orion_light {
  int32_t type;
  int32_t prim;            /* area: index of the emissive triangle */
  float L[3];              /* area Le, point/spot I, distant/env L */
  float p[3];              /* point/spot: world position */
  float dir[3];            /* distant: unit direction towards which light travels from `from` */
  float l2w[12], w2l[12];  /* spot/env: light<->world, 3x4 row-major */
  float cos_total, cos_falloff; /* spot */
  int32_t image;           /* env: 0 = constant map, k = the scene's image k - 1 (times L) */
  int32_t reserved;
} orion_light;

/* An image of a scene (environment map or material texture texels): linear
 * RGB floats, row 0 at the top, as the reference's ImageMemory holds them
 * (8-bit files: byte / 255, src/texture/imagetexture.cpp:16-52). */
typedef struct orion_image {
  int32_t width, height;
  const float* rgb;        /* width x height x 3 */
} orion_image;

/* ---------------------------------------------------------------- camera */
typedef struct orion_camera {
  float c2w[16];           /* camera-to-world, 4x4 row-major (src/core/transform.cpp:197-217) */
  float fov;               /* vertical field of view, degrees */
  float lens_radius;       /* 0 = pinhole (src/camera/pinhole.cpp:23-29) */
  float focal_distance;
  int32_t width, height;   /* film size */
} orion_camera;

/* ------------------------------------------------------------ integrator */
/* <Integrator type=...> (src/util/parser.cpp:123-137). */
enum { ORION_INTEGRATOR_PATH = 0, ORION_INTEGRATOR_SPPM = 1 };

/* SPPM parameters (createSPPMIntegrator, src/integrator/sppm.cpp:324-333). */
typedef struct orion_sppm_params {
  int32_t iterations;        /* numIterations */
  int32_t photons_per_iter;  /* photonsPerIteration; < 0 = film width x height */
  float initial_radius;      /* initRadius */
  int32_t max_depth;         /* maxDepth */
} orion_sppm_params;

/* ----------------------------------------------------------------- scene */
/* Flat, de-indexed scene in primitive (primID) order: the data the
 * reference hands to Embree plus what shading needs per primitive. */
typedef struct orion_scene_desc {
  int64_t num_prims;
  const float* positions;        /* num_prims x 9: p0, p1, p2 in world space */
  const float* normals;          /* num_prims x 9: per-corner shading normals */
  const float* uvs;              /* num_prims x 6, or NULL */
  const int32_t* material_of_prim;
  const int32_t* light_of_prim;  /* index into lights of the prim's area light, or -1 */
  int32_t num_materials;
  int32_t num_lights;
  const orion_material* materials;
  const orion_light* lights;
  orion_camera camera;
  int32_t spp;                   /* <Integrator> nSamplesPerPixel */
  int32_t max_depth;             /* <Integrator> maxDepth */
  int32_t num_images;
  int32_t reserved;
  const orion_image* images;     /* referenced by orion_light.image and orion_material.tex */
  int32_t integrator;            /* ORION_INTEGRATOR_*; spp and max_depth above are the path tracer's */
  int32_t reserved2;
  orion_sppm_params sppm;        /* ORION_INTEGRATOR_SPPM: its parameters */
} orion_scene_desc;

typedef struct orion_host_scene orion_host_scene;

/* Parse a .ori scene file and its OBJ meshes (src/util/parser.cpp:463-471). */
int orion_scene_load_ori(const char* path, orion_host_scene** out);
/* Copy a caller-built description into a new host scene. */
int orion_scene_from_desc(const orion_scene_desc* desc, orion_host_scene** out);
/* View of a host scene's arrays; valid until orion_scene_free. */
int orion_scene_get_desc(const orion_host_scene* scene, orion_scene_desc* out);
void orion_scene_free(orion_host_scene* scene);

/* --------------------------------------------------------------- context */
typedef struct orion_gpu_ctx orion_gpu_ctx;

typedef struct orion_gpu_opts {
  int32_t device;          /* CUDA device ordinal */
  int32_t reserved;
  int64_t memory_budget;   /* bytes the context may hold for scenes + path state; 0 = 90% of free memory */
  const char* sobol_path;  /* Sobol matrix file; NULL = sobol_matrices.bin beside the library */
} orion_gpu_opts;

int orion_gpu_create(const orion_gpu_opts* opts, orion_gpu_ctx** out);
int orion_gpu_destroy(orion_gpu_ctx* ctx);

typedef int32_t orion_scene_id;

/* Build the BVH on the host and upload the scene (replaces EmbreeKernel::build,
 * src/core/kernel.cpp:63-110). The scene stays resident until released. */
int orion_gpu_scene_upload(orion_gpu_ctx* ctx, const orion_host_scene* scene, orion_scene_id* out);
int orion_gpu_scene_release(orion_gpu_ctx* ctx, orion_scene_id id);
/* Device bytes held by a resident scene (BVH + triangles + shading data). */
int orion_gpu_scene_bytes(orion_gpu_ctx* ctx, orion_scene_id id, int64_t* bytes);

typedef struct orion_render_params {
  int32_t spp;               /* 0 = the scene's nSamplesPerPixel */
  int32_t max_depth;         /* -1 = the scene's maxDepth */
  int32_t rr_depth;          /* Russian roulette when bounces > rr_depth; the reference uses 3 (path.cpp:91) */
  int32_t flags;             /* ORION_RENDER_* */
  int64_t first_pass;        /* k0: sample index of (i, j, k) is (k0 + k)*W*H + j*W + i */
  int32_t wave_paths;        /* paths per wavefront wave; 0 = autotuned */
  int32_t reserved;
} orion_render_params;

enum {
  ORION_RENDER_FP64 = 1      /* also accumulate FP64 sums and sums of squares */
};

/* SPPM::render (src/integrator/sppm.cpp:58-322) of a resident scene with
 * its camera: `params` NULL = the scene's <Integrator type="sppm">
 * parameters. film_rgb_sum: W*H*3 floats, the sum over iterations of each
 * iteration's estimate (the reference accumulates one per iteration into
 * its film); film_count: W*H (each = iterations) or NULL. Stats: paths =
 * camera paths + photons, rays = all rays traced. */
int orion_gpu_render_sppm(orion_gpu_ctx* ctx, orion_scene_id id, const orion_sppm_params* params,
                          float* film_rgb_sum, uint32_t* film_count);

/* Render statistics of the last orion_gpu_render on a context. */
typedef struct orion_render_stats {
  int64_t paths;             /* camera paths traced */
  int64_t rays;              /* all rays: extension + shadow + MIS */
  int64_t ext_rays, shadow_rays, mis_rays;
  int64_t kernel_launches;
  double device_ms;          /* device time of the render (CUDA events) */
} orion_render_stats;

/* Integrator::render(): traces W*H*spp paths and writes the film.
 * film_rgb_sum: W*H*3 floats, per-pixel FP32 sums in sample order (as
 * RenderTarget::acumulate, src/texture/rendertarget.cpp:22-27).
 * film_count: W*H sample counts, or NULL. Both are host buffers. */
int orion_gpu_render(orion_gpu_ctx* ctx, orion_scene_id id, const orion_render_params* params,
                     float* film_rgb_sum, uint32_t* film_count);
/* Same, with FP64 per-pixel sums and sums of squares (W*H*3 doubles each). */
int orion_gpu_render_fp64(orion_gpu_ctx* ctx, orion_scene_id id, const orion_render_params* params,
                          double* sum, double* sumsq);
int orion_gpu_last_stats(orion_gpu_ctx* ctx, orion_render_stats* out);

/* Per-stage device time of the last render, filled only while profiling is
 * on (CUDA events around every kernel; adds a little launch overhead).
 * Stages: 0 camera, 1 extension-ray trace, 2 shade, 3 shadow-ray trace,
 * 4 MIS-ray trace, 5 direct-light resolve, 6 film, 7 bookkeeping.
 * A batched render under profiling runs its loop from the host instead of a
 * graph while-node (same kernels and results; stage 0 is then slot refill,
 * stage 6 retirement into the films). */
#define ORION_NUM_STAGES 8
typedef struct orion_stage_times {
  double ms[ORION_NUM_STAGES];
  int64_t launches[ORION_NUM_STAGES];
} orion_stage_times;
/* `enable` is a bit set: ORION_PROFILE_STAGES times every stage as above;
 * ORION_PROFILE_TRAVERSAL makes plain renders count the BVH work of their
 * trace kernels (same traversal and film, slower kernels), read back with
 * orion_gpu_traversal_work. 0 turns both off. */
#define ORION_PROFILE_STAGES 1
#define ORION_PROFILE_TRAVERSAL 2
int orion_gpu_set_profiling(orion_gpu_ctx* ctx, int32_t enable);
int orion_gpu_stage_times(orion_gpu_ctx* ctx, orion_stage_times* out);

/* BVH work of the last plain render made with ORION_PROFILE_TRAVERSAL (all
 * zero otherwise), per ray kind [extension, shadow, MIS]: rays traced,
 * 8-wide nodes visited (80 bytes each) and triangles tested (48 bytes each).
 * Embree's traversal inside EmbreeKernel::intersect (src/core/kernel.cpp:111)
 * has no counterpart; these figures explain the trace kernels' memory
 * traffic. */
typedef struct orion_traversal_work {
  int64_t rays[3];
  int64_t nodes[3];
  int64_t triangles[3];
} orion_traversal_work;
int orion_gpu_traversal_work(orion_gpu_ctx* ctx, orion_traversal_work* out);

/* ----------------------------------------------------------- film output */
/* saveAsBmp (src/core/texture.cpp:77-136): the averaged film `rgb`
 * (height x width x 3, row 0 at the top, as RenderTarget::getAveraged
 * returns it) as a 32-bit BMP: rows bottom-up, bytes B, G, R, 255, each
 * channel clamp(c, 0, 1) * 255 truncated (NaN -> 0), no tone mapping. */
int orion_film_write_bmp(const char* path, int32_t width, int32_t height, const float* rgb);

/* ------------------------------------------------------------- batches */
/* Many render() calls in one launch. There is no single reference call for
 * this: it runs PathTracing::render (src/integrator/path.cpp:15-37) for every
 * job, sharing one pool of path slots across jobs (finished slots are
 * refilled with the next job's paths), inside one CUDA graph launch whose
 * device-side loop runs until every job's paths are done. Per-path results
 * are the plain render's; films are accumulated in FP64. */
typedef struct orion_job {
  orion_scene_id scene;
  int32_t reserved;
  orion_render_params params;  /* spp 0 = scene's; max_depth -1 = scene's; rr_depth; first_pass */
  const orion_camera* camera;  /* another view of the resident scene (its own film size), or NULL */
  double* sum;                 /* host W*H*3 FP64 radiance sums, or NULL */
  double* sumsq;               /* host W*H*3 FP64 sums of squares, or NULL */
  uint32_t* count;             /* host W*H samples per pixel, or NULL */
  float* sum32;                /* host W*H*3 radiance sums rounded to FP32 on the device (half the
                                  read-back of `sum`, the film type of orion_gpu_render), or NULL */
} orion_job;

typedef struct orion_batch_stats {
  int64_t paths;               /* camera paths traced */
  int64_t rays;                /* extension + shadow + MIS rays */
  int64_t iterations;          /* device loop iterations */
  int64_t capacity;            /* path slots in the pool */
  double device_ms;            /* device time of the graph launch */
} orion_batch_stats;

int orion_gpu_render_batch(orion_gpu_ctx* ctx, int32_t njobs, const orion_job* jobs, orion_batch_stats* stats);

/* Launch configuration: the autotuned knobs. */
typedef struct orion_launch_config {
  int32_t trace_block;    /* threads per block of the traversal kernels (64..512) */
  int32_t shade_block;    /* threads per block of the shading kernels (64..512) */
  int32_t smem_stack;     /* traversal stack entries kept in shared memory: 0, 8, 16, 24 or 32 */
  int32_t blocks_per_sm;  /* persistent trace blocks per SM; the grid-stride kernels launch twice as many */
  int32_t wave_paths;     /* paths per plain-render wave */
  int32_t batch_slots;    /* batches: path slots of the pool (pooled mode) or paths per wave (wave mode) */
  int32_t refill_below;   /* a traversal warp takes new rays once fewer lanes than this hold one (1..32);
                             plain renders' any-hit launches use this + 4 (at most 32) */
  int32_t streams;        /* plain renders: waves in flight at once, each on its own stream (1..4);
                             batches: concurrent engines, set to min(streams, 2) here; 0 = keep.
                             orion_gpu_autotune_batch tunes the engine count alone (reported here
                             by it) and leaves plain renders' waves as they were */
} orion_launch_config;

/* How orion_gpu_render_batch (and the server) run a batch:
 * ORION_BATCH_WAVES (default): the jobs' concatenated work list in waves of
 *   batch_slots paths, each wave's paths bouncing until none is alive;
 * ORION_BATCH_POOLED: a pool of batch_slots path slots refilled from the
 *   work list every bounce. */
enum { ORION_BATCH_POOLED = 0, ORION_BATCH_WAVES = 1 };
int orion_gpu_set_batch_mode(orion_gpu_ctx* ctx, int32_t mode);

int orion_gpu_get_config(orion_gpu_ctx* ctx, orion_launch_config* out);
int orion_gpu_set_config(orion_gpu_ctx* ctx, const orion_launch_config* cfg);

/* Autotuner: times renders of `id` (at `spp` samples per pixel) over a grid
 * of launch configurations within about `budget_ms` of device time, keeps
 * the fastest on the context and returns it. */
int orion_gpu_autotune(orion_gpu_ctx* ctx, orion_scene_id id, int32_t spp, double budget_ms,
                       orion_launch_config* best, double* best_mpaths);
/* Autotuner for the batched engine: times orion_gpu_render_batch-style
 * launches of `jobs` (spp capped at `spp_cap` when > 0; films are scratch and
 * discarded) over the same knobs plus the path-slot count, keeps the fastest
 * on the context and returns it. best_mpaths: paths/s of the best trial. */
int orion_gpu_autotune_batch(orion_gpu_ctx* ctx, int32_t njobs, const orion_job* jobs, int32_t spp_cap,
                             double budget_ms, orion_launch_config* best, double* best_mpaths);

/* ------------------------------------------------------------- serving */
/* A request loop on a context: render requests (a resident scene, a view,
 * render parameters) are admitted as device memory allows, progress in
 * chunks of samples per pixel, and every launch traces all admitted requests
 * together (orion_gpu_render_batch), so requests that arrive while others are
 * running join the next launch. Scenes are uploaded on first use and stay
 * resident (least recently used ones are evicted when memory is needed).
 * A request's result is its film's FP64 sums over all its samples; it does
 * not depend on which other requests shared its launches. */
typedef struct orion_server orion_server;

typedef struct orion_server_opts {
  int64_t memory_budget;   /* bytes for resident scenes + request films + path slots; 0 = context budget */
  int32_t spp_chunk;       /* samples per pixel a request advances per launch; 0 = 4 */
  int32_t max_jobs;        /* requests in one launch; 0 = 512 */
} orion_server_opts;

enum { ORION_REQ_QUEUED = 0, ORION_REQ_RUNNING = 1, ORION_REQ_DONE = 2, ORION_REQ_CANCELLED = 3, ORION_REQ_FAILED = 4 };

typedef struct orion_request_status {
  int32_t state;
  int32_t spp_done, spp_total;
  int32_t width, height;
  int32_t reserved;
  double t_submit, t_admit, t_done;  /* seconds since the server started; 0 until reached */
} orion_request_status;

typedef struct orion_server_stats {
  int64_t submitted, completed, launches, paths, resident_scenes, bytes_in_use;
  double device_ms;
} orion_server_stats;

int orion_server_create(orion_gpu_ctx* ctx, const orion_server_opts* opts, orion_server** out);
/* `scene` must stay alive until the request is released. camera: NULL = the scene's view. */
int orion_server_submit(orion_server* srv, const orion_host_scene* scene, const orion_render_params* params,
                        const orion_camera* camera, int64_t* ticket);
int orion_server_status(orion_server* srv, int64_t ticket, orion_request_status* out);
/* ORION_OK once the request is done, ORION_ERR_NOT_READY after `timeout_s` seconds. */
int orion_server_wait(orion_server* srv, int64_t ticket, double timeout_s);
/* Copies the request's film so far (progressive results): W*H*3 sums and sums of squares, W*H counts. */
int orion_server_result(orion_server* srv, int64_t ticket, double* sum, double* sumsq, uint32_t* count);
/* The request's film so far as 8-bit pixels B, G, R, 255 (W*H*4 bytes):
 * RenderTarget::getAveraged then saveAsBmp's clamp(c, 0, 1) * 255 truncated
 * (src/core/texture.cpp:77-136), computed on the device. Rows top-down, or
 * bottom-up as in a BMP file with ORION_PREVIEW_BOTTOM_UP. Unsampled pixels
 * are black. */
enum { ORION_PREVIEW_BOTTOM_UP = 1 };
int orion_server_preview(orion_server* srv, int64_t ticket, uint8_t* bgra, int32_t flags);
int orion_server_cancel(orion_server* srv, int64_t ticket);
/* Frees a finished, failed or cancelled request's film. */
int orion_server_release(orion_server* srv, int64_t ticket);
int orion_server_stats_get(orion_server* srv, orion_server_stats* out);
int orion_server_destroy(orion_server* srv);

/* ------------------------------------------------- component test hooks */
/* sobol::sample (src/sampler/sobol.h:28-43) for n (index, dim) pairs. */
int orion_gpu_sobol(orion_gpu_ctx* ctx, int64_t n, const uint64_t* index, const uint32_t* dim, float* out);
/* Closest hit (any_hit = 0) or occlusion (any_hit = 1) for n rays given as
 * n x 8 floats (o, d, tnear, tfar). prim = -1 for a miss. */
int orion_gpu_trace(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays, int32_t any_hit,
                    float* t, float* u, float* v, int32_t* prim);
/* The same queries traced by the renderer's own persistent kernels: closest-hit
 * rays become a wave's extension rays (k_trace), any-hit rays its shadow rays
 * (k_trace_sh, occlusion within (0, tfar]). Every ray's tnear must be 0, as
 * for the renderer's rays; closest-hit rays ignore tfar (extension rays are
 * unbounded). prim = -1 for a miss; for any_hit = 1, prim = 1 when occluded
 * and t, u, v are 0. Replaces rtcIntersect / rtcOccluded as the renderer calls
 * them (src/core/kernel.cpp:111-174, src/core/light.h:17-30). Returns
 * ORION_ERR_DEVICE if a traversal overflowed its stack. */
int orion_gpu_trace_wave(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays, int32_t any_hit,
                         float* t, float* u, float* v, int32_t* prim);
/* Free and total bytes of the context's device (cudaMemGetInfo): lets a caller
 * check that a call allocated nothing. No counterpart in the reference. */
int orion_gpu_mem_info(orion_gpu_ctx* ctx, int64_t* free_bytes, int64_t* total_bytes);
/* Failure-path test knobs (0, 0 = normal operation). stack_entries = 2 makes
 * plain renders and orion_gpu_trace_wave trace with kernels whose traversal
 * stack holds 2 entries, so deep traversals overflow and the call returns
 * ORION_ERR_DEVICE; batch_iterations > 0 stops every batch loop after that
 * many iterations, so unfinished batches return ORION_ERR_DEVICE. No
 * counterpart in the reference, which prints and continues (src/orion.h:33-37). */
int orion_gpu_set_test_limits(orion_gpu_ctx* ctx, int32_t stack_entries, int32_t batch_iterations);
/* orion_gpu_trace without any device allocation. No counterpart in the
 * reference: it exists for callers that must not allocate, such as a ray query
 * (picking) from a second context while a long render runs on the same device
 * (cudaFree in orion_gpu_trace synchronises the whole device, and a serving
 * memory budget has already committed every device byte). Rays and hits go
 * through one fixed static device array of ORION_NOALLOC_MAX_RAYS rays
 * (3 MiB); larger n is rejected with ORION_ERR_INVALID. Nothing in that array
 * must start at zero. Calls on one context are serialised by the context; calls
 * that overlap on one device from different contexts race on the array. The
 * first call on a device looks up the array's address and should come before
 * any stream capture on that device. Same arguments and results as
 * orion_gpu_trace. */
#define ORION_NOALLOC_MAX_RAYS 65536
int orion_gpu_trace_noalloc(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays, int32_t any_hit,
                            float* t, float* u, float* v, int32_t* prim);
/* Camera rays (src/camera/pinhole.cpp:8-33) for sample indices: n x 6 floats. */
int orion_gpu_camera_rays(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const int64_t* sample_index,
                          float* rays);
/* BSDF at a synthetic hit: frame n x 12 (ng, ns, u, v); wo, wi n x 3; rnd n x 2.
 * Outputs f, pdf for (wi, wo), and sample_f's f, wi, pdf, sampled type, and the
 * number of non-specular lobes (src/core/bsdf.cpp:4-106). */
int orion_gpu_bsdf_eval(orion_gpu_ctx* ctx, const orion_material* mat, int64_t n, const float* frame,
                        const float* wo, const float* wi, const float* rnd, int32_t type, float* f, float* pdf,
                        float* sf, float* swi, float* spdf, int32_t* stype, int32_t* nbxdf);

#ifdef __cplusplus
}
#endif
#endif /* ORION_GPU_H_ */
