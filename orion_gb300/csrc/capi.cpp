// C ABI (include/orion_gpu.h): context, resident scenes, render driver.
//
// PathTracing::render (src/integrator/path.cpp:15-37) loops over spp passes
// and pixels, one CPU thread per row. Here the sample indices
// [k0*W*H, (k0+spp)*W*H) are cut into waves of up to `wave_paths` paths; each
// wave is one fixed sequence of kernels on the context's stream (no host
// synchronisation inside a render), and the film is accumulated per pixel in
// sample order so its FP32 sums follow the reference's addition order.
#include <cuda_runtime.h>
#include <dlfcn.h>

#include <algorithm>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

using namespace orion_gb300;

namespace {
template <class T>
void pin(orion_host_scene* h, const std::vector<T>& v) {
  if (v.empty()) return;
  void* p = const_cast<T*>(v.data());
  if (cudaHostRegister(p, v.size() * sizeof(T), cudaHostRegisterPortable) == cudaSuccess)
    h->pinned.push_back(p);
  else
    cudaGetLastError();  // stays pageable: copies are slower, results the same
}
}  // namespace

namespace orion_gb300 {

namespace {
thread_local std::string g_error;
}  // namespace

int fail(int code, const std::string& msg) {
  g_error = msg;
  return code;
}

namespace {
std::mutex g_pools_mu;
std::vector<cudaMemPool_t> g_pools;  // every live context's scene pool
}  // namespace

void trim_scene_pools() {
  std::lock_guard<std::mutex> g(g_pools_mu);
  for (cudaMemPool_t pool : g_pools) cudaMemPoolTrimTo(pool, 0);
}

}  // namespace orion_gb300

// Why a launch configuration cannot run on this context ("" if it can).
std::string orion_gb300::config_problem(const orion_gpu_ctx* ctx, const LaunchConfig& c) {
  const int st = c.smem_stack;
  if (c.trace_block < 32 || c.trace_block % 32 || c.trace_block > ctx->limits.max_trace_block)
    return "trace_block must be a multiple of 32 up to " + std::to_string(ctx->limits.max_trace_block);
  if (c.shade_block < 32 || c.shade_block % 32 || c.shade_block > ctx->limits.max_shade_block)
    return "shade_block must be a multiple of 32 up to " + std::to_string(ctx->limits.max_shade_block);
  if (!(st == 0 || st == 8 || st == 16 || st == 24 || st == 32)) return "smem_stack must be 0, 8, 16, 24 or 32";
  if ((int64_t)st * c.trace_block * 8 + (int64_t)(c.trace_block / 32) * kTriScratchBytes > ctx->smem_limit)
    return "traversal stack (smem_stack x trace_block x 8 bytes) and triangle scratch exceed " +
           std::to_string(ctx->smem_limit) + " bytes of shared memory";
  if (c.blocks_per_sm < 1 || c.blocks_per_sm > 64) return "blocks_per_sm out of range (1..64)";
  if (c.refill_below < 1 || c.refill_below > 32) return "refill_below out of range (1..32)";
  return std::string();
}

extern "C" const char* orion_last_error(void) { return orion_gb300::g_error.c_str(); }

// ------------------------------------------------------------- scenes

extern "C" int orion_scene_load_ori(const char* path, orion_host_scene** out) {
  if (!path || !out) return fail(ORION_ERR_INVALID, "null argument");
  std::unique_ptr<orion_host_scene> h(new orion_host_scene());
  std::string err;
  int rc = load_ori(path, &h->s, &err);
  if (rc != ORION_OK) return fail(rc, err);
  *out = h.release();
  return ORION_OK;
}

extern "C" int orion_scene_from_desc(const orion_scene_desc* desc, orion_host_scene** out) {
  if (!desc || !out) return fail(ORION_ERR_INVALID, "null argument");
  std::unique_ptr<orion_host_scene> h(new orion_host_scene());
  std::string err;
  int rc = scene_from_desc(*desc, &h->s, &err);
  if (rc != ORION_OK) return fail(rc, err);
  *out = h.release();
  return ORION_OK;
}

extern "C" int orion_scene_get_desc(const orion_host_scene* scene, orion_scene_desc* out) {
  if (!scene || !out) return fail(ORION_ERR_INVALID, "null argument");
  scene->s.desc(out);
  return ORION_OK;
}

extern "C" void orion_scene_free(orion_host_scene* scene) { delete scene; }

// ------------------------------------------------------------ context

static std::string default_sobol_path() {
  Dl_info info;
  if (dladdr(reinterpret_cast<void*>(&default_sobol_path), &info) && info.dli_fname) {
    std::string p(info.dli_fname);
    size_t slash = p.find_last_of('/');
    std::string dir = slash == std::string::npos ? std::string(".") : p.substr(0, slash);
    return dir + "/data/sobol_matrices.bin";
  }
  return "data/sobol_matrices.bin";
}

// The message for a launch's error word (kErr* bits).
static std::string kernel_error(int bits) {
  std::string m = "kernel error word " + std::to_string(bits) + ":";
  if (bits & kErrIterationCap) m += " iteration cap reached;";
  if (bits & kErrTraversalStack) m += " a BVH traversal overflowed its stack (its rays were counted as misses);";
  return m;
}

static int ensure_film(orion_gpu_ctx* c, int64_t pixels, bool fp64) {
  if (pixels > c->film_pixels) {
    int rc;
    if ((rc = c->film_sum.alloc(pixels * 3 * sizeof(float))) != ORION_OK) return rc;
    if ((rc = c->film_count.alloc(pixels * sizeof(uint32_t))) != ORION_OK) return rc;
    c->film64.alloc(0);
    c->filmsq64.alloc(0);
    c->film_pixels = pixels;
  }
  if (fp64 && c->film64.bytes < (size_t)pixels * 3 * sizeof(double)) {
    int rc;
    if ((rc = c->film64.alloc(pixels * 3 * sizeof(double))) != ORION_OK) return rc;
    if ((rc = c->filmsq64.alloc(pixels * 3 * sizeof(double))) != ORION_OK) return rc;
  }
  return ORION_OK;
}

int orion_gb300::alloc_wave(Wave& wave, int capacity) {
  if (wave.capacity >= capacity) return ORION_OK;
  const size_t n = (size_t)capacity;
  auto round256 = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t recb = round256(n * sizeof(PathRec)), neeb = round256(n * sizeof(NeeRec));
  const size_t f4 = round256(n * sizeof(float4)), i4 = round256(n * sizeof(int)), fb = round256(n);
  const size_t bytes = recb + neeb + f4 + (8 + kShadeClasses) * i4 + fb + 256 + 4096;
  int rc = wave.block.alloc(bytes);
  if (rc != ORION_OK) {
    wave.capacity = 0;
    return rc;
  }
  char* p = wave.block.as<char>();
  WaveView& w = wave.view;
  w.rec = reinterpret_cast<PathRec*>(p);
  p += recb;
  w.nee = reinterpret_cast<NeeRec*>(p);
  p += neeb;
  w.mis_hit = reinterpret_cast<float4*>(p);
  p += f4;
  char* rb = reinterpret_cast<char*>(w.rec);
  char* nb = reinterpret_cast<char*>(w.nee);
  auto rec4 = [&](size_t off) { return RecF4{reinterpret_cast<float4*>(rb + off)}; };
  auto reci = [&](size_t off) { return RecI{reinterpret_cast<int*>(rb + off)}; };
  auto nee4 = [&](size_t off) { return NeeF4{reinterpret_cast<float4*>(nb + off)}; };
  w.ray_o = rec4(offsetof(PathRec, o));
  w.ray_d = rec4(offsetof(PathRec, d));
  w.beta = rec4(offsetof(PathRec, beta));
  w.L = rec4(offsetof(PathRec, L));
  w.hit = rec4(offsetof(PathRec, hit));
  w.dim = reci(offsetof(PathRec, meta));
  w.job = reci(offsetof(PathRec, meta) + 4);
  w.bounce = reci(offsetof(PathRec, meta) + 8);
  w.index_hi = reci(offsetof(PathRec, meta) + 12);
  w.nee_p = nee4(offsetof(NeeRec, p));
  w.nee_beta = nee4(offsetof(NeeRec, beta));
  w.nee_ld = nee4(offsetof(NeeRec, ld));
  w.nee_f = nee4(offsetof(NeeRec, f));
  w.sh_o = nee4(offsetof(NeeRec, sh_o));
  w.sh_d = nee4(offsetof(NeeRec, sh_d));
  w.mis_o = nee4(offsetof(NeeRec, mis_o));
  w.mis_d = nee4(offsetof(NeeRec, mis_d));
  int** i4s[] = {&w.occluded, &w.mis_occluded, &w.q_ext[0], &w.q_ext[1],
                 &w.q_nee,    &w.q_sh,         &w.q_mis,    &w.q_mis_env};
  for (int** q : i4s) {
    *q = reinterpret_cast<int*>(p);
    p += i4;
  }
  w.q_cls = reinterpret_cast<int*>(p);  // class c at q_cls + c * capacity
  p += kShadeClasses * i4;
  w.qflags = reinterpret_cast<uint8_t*>(p);
  p += fb;
  w.counters = reinterpret_cast<int*>(p);
  p += 128;
  w.ray_stats = reinterpret_cast<unsigned long long*>(p);  // [0, 3) rays, [4, 10) traversal work
  w.trace_work = nullptr;
  p += 128;
  w.error_word = reinterpret_cast<int*>(p);
  w.capacity = capacity;
  wave.capacity = capacity;
  return ORION_OK;
}

static int ensure_wave(orion_gpu_ctx* c, int capacity) { return alloc_wave(c->wave, capacity); }

extern "C" int orion_gpu_create(const orion_gpu_opts* opts, orion_gpu_ctx** out) {
  if (!out) return fail(ORION_ERR_INVALID, "null argument");
  std::unique_ptr<orion_gpu_ctx> c(new orion_gpu_ctx());
  c->device = opts ? opts->device : 0;
  int ndev = 0;
  CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (c->device < 0 || c->device >= ndev) return fail(ORION_ERR_INVALID, "no such CUDA device");
  CUDA_TRY(cudaSetDevice(c->device));
  cudaDeviceProp prop;
  CUDA_TRY(cudaGetDeviceProperties(&prop, c->device));
  c->num_sms = prop.multiProcessorCount;
  CUDA_TRY(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
  {
    cudaMemPoolProps props = {};
    props.allocType = cudaMemAllocationTypePinned;
    props.location.type = cudaMemLocationTypeDevice;
    props.location.id = c->device;
    CUDA_TRY(cudaMemPoolCreate(&c->scene_pool, &props));
    uint64_t keep = UINT64_MAX;  // freed scene memory stays with the pool for the next upload
    CUDA_TRY(cudaMemPoolSetAttribute(c->scene_pool, cudaMemPoolAttrReleaseThreshold, &keep));
    std::lock_guard<std::mutex> g(g_pools_mu);
    g_pools.push_back(c->scene_pool);
  }
  for (cudaStream_t& x : c->xstream) CUDA_TRY(cudaStreamCreateWithFlags(&x, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreate(&c->ev0));
  CUDA_TRY(cudaEventCreate(&c->ev1));
  CUDA_TRY(cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming));
  for (cudaEvent_t& e : c->ev_join) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  for (cudaEvent_t& e : c->ev_film) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  size_t free_b = 0, total_b = 0;
  CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
  c->budget = (opts && opts->memory_budget > 0) ? opts->memory_budget : (int64_t)(free_b * 0.9);
  std::string path = (opts && opts->sobol_path) ? std::string(opts->sobol_path) : default_sobol_path();
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return fail(ORION_ERR_IO, "cannot open Sobol matrices " + path);
  std::vector<uint32_t> m((size_t)kSobolDims * kSobolBits);
  size_t got = std::fread(m.data(), sizeof(uint32_t), m.size(), f);
  std::fclose(f);
  if (got != m.size()) return fail(ORION_ERR_IO, "short Sobol matrix file " + path);
  // Device form: for each dimension and each byte of the sample index, the XOR
  // of that byte's direction numbers for all 256 byte values, so a sample is
  // one lookup per non-zero index byte (sobol_sample, dmath.cuh).
  std::vector<uint32_t> tab((size_t)kSobolDims * kSobolBytes * 256);
  for (int d = 0; d < kSobolDims; ++d)
    for (int k = 0; k < kSobolBytes; ++k) {
      uint32_t* t = tab.data() + ((size_t)d * kSobolBytes + k) * 256;
      t[0] = 0u;
      for (int v = 1; v < 256; ++v) {  // v's lowest set bit j, and v without it
        const int j = __builtin_ctz((unsigned)v), b = 8 * k + j;
        t[v] = t[v & (v - 1)] ^ (b < kSobolBits ? m[(size_t)d * kSobolBits + b] : 0u);
      }
    }
  int rc = c->sobol.alloc(tab.size() * sizeof(uint32_t));
  if (rc != ORION_OK) return rc;
  CUDA_TRY(cudaMemcpy(c->sobol.p, tab.data(), tab.size() * sizeof(uint32_t), cudaMemcpyHostToDevice));
  c->cfg.num_sms = c->num_sms;
  c->cfg.trace_block = 128;
  c->cfg.shade_block = 128;
  c->cfg.blocks_per_sm = 6;
  c->cfg.smem_stack = 8;  // C2: 798 Mpaths/s against 793 at 16, 781 at 0, 721 at 24
  c->cfg.refill_below = 20;
  c->smem_limit = (int)prop.sharedMemPerBlockOptin;
  c->limits = KernelLimits{1024, 1024};
  CUDA_TRY(configure_kernels(c->smem_limit, &c->limits));
  CUDA_TRY(configure_batch_kernels(c->smem_limit, &c->limits));
  *out = c.release();
  return ORION_OK;
}

extern "C" int orion_gpu_destroy(orion_gpu_ctx* ctx) {
  if (!ctx) return ORION_OK;
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  for (cudaStream_t x : ctx->xstream)
    if (x) cudaStreamSynchronize(x);
  ctx->scenes.clear();
  cudaStreamSynchronize(ctx->stream);  // the scenes' pooled memory is back in the pool
  ctx->wave.block.alloc(0);
  for (Wave& w : ctx->xwave) w.block.alloc(0);
  for (BatchEngine& e : ctx->beng) e.drop_graph();
  for (cudaEvent_t e : ctx->prof_events) cudaEventDestroy(e);
  if (ctx->ev0) cudaEventDestroy(ctx->ev0);
  if (ctx->ev1) cudaEventDestroy(ctx->ev1);
  if (ctx->ev_fork) cudaEventDestroy(ctx->ev_fork);
  for (cudaEvent_t e : ctx->ev_join)
    if (e) cudaEventDestroy(e);
  for (cudaEvent_t e : ctx->ev_film)
    if (e) cudaEventDestroy(e);
  for (cudaStream_t x : ctx->xstream)
    if (x) cudaStreamDestroy(x);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  if (ctx->scene_pool) {
    {
      std::lock_guard<std::mutex> g(g_pools_mu);
      g_pools.erase(std::remove(g_pools.begin(), g_pools.end(), ctx->scene_pool), g_pools.end());
    }
    cudaMemPoolDestroy(ctx->scene_pool);
  }
  delete ctx;
  return ORION_OK;
}

template <class T>
static int upload(DevBuf& b, const std::vector<T>& v, cudaMemPool_t pool, cudaStream_t s, int64_t* bytes) {
  int rc = b.alloc_pooled(v.size() * sizeof(T), pool, s);
  if (rc != ORION_OK) return rc;
  if (!v.empty()) CUDA_TRY(cudaMemcpyAsync(b.p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  *bytes += (int64_t)b.bytes;
  return ORION_OK;
}

extern "C" int orion_gpu_scene_upload(orion_gpu_ctx* ctx, const orion_host_scene* scene, orion_scene_id* out) {
  if (!ctx || !scene || !out) return fail(ORION_ERR_INVALID, "null argument");
  NvtxRange range("orion_gpu_scene_upload");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  const HostScene& hs = scene->s;
  orion_host_scene* hsm = const_cast<orion_host_scene*>(scene);
  {
    std::lock_guard<std::mutex> sg(hsm->mu);
    if (!hsm->prep) {
      std::unique_ptr<PreparedScene> ps(new PreparedScene());
      std::string err;
      if (!prepare_scene(hs, ps.get(), &err)) return fail(ORION_ERR_INVALID, err);
      if (ps->env_idx.size() > 8) return fail(ORION_ERR_UNSUPPORTED, "more than 8 environment lights");
      hsm->prep = std::move(ps);
    }
    if (!hsm->bvh) {
      std::unique_ptr<BvhBuild> b(new BvhBuild());
      BvhBuildOptions bo;
      bo.wide = true;
      bo.max_leaf = 3;
      build_bvh(hs.positions.data(), hs.num_prims(), bo, b.get());
      if (b->depth >= kMaxBvhDepth) return fail(ORION_ERR_UNSUPPORTED, "BVH deeper than the traversal stack bound");
      hsm->tri_class.resize(b->tri_prim.size());
      hsm->class_mask = 1u << SC_MISS;
      for (size_t i = 0; i < hsm->tri_class.size(); ++i) {
        hsm->tri_class[i] = (uint8_t)hsm->prep->mats[hsm->prep->prims[b->tri_prim[i]].material].shade_class;
        hsm->class_mask |= 1u << hsm->tri_class[i];
      }
      hsm->bvh = std::move(b);
      pin(hsm, hsm->bvh->wide);
      pin(hsm, hsm->bvh->woop);
      pin(hsm, hsm->bvh->tri_prim);
      pin(hsm, hsm->tri_class);
      pin(hsm, hsm->prep->prims);
    }
  }
  const PreparedScene& ps = *hsm->prep;
  const BvhBuild& bvh = *hsm->bvh;
  std::unique_ptr<DeviceScene> d(new DeviceScene());
  int64_t bytes = 0;
  int rc;
  if ((rc = upload(d->nodes, bvh.wide, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->woop, bvh.woop, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->tri_prim, bvh.tri_prim, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  d->class_mask = hsm->class_mask;
  if ((rc = upload(d->tri_class, hsm->tri_class, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->prims, ps.prims, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->mats, ps.mats, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->lights, ps.lights, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->lfunc, ps.light_func, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  if ((rc = upload(d->lcdf, ps.light_cdf, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  // Image environment maps: the float block, then their records pointing into it.
  if ((rc = upload(d->env_data, ps.env_data, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  std::vector<DevEnvMap> envs;
  const float* eb = d->env_data.as<float>();
  for (const PreparedScene::EnvMapLayout& e : ps.envmaps)
    envs.push_back(DevEnvMap{e.width, e.height, e.marg_int, 0, eb + e.texels, eb + e.cond_func, eb + e.cond_cdf,
                             eb + e.cond_int, eb + e.marg_func, eb + e.marg_cdf});
  if ((rc = upload(d->envmaps, envs, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  // Image textures: records pointing into the same block, the materials'
  // builder inputs, and per-primitive texture coordinates.
  std::vector<DevTexture> texs;
  for (const PreparedScene::TextureLayout& t : ps.textures) texs.push_back(DevTexture{t.width, t.height, eb + t.texels});
  if (!texs.empty()) {
    if ((rc = upload(d->textures, texs, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
    if ((rc = upload(d->mat_src, ps.mat_src, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
    if ((rc = upload(d->prim_uv, ps.prim_uv, ctx->scene_pool, ctx->stream, &bytes)) != ORION_OK) return rc;
  }
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  SceneView& v = d->view;
  v.nodes = d->nodes.as<float4>();
  v.woop = d->woop.as<float4>();
  v.tri_prim = d->tri_prim.as<int>();
  v.tri_class = d->tri_class.as<uint8_t>();
  v.prims = d->prims.as<PrimShade>();
  v.mats = d->mats.as<DevMaterial>();
  v.lights = d->lights.as<DevLight>();
  v.light_func = d->lfunc.as<float>();
  v.light_cdf = d->lcdf.as<float>();
  v.envmaps = d->envmaps.as<DevEnvMap>();
  v.textures = d->textures.as<DevTexture>();
  v.mat_src = d->mat_src.as<DevMaterialSrc>();
  v.prim_uv = d->prim_uv.as<float>();
  v.class_mask = d->class_mask;
  v.light_func_int = ps.light_func_int;
  v.num_lights = (int)ps.lights.size();
  v.num_env = (int)ps.env_idx.size();
  v.num_area_lights = 0;
  for (const DevLight& l : ps.lights) v.num_area_lights += l.kind == DL_AREA ? 1 : 0;
  for (int i = 0; i < v.num_env; ++i) v.env_idx[i] = ps.env_idx[i];
  v.world_radius = ps.world_radius;
  for (int k = 0; k < 3; ++k) v.world_center[k] = ps.world_center[k];
  v.cam = ps.cam;
  d->bytes = bytes;
  d->num_prims = hs.num_prims();
  d->width = hs.camera.width;
  d->height = hs.camera.height;
  d->spp = hs.spp;
  d->max_depth = hs.max_depth;
  d->bvh_depth = bvh.depth;
  d->sppm = hs.sppm;
  int id = ctx->next_id++;
  ctx->scenes[id] = std::move(d);
  *out = id;
  return ORION_OK;
}

extern "C" int orion_gpu_scene_release(orion_gpu_ctx* ctx, orion_scene_id id) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> g(ctx->mu);
  cudaSetDevice(ctx->device);
  cudaStreamSynchronize(ctx->stream);
  if (!ctx->scenes.erase(id)) return fail(ORION_ERR_INVALID, "unknown scene id");
  return ORION_OK;
}

extern "C" int orion_gpu_scene_bytes(orion_gpu_ctx* ctx, orion_scene_id id, int64_t* bytes) {
  if (!ctx || !bytes) return fail(ORION_ERR_INVALID, "null argument");
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  *bytes = it->second->bytes;
  return ORION_OK;
}

// ------------------------------------------------------------- render

static int render_impl(orion_gpu_ctx* ctx, orion_scene_id id, const orion_render_params* params, float* film_rgb,
                       uint32_t* film_count, double* sum64, double* sumsq64, bool take_lock = true) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  NvtxRange range("orion_gpu_render");
  std::unique_lock<std::mutex> g(ctx->mu, std::defer_lock);
  if (take_lock) g.lock();
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  DeviceScene& d = *it->second;
  orion_render_params p{};
  if (params) p = *params;
  const int spp = p.spp > 0 ? p.spp : d.spp;
  const int max_depth = p.max_depth >= 0 && params ? p.max_depth : d.max_depth;
  const int rr_depth = params ? p.rr_depth : 3;
  if (max_depth < 0 || max_depth > 120) return fail(ORION_ERR_INVALID, "max_depth out of range");
  const int64_t wh = (int64_t)d.width * d.height;
  const int64_t total = wh * spp;
  const int64_t first = p.first_pass * wh;
  // Dimensions used: 5 + 2 (lens) + per bounce up to 8; the table has 1024.
  if (9 + 8 * (int64_t)(max_depth + 1) > 1024) return fail(ORION_ERR_INVALID, "max_depth exceeds Sobol dimensions");
  int64_t wave = p.wave_paths > 0 ? p.wave_paths : ctx->default_wave;
  wave = std::min<int64_t>(wave, std::max<int64_t>(total, 1));
  if (p.wave_paths <= 0 && !ctx->profiling) {
    // A render smaller than two waves is split into two equal waves (none
    // under 256K paths), so its waves overlap too. (Four ways, one per
    // stream, made the 1M-path Cornell render slower: 355 Mpaths/s against
    // 382-402 split two ways, in full bench runs.)
    const int64_t min_split = 1 << 18;
    int64_t nw = (total + wave - 1) / std::max<int64_t>(wave, 1);
    const int64_t want = std::min<int64_t>(std::min(ctx->wave_streams, 2), std::max<int64_t>(1, total / min_split));
    if (nw < want) nw = want;
    wave = std::max<int64_t>(1, (total + nw - 1) / nw);
  }
  int rc = ensure_wave(ctx, (int)wave);
  if (rc != ORION_OK) return rc;
  // Consecutive waves take turns on `ns` streams, each with its own
  // path-state block, so one wave's kernels fill the SMs that another's
  // kernel tails leave idle; the film is written wave after wave (events),
  // so every pixel still sums its samples in sample order. Profiled renders
  // stay on one stream so that stage times add up.
  const int64_t nwaves = (total + wave - 1) / wave;
  const int ns = ctx->profiling ? 1 : (int)std::min<int64_t>(ctx->wave_streams, nwaves);
  for (int i = 1; i < ns; ++i)
    if ((rc = alloc_wave(ctx->xwave[i - 1], (int)wave)) != ORION_OK) return rc;
  auto wave_view = [&](int i) -> const WaveView& { return i == 0 ? ctx->wave.view : ctx->xwave[i - 1].view; };
  auto wave_stream = [&](int i) { return i == 0 ? ctx->stream : ctx->xstream[i - 1]; };
  const bool fp64 = sum64 != nullptr;
  if ((rc = ensure_film(ctx, wh, fp64)) != ORION_OK) return rc;
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemsetAsync(ctx->film_sum.p, 0, wh * 3 * sizeof(float), s));
  CUDA_TRY(cudaMemsetAsync(ctx->film_count.p, 0, wh * sizeof(uint32_t), s));
  if (fp64) {
    CUDA_TRY(cudaMemsetAsync(ctx->film64.p, 0, wh * 3 * sizeof(double), s));
    CUDA_TRY(cudaMemsetAsync(ctx->filmsq64.p, 0, wh * 3 * sizeof(double), s));
  }
  const bool count_work = ctx->count_work;
  for (int i = 0; i < ns; ++i) {
    CUDA_TRY(cudaMemsetAsync(wave_view(i).ray_stats, 0, 10 * sizeof(unsigned long long), s));
    CUDA_TRY(cudaMemsetAsync(wave_view(i).error_word, 0, sizeof(int), s));
  }
  FilmView film{ctx->film_sum.as<float>(), ctx->film_count.as<uint32_t>(), fp64 ? ctx->film64.as<double>() : nullptr,
                fp64 ? ctx->filmsq64.as<double>() : nullptr};
  int launches = 0;
  StageTimer timer{nullptr, nullptr, 0, 0};
  if (ctx->profiling) {
    const int64_t waves = (total + wave - 1) / wave;
    const int need = (int)std::min<int64_t>(waves * (8 * (max_depth + 1) + 4), 200000);
    while ((int)ctx->prof_events.size() < 2 * need) {
      cudaEvent_t e;
      CUDA_TRY(cudaEventCreate(&e));
      ctx->prof_events.push_back(e);
    }
    ctx->prof_stage.resize(need);
    timer = StageTimer{ctx->prof_events.data(), ctx->prof_stage.data(), need, 0};
  }
  CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  if (ns > 1) {
    CUDA_TRY(cudaEventRecord(ctx->ev_fork, s));
    for (int i = 1; i < ns; ++i) CUDA_TRY(cudaStreamWaitEvent(wave_stream(i), ctx->ev_fork, 0));
  }
  int64_t k = 0;
  for (int64_t off = 0; off < total; off += wave, ++k) {
    const int slot = (int)(k % ns);
    WaveArgs a;
    a.sobol = ctx->sobol.as<uint32_t>();
    a.base_index = first + off;
    a.n_paths = (int)std::min<int64_t>(wave, total - off);
    a.width = d.width;
    a.height = d.height;
    a.max_depth = max_depth;
    a.rr_depth = rr_depth;
    a.class_mask = d.class_mask;
    const cudaEvent_t film_wait = ns > 1 && k > 0 ? ctx->ev_film[(k - 1) % ns] : nullptr;
    const cudaEvent_t film_done = ns > 1 ? ctx->ev_film[k % ns] : nullptr;
    WaveView wv = wave_view(slot);
    if (count_work) wv.trace_work = wv.ray_stats + 4;
    launch_wave(d.view, wv, a, film, ctx->cfg, wave_stream(slot), &launches, ctx->profiling ? &timer : nullptr,
                film_wait, film_done);
  }
  CUDA_TRY(cudaGetLastError());
  for (int i = 1; i < ns; ++i) {
    CUDA_TRY(cudaEventRecord(ctx->ev_join[i - 1], wave_stream(i)));
    CUDA_TRY(cudaStreamWaitEvent(s, ctx->ev_join[i - 1], 0));
  }
  CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  if (film_rgb)
    CUDA_TRY(cudaMemcpyAsync(film_rgb, ctx->film_sum.p, wh * 3 * sizeof(float), cudaMemcpyDeviceToHost, s));
  if (film_count)
    CUDA_TRY(cudaMemcpyAsync(film_count, ctx->film_count.p, wh * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  if (fp64) {
    CUDA_TRY(cudaMemcpyAsync(sum64, ctx->film64.p, wh * 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(sumsq64, ctx->filmsq64.p, wh * 3 * sizeof(double), cudaMemcpyDeviceToHost, s));
  }
  unsigned long long wstats[kMaxWaveStreams][10] = {};
  int werr[kMaxWaveStreams] = {};
  for (int i = 0; i < ns; ++i) {
    CUDA_TRY(cudaMemcpyAsync(wstats[i], wave_view(i).ray_stats, sizeof(wstats[i]), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(&werr[i], wave_view(i).error_word, sizeof(int), cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(cudaStreamSynchronize(s));
  unsigned long long stats[10] = {};
  int err_word = 0;
  for (int i = 0; i < ns; ++i) {
    for (int j = 0; j < 10; ++j) stats[j] += wstats[i][j];
    err_word = err_word ? err_word : werr[i];
  }
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  ctx->last.paths = total;
  ctx->last.ext_rays = (int64_t)stats[0];
  ctx->last.shadow_rays = (int64_t)stats[1];
  ctx->last.mis_rays = (int64_t)stats[2];
  ctx->last.rays = (int64_t)(stats[0] + stats[1] + stats[2]);
  ctx->last.kernel_launches = launches;
  ctx->last.device_ms = ms;
  std::memset(&ctx->last_work, 0, sizeof(ctx->last_work));
  if (count_work)
    for (int j = 0; j < 3; ++j) {
      ctx->last_work.rays[j] = (int64_t)stats[j];
      ctx->last_work.nodes[j] = (int64_t)stats[4 + j];
      ctx->last_work.triangles[j] = (int64_t)stats[7 + j];
    }
  std::memset(&ctx->stage_times, 0, sizeof(ctx->stage_times));
  for (int i = 0; i < std::min(timer.used, timer.capacity); ++i) {
    float e = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&e, timer.events[2 * i], timer.events[2 * i + 1]));
    ctx->stage_times.ms[timer.stage[i]] += e;
    ctx->stage_times.launches[timer.stage[i]] += 1;
  }
  if (err_word) return fail(ORION_ERR_DEVICE, kernel_error(err_word));
  return ORION_OK;
}

extern "C" int orion_gpu_render(orion_gpu_ctx* ctx, orion_scene_id id, const orion_render_params* params,
                                float* film_rgb_sum, uint32_t* film_count) {
  return render_impl(ctx, id, params, film_rgb_sum, film_count, nullptr, nullptr);
}

extern "C" int orion_gpu_render_fp64(orion_gpu_ctx* ctx, orion_scene_id id, const orion_render_params* params,
                                     double* sum, double* sumsq) {
  if (!sum || !sumsq) return fail(ORION_ERR_INVALID, "null output");
  return render_impl(ctx, id, params, nullptr, nullptr, sum, sumsq);
}

extern "C" int orion_gpu_last_stats(orion_gpu_ctx* ctx, orion_render_stats* out) {
  if (!ctx || !out) return fail(ORION_ERR_INVALID, "null argument");
  *out = ctx->last;
  return ORION_OK;
}

extern "C" int orion_gpu_set_profiling(orion_gpu_ctx* ctx, int32_t enable) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->profiling = (enable & ORION_PROFILE_STAGES) != 0;
  ctx->count_work = (enable & ORION_PROFILE_TRAVERSAL) != 0;
  return ORION_OK;
}

extern "C" int orion_gpu_traversal_work(orion_gpu_ctx* ctx, orion_traversal_work* out) {
  if (!ctx || !out) return fail(ORION_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  *out = ctx->last_work;
  return ORION_OK;
}

extern "C" int orion_gpu_stage_times(orion_gpu_ctx* ctx, orion_stage_times* out) {
  if (!ctx || !out) return fail(ORION_ERR_INVALID, "null argument");
  *out = ctx->stage_times;
  return ORION_OK;
}

// ------------------------------------------------------ internal hooks

namespace orion_gb300 {

int ctx_fail(int code, const char* msg) { return fail(code, msg); }
int ctx_device(orion_gpu_ctx* ctx) { return ctx->device; }
cudaStream_t ctx_stream(orion_gpu_ctx* ctx) { return ctx->stream; }
int64_t ctx_pool_bytes(orion_gpu_ctx* ctx) { return (int64_t)ctx->wave.block.bytes; }

int ctx_copy_to_host(orion_gpu_ctx* ctx, void* dst, const void* src, size_t bytes) {
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  CUDA_TRY(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

int ctx_film_preview(orion_gpu_ctx* ctx, const void* film, int width, int height, int bottom_up, uint8_t* bgra) {
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  const size_t wh = (size_t)width * height;
  if (ctx->preview.bytes < wh * 4) RC(ctx->preview.alloc(wh * 4));
  const char* base = static_cast<const char*>(film);
  launch_film_preview(reinterpret_cast<const double*>(base), reinterpret_cast<const uint32_t*>(base + wh * 48), width,
                      height, bottom_up, ctx->preview.as<uint8_t>(), ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(bgra, ctx->preview.p, wh * 4, cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

int ctx_scene_info(orion_gpu_ctx* ctx, orion_scene_id id, int* width, int* height, int* spp, int* max_depth) {
  std::lock_guard<std::mutex> g(ctx->mu);
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  *width = it->second->width;
  *height = it->second->height;
  *spp = it->second->spp;
  *max_depth = it->second->max_depth;
  return ORION_OK;
}

}  // namespace orion_gb300

// ---------------------------------------------------- launch config, tuning

extern "C" int orion_gpu_get_config(orion_gpu_ctx* ctx, orion_launch_config* out) {
  if (!ctx || !out) return fail(ORION_ERR_INVALID, "null argument");
  out->trace_block = ctx->cfg.trace_block;
  out->shade_block = ctx->cfg.shade_block;
  out->smem_stack = ctx->cfg.smem_stack;
  out->blocks_per_sm = ctx->cfg.blocks_per_sm;
  out->wave_paths = ctx->default_wave;
  out->batch_slots = ctx->default_batch_slots;
  out->refill_below = ctx->cfg.refill_below;
  out->streams = ctx->wave_streams;
  return ORION_OK;
}

extern "C" int orion_gpu_set_config(orion_gpu_ctx* ctx, const orion_launch_config* cfg) {
  if (!ctx || !cfg) return fail(ORION_ERR_INVALID, "null argument");
  LaunchConfig c = ctx->cfg;
  c.trace_block = cfg->trace_block;
  c.shade_block = cfg->shade_block;
  c.smem_stack = cfg->smem_stack;
  c.blocks_per_sm = cfg->blocks_per_sm;
  c.refill_below = cfg->refill_below;
  std::string why = config_problem(ctx, c);
  if (!why.empty()) return fail(ORION_ERR_INVALID, "launch configuration: " + why);
  if (cfg->wave_paths < 1024 || cfg->batch_slots < 1024)
    return fail(ORION_ERR_INVALID, "launch configuration: wave_paths and batch_slots must be >= 1024");
  if (cfg->streams < 0 || cfg->streams > kMaxWaveStreams)
    return fail(ORION_ERR_INVALID, "launch configuration: streams must be 0.." + std::to_string(kMaxWaveStreams));
  std::lock_guard<std::mutex> g(ctx->mu);
  if (cfg->streams > 0) {
    ctx->wave_streams = cfg->streams;
    ctx->batch_engines = std::min(cfg->streams, (int)orion_gpu_ctx::kBatchEngines);
  }
  ctx->cfg = c;
  ctx->default_wave = cfg->wave_paths;
  ctx->default_batch_slots = cfg->batch_slots;
  return ORION_OK;
}

// Coordinate descent over the launch knobs: each knob in turn is swept with
// the others held at the best values so far; each trial is one timed render
// (device time), repeated until the budget is used.
extern "C" int orion_gpu_autotune(orion_gpu_ctx* ctx, orion_scene_id id, int32_t spp, double budget_ms,
                                  orion_launch_config* best_out, double* best_mpaths) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  std::lock_guard<std::mutex> g(ctx->mu);
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  const DeviceScene& d = *it->second;
  const int64_t paths = (int64_t)d.width * d.height * std::max(1, spp);
  orion_render_params p{};
  p.spp = std::max(1, spp);
  p.max_depth = -1;
  p.rr_depth = 3;
  LaunchConfig best = ctx->cfg;
  int best_wave = ctx->default_wave, best_streams = ctx->wave_streams;
  double best_ms = 1e30, used = 0;
  auto trial = [&](const LaunchConfig& c, int wave, int streams, double* ms) -> int {
    LaunchConfig saved = ctx->cfg;
    int saved_wave = ctx->default_wave, saved_streams = ctx->wave_streams;
    ctx->cfg = c;
    ctx->default_wave = wave;
    ctx->wave_streams = streams;
    int rc = render_impl(ctx, id, &p, nullptr, nullptr, nullptr, nullptr, false);
    *ms = ctx->last.device_ms;
    ctx->cfg = saved;
    ctx->default_wave = saved_wave;
    ctx->wave_streams = saved_streams;
    used += *ms;
    return rc;
  };
  double ms;
  int rc = trial(best, best_wave, best_streams, &ms);  // warm-up and baseline
  if (rc != ORION_OK) return rc;
  rc = trial(best, best_wave, best_streams, &best_ms);
  if (rc != ORION_OK) return rc;
  const int trace_blocks[] = {64, 128, 256};
  const int stacks[] = {8, 16, 32};
  const int shade_blocks[] = {64, 128, 256};
  const int bpsm[] = {4, 6, 8, 12};
  const int waves[] = {1 << 22, 1 << 23, 1 << 24, 1 << 25};
  const int refills[] = {8, 16, 24, 32};
  const int stream_counts[] = {1, 2, 3, 4};
  for (int knob = 0; knob < 7 && used < budget_ms; ++knob) {
    int n = knob >= 3 ? 4 : 3;
    for (int v = 0; v < n && used < budget_ms; ++v) {
      LaunchConfig c = best;
      int wave = best_wave, streams = best_streams;
      if (knob == 0) c.trace_block = trace_blocks[v];
      if (knob == 1) c.smem_stack = stacks[v];
      if (knob == 2) c.shade_block = shade_blocks[v];
      if (knob == 3) c.blocks_per_sm = bpsm[v];
      if (knob == 4) wave = waves[v];
      if (knob == 5) c.refill_below = refills[v];
      if (knob == 6) streams = stream_counts[v];
      if (wave > 2 * paths && wave != best_wave) continue;
      if (std::memcmp(&c, &best, sizeof(c)) == 0 && wave == best_wave && streams == best_streams) continue;
      if (!config_problem(ctx, c).empty()) continue;
      rc = trial(c, wave, streams, &ms);
      if (rc == ORION_ERR_NOMEM) continue;
      if (rc != ORION_OK) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
        best_wave = wave;
        best_streams = streams;
      }
    }
  }
  ctx->cfg = best;
  ctx->default_wave = best_wave;
  ctx->wave_streams = best_streams;
  ctx->default_batch_slots = best_wave;
  if (best_out) {
    best_out->trace_block = best.trace_block;
    best_out->shade_block = best.shade_block;
    best_out->smem_stack = best.smem_stack;
    best_out->blocks_per_sm = best.blocks_per_sm;
    best_out->wave_paths = best_wave;
    best_out->batch_slots = best_wave;
    best_out->refill_below = best.refill_below;
    best_out->streams = ctx->wave_streams;
  }
  if (best_mpaths) *best_mpaths = paths / (best_ms * 1e-3) / 1e6;
  return ORION_OK;
}

// --------------------------------------------------------- test hooks

namespace {
template <class T>
int to_device(DevBuf& b, const T* host, size_t n, cudaStream_t s) {
  int rc = b.alloc(n * sizeof(T));
  if (rc != ORION_OK) return rc;
  if (n) CUDA_TRY(cudaMemcpyAsync(b.p, host, n * sizeof(T), cudaMemcpyHostToDevice, s));
  return ORION_OK;
}
template <class T>
int to_host(T* host, const DevBuf& b, size_t n, cudaStream_t s) {
  if (n) CUDA_TRY(cudaMemcpyAsync(host, b.p, n * sizeof(T), cudaMemcpyDeviceToHost, s));
  return ORION_OK;
}
}  // namespace


extern "C" int orion_gpu_sobol(orion_gpu_ctx* ctx, int64_t n, const uint64_t* index, const uint32_t* dim, float* out) {
  if (!ctx || n < 0 || (n > 0 && (!index || !dim || !out))) return fail(ORION_ERR_INVALID, "bad argument");
  for (int64_t i = 0; i < n; ++i)
    if (dim[i] >= 1024) return fail(ORION_ERR_INVALID, "Sobol dimension >= 1024");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  DevBuf di, dd, dout;
  RC(to_device(di, index, n, ctx->stream));
  RC(to_device(dd, dim, n, ctx->stream));
  RC(dout.alloc(n * sizeof(float)));
  launch_sobol(ctx->sobol.as<uint32_t>(), n, di.as<uint64_t>(), dd.as<uint32_t>(), dout.as<float>(), ctx->stream);
  CUDA_TRY(cudaGetLastError());
  RC(to_host(out, dout, n, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

extern "C" int orion_gpu_trace(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays, int32_t any_hit,
                               float* t, float* u, float* v, int32_t* prim) {
  if (!ctx || n < 0 || (n > 0 && (!rays || !t || !u || !v || !prim))) return fail(ORION_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  DevBuf dr, dt, du, dv, dp;
  RC(to_device(dr, rays, 8 * (size_t)n, ctx->stream));
  RC(dt.alloc(n * 4));
  RC(du.alloc(n * 4));
  RC(dv.alloc(n * 4));
  RC(dp.alloc(n * 4));
  launch_trace(it->second->view, n, dr.as<float>(), any_hit, dt.as<float>(), du.as<float>(), dv.as<float>(),
               dp.as<int>(), ctx->cfg, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  RC(to_host(t, dt, n, ctx->stream));
  RC(to_host(u, du, n, ctx->stream));
  RC(to_host(v, dv, n, ctx->stream));
  RC(to_host(prim, dp, n, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

extern "C" int orion_gpu_trace_wave(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays,
                                    int32_t any_hit, float* t, float* u, float* v, int32_t* prim) {
  if (!ctx || n < 0 || (n > 0 && (!rays || !t || !u || !v || !prim))) return fail(ORION_ERR_INVALID, "bad argument");
  if (n > (int64_t)1 << 30) return fail(ORION_ERR_INVALID, "orion_gpu_trace_wave: more than 2^30 rays");
  for (int64_t i = 0; i < n; ++i)
    if (rays[8 * i + 6] != 0.f)
      return fail(ORION_ERR_INVALID, "orion_gpu_trace_wave: tnear must be 0 (ray " + std::to_string(i) + ")");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  if (n == 0) return ORION_OK;
  RC(ensure_wave(ctx, (int)n));
  const WaveView& w = ctx->wave.view;
  DevBuf dr, dt, du, dv, dp;
  RC(to_device(dr, rays, 8 * (size_t)n, ctx->stream));
  RC(dt.alloc(n * 4));
  RC(du.alloc(n * 4));
  RC(dv.alloc(n * 4));
  RC(dp.alloc(n * 4));
  CUDA_TRY(cudaMemsetAsync(w.error_word, 0, sizeof(int), ctx->stream));
  launch_trace_wave(it->second->view, w, (int)n, dr.as<float>(), any_hit, dt.as<float>(), du.as<float>(),
                    dv.as<float>(), dp.as<int>(), ctx->cfg, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  int err_word = 0;
  RC(to_host(t, dt, n, ctx->stream));
  RC(to_host(u, du, n, ctx->stream));
  RC(to_host(v, dv, n, ctx->stream));
  RC(to_host(prim, dp, n, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(&err_word, w.error_word, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  if (err_word) return fail(ORION_ERR_DEVICE, kernel_error(err_word));
  return ORION_OK;
}

extern "C" int orion_gpu_mem_info(orion_gpu_ctx* ctx, int64_t* free_bytes, int64_t* total_bytes) {
  if (!ctx || !free_bytes || !total_bytes) return fail(ORION_ERR_INVALID, "null argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  size_t f = 0, t = 0;
  CUDA_TRY(cudaMemGetInfo(&f, &t));
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  return ORION_OK;
}

extern "C" int orion_gpu_set_test_limits(orion_gpu_ctx* ctx, int32_t stack_entries, int32_t batch_iterations) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  if (!(stack_entries == 0 || stack_entries == kTestStackEntries))
    return fail(ORION_ERR_INVALID, "stack_entries must be 0 or " + std::to_string(kTestStackEntries));
  if (batch_iterations < 0) return fail(ORION_ERR_INVALID, "batch_iterations must be >= 0");
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->cfg.test_stack_entries = stack_entries;
  ctx->cfg.test_batch_iterations = batch_iterations;
  for (orion_gb300::BatchEngine& e : ctx->beng) e.drop_graph();  // captured loops hold the old kernels
  return ORION_OK;
}

extern "C" int orion_gpu_trace_noalloc(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const float* rays,
                                       int32_t any_hit, float* t, float* u, float* v, int32_t* prim) {
  if (!ctx || n < 0 || (n > 0 && (!rays || !t || !u || !v || !prim))) return fail(ORION_ERR_INVALID, "bad argument");
  if (n > ORION_NOALLOC_MAX_RAYS)
    return fail(ORION_ERR_INVALID, "orion_gpu_trace_noalloc: " + std::to_string(n) +
                                       " rays exceed its fixed scratch of ORION_NOALLOC_MAX_RAYS = " +
                                       std::to_string(ORION_NOALLOC_MAX_RAYS) +
                                       " rays; split the query or call orion_gpu_trace");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  unsigned char* base = nullptr;
  std::string err;
  if (noalloc_trace_scratch(ctx->device, &base, &err) != cudaSuccess) return fail(ORION_ERR_CUDA, err);
  if (n == 0) return ORION_OK;
  float *dr, *dt, *du, *dv;
  int* dp;
  noalloc_trace_layout(base, &dr, &dt, &du, &dv, &dp);
  CUDA_TRY(cudaMemcpyAsync(dr, rays, (size_t)n * 8 * sizeof(float), cudaMemcpyHostToDevice, ctx->stream));
  launch_trace(it->second->view, n, dr, any_hit, dt, du, dv, dp, ctx->cfg, ctx->stream);
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpyAsync(t, dt, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(u, du, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(v, dv, (size_t)n * sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaMemcpyAsync(prim, dp, (size_t)n * sizeof(int32_t), cudaMemcpyDeviceToHost, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

extern "C" int orion_gpu_camera_rays(orion_gpu_ctx* ctx, orion_scene_id id, int64_t n, const int64_t* sample_index,
                                     float* rays) {
  if (!ctx || n < 0 || (n > 0 && (!sample_index || !rays))) return fail(ORION_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  auto it = ctx->scenes.find(id);
  if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
  for (int64_t i = 0; i < n; ++i)
    if (sample_index[i] < 0) return fail(ORION_ERR_INVALID, "negative sample index");
  DevBuf di, dr;
  RC(to_device(di, sample_index, n, ctx->stream));
  RC(dr.alloc(6 * n * sizeof(float)));
  launch_camera_rays(it->second->view, ctx->sobol.as<uint32_t>(), n, di.as<int64_t>(), dr.as<float>(), ctx->stream);
  CUDA_TRY(cudaGetLastError());
  RC(to_host(rays, dr, 6 * (size_t)n, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}

extern "C" int orion_gpu_bsdf_eval(orion_gpu_ctx* ctx, const orion_material* mat, int64_t n, const float* frame,
                                   const float* wo, const float* wi, const float* rnd, int32_t type, float* f,
                                   float* pdf, float* sf, float* swi, float* spdf, int32_t* stype, int32_t* nbxdf) {
  if (!ctx || !mat || n < 0) return fail(ORION_ERR_INVALID, "bad argument");
  if (mat->type < ORION_MAT_MATTE || mat->type > ORION_MAT_UBER) return fail(ORION_ERR_INVALID, "bad material type");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  DevMaterial dm = prepare_material(*mat);
  DevBuf dmat, dfr, dwo, dwi, drn, df, dpdf, dsf, dswi, dspdf, dst, dnb;
  RC(to_device(dmat, &dm, 1, ctx->stream));
  RC(to_device(dfr, frame, 12 * (size_t)n, ctx->stream));
  RC(to_device(dwo, wo, 3 * (size_t)n, ctx->stream));
  RC(to_device(dwi, wi, 3 * (size_t)n, ctx->stream));
  RC(to_device(drn, rnd, 2 * (size_t)n, ctx->stream));
  RC(df.alloc(12 * n));
  RC(dpdf.alloc(4 * n));
  RC(dsf.alloc(12 * n));
  RC(dswi.alloc(12 * n));
  RC(dspdf.alloc(4 * n));
  RC(dst.alloc(4 * n));
  RC(dnb.alloc(4 * n));
  launch_bsdf_eval(dmat.as<DevMaterial>(), n, dfr.as<float>(), dwo.as<float>(), dwi.as<float>(), drn.as<float>(), type,
                   df.as<float>(), dpdf.as<float>(), dsf.as<float>(), dswi.as<float>(), dspdf.as<float>(),
                   dst.as<int>(), dnb.as<int>(), ctx->stream);
  CUDA_TRY(cudaGetLastError());
  RC(to_host(f, df, 3 * (size_t)n, ctx->stream));
  RC(to_host(pdf, dpdf, (size_t)n, ctx->stream));
  RC(to_host(sf, dsf, 3 * (size_t)n, ctx->stream));
  RC(to_host(swi, dswi, 3 * (size_t)n, ctx->stream));
  RC(to_host(spdf, dspdf, (size_t)n, ctx->stream));
  RC(to_host(stype, dst, (size_t)n, ctx->stream));
  RC(to_host(nbxdf, dnb, (size_t)n, ctx->stream));
  CUDA_TRY(cudaStreamSynchronize(ctx->stream));
  return ORION_OK;
}
