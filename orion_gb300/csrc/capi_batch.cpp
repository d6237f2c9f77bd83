// C ABI, batched rendering (include/orion_gpu.h: orion_gpu_render_batch,
// orion_gpu_set_batch_mode, orion_gpu_autotune_batch).
//
// PathTracing::render (src/integrator/path.cpp:15-37) renders one scene per
// call. A batch renders many (scene, spp, film) jobs in one device-side loop,
// captured once as a CUDA graph and replayed until every job's samples are
// done. Two modes share the plain render's kernels:
//   pooled - a fixed pool of path slots; finished paths retire their film
//            sample and the slot takes the next sample index of any job;
//   waves  - the jobs' sample indices are laid end to end and cut into waves
//            of `batch_slots` paths, each wave run to completion.
// Up to two engines run a batch concurrently, engine e on the wave state and
// stream of plain-render wave slot e.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <string>
#include <vector>

#include "context.h"

using namespace orion_gb300;

// Wave state and stream of batch engine e (shared with plain-render wave slot e).
static Wave& engine_wave(orion_gpu_ctx* ctx, int e) { return e == 0 ? ctx->wave : ctx->xwave[e - 1]; }
static cudaStream_t engine_stream(orion_gpu_ctx* ctx, int e) { return e == 0 ? ctx->stream : ctx->xstream[e - 1]; }

// The captured loop launches the shading kernels of the classes in `mask`;
// a graph that launches a superset is reused (an absent class's kernel
// finds an empty queue), so the mask of a long-lived context only grows.
static int build_batch_graph(orion_gpu_ctx* ctx, int e, int mode, const BatchView& bv, int slots, unsigned mask) {
  BatchEngine& eng = ctx->beng[e];
  BatchGraph& be = eng.loop[mode];
  Wave& wave = engine_wave(ctx, e);
  const void* key[4] = {wave.block.p, eng.jobs.p, eng.retire.p, eng.ctl.p};
  bool same = be.exec && be.slots == slots && std::memcmp(key, be.key, sizeof(key)) == 0 &&
              std::memcmp(&be.cfg, &ctx->cfg, sizeof(LaunchConfig)) == 0 && (mask & ~be.mask) == 0;
  if (same) return ORION_OK;
  if (be.exec) mask |= be.mask;
  be.drop();
  CUDA_TRY(cudaGraphCreate(&be.graph, 0));
  cudaGraphConditionalHandle cond;
  CUDA_TRY(cudaGraphConditionalHandleCreate(&cond, be.graph, 1, cudaGraphCondAssignDefault));
  // cudaGraphNodeParams has no usable default constructor in host C++;
  // zeroed storage is its documented initial state.
  alignas(cudaGraphNodeParams) unsigned char np_storage[sizeof(cudaGraphNodeParams)] = {};
  cudaGraphNodeParams& np = *reinterpret_cast<cudaGraphNodeParams*>(np_storage);
  np.type = cudaGraphNodeTypeConditional;
  np.conditional.handle = cond;
  np.conditional.type = cudaGraphCondTypeWhile;
  np.conditional.size = 1;
  cudaGraphNode_t node;
  CUDA_TRY(cudaGraphAddNode(&node, be.graph, nullptr, nullptr, 0, &np));
  cudaGraph_t body = np.conditional.phGraph_out[0];
  cudaError_t ce = capture_batch_iteration(wave.view, bv, ctx->sobol.as<uint32_t>(), ctx->cfg, mask, mode == ORION_BATCH_WAVES, cond, engine_stream(ctx, e), body);
  if (ce != cudaSuccess) {
    // A graph whose loop-body capture was invalidated is dropped, not
    // destroyed: nothing is assumed about its state after the failure.
    be.graph = nullptr;
    cudaGetLastError();
    return fail(ORION_ERR_CUDA, std::string("batch loop capture: ") + cudaGetErrorString(ce));
  }
  CUDA_TRY(cudaGraphInstantiate(&be.exec, be.graph, 0));
  std::memcpy(be.key, key, sizeof(key));
  be.cfg = ctx->cfg;
  be.slots = slots;
  be.mask = mask;
  return ORION_OK;
}

// Buffers of engine e for `njobs` jobs and up to `slots` path slots.
static int prepare_engine(orion_gpu_ctx* ctx, int e, int njobs, int slots, BatchView* bv, int* cap) {
  BatchEngine& be = ctx->beng[e];
  Wave& wave = engine_wave(ctx, e);
  int rc;
  if ((rc = alloc_wave(wave, slots)) != ORION_OK) return rc;
  *cap = wave.capacity;
  if (be.slots_alloc < *cap) {
    if ((rc = be.retire.alloc((size_t)*cap * 4)) != ORION_OK) return rc;
    if ((rc = be.free_list.alloc((size_t)*cap * 4)) != ORION_OK) return rc;
    be.slots_alloc = *cap;
  }
  if (!be.ctl.p && (rc = be.ctl.alloc(sizeof(BatchCtl))) != ORION_OK) return rc;
  if (be.jobs_alloc < njobs) {
    const int n = std::max(njobs, 64);
    if ((rc = be.jobs.alloc((size_t)n * sizeof(DevJob))) != ORION_OK) return rc;
    be.jobs_alloc = n;
  }
  bv->jobs = be.jobs.as<DevJob>();
  bv->ctl = be.ctl.as<BatchCtl>();
  bv->q_retire = be.retire.as<int>();
  bv->q_free = be.free_list.as<int>();
  return ORION_OK;
}

// Control block of a fresh batch of `total` work items on `cap` slots.
// `test_iterations` > 0 (orion_gpu_set_test_limits) replaces the loop bound.
static BatchCtl initial_ctl(unsigned long long total, int njobs, int cap, int max_depth_all, int test_iterations) {
  BatchCtl c;
  std::memset(&c, 0, sizeof(c));
  c.total = total;
  c.njobs = njobs;
  c.counters[CNT_FREE] = cap;
  // Every live path advances one bounce per iteration: a bound on the loop.
  const unsigned long long refills = (total + cap - 1) / cap + 1;
  c.max_iterations = (int)std::min<unsigned long long>(2ULL * refills * (max_depth_all + 2) + 64, 1u << 30);
  if (test_iterations > 0) c.max_iterations = test_iterations;
  return c;
}

// The error a batch's control block reports (its error bits), or "" for none.
static std::string batch_error(int bits) {
  std::string m;
  if (bits & kErrIterationCap) m += "batch loop reached its iteration cap";
  if (bits & kErrTraversalStack) m += std::string(m.empty() ? "" : "; ") + "a traversal overflowed its stack";
  return m;
}

// One batch over `dj` (film pointers set; films zeroed or holding earlier
// passes to add to, in stream order on ctx->stream before this call).
// Caller holds ctx->mu. With more than one job, the jobs are split into
// groups of about equal path counts, one per engine, and the engines run
// concurrently on their own streams (each group's paths fill the SMs the
// other group's kernel tails leave idle). Profiled batches run on one
// engine, driven from the host. On return `out` holds the engines' summed
// counts (iterations: the most any engine ran), `ms` the device time.
static int run_batch_pooled_locked(orion_gpu_ctx* ctx, std::vector<DevJob>& dj, unsigned long long total,
                                   int max_depth_all, BatchCtl* out_ctl, float* ms_out) {
  const int njobs = (int)dj.size();
  int rc;
  const int ne = ctx->profiling ? 1 : std::min(std::min(ctx->batch_engines, (int)orion_gpu_ctx::kBatchEngines), njobs);
  // Split by path count: largest jobs first, each to the lighter group.
  std::vector<std::vector<DevJob>> group(ne);
  std::vector<unsigned long long> gtotal(ne, 0);
  std::vector<int> order(njobs);
  for (int i = 0; i < njobs; ++i) order[i] = i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return dj[a].num_paths > dj[b].num_paths; });
  for (int i : order) {
    int g = 0;
    for (int k = 1; k < ne; ++k)
      if (gtotal[k] < gtotal[g]) g = k;
    DevJob J = dj[i];
    J.work_begin = (long long)gtotal[g];
    group[g].push_back(J);
    gtotal[g] += (unsigned long long)J.num_paths;
  }
  int ng = 0;  // engines with work
  for (int g = 0; g < ne; ++g) ng += gtotal[g] > 0 ? 1 : 0;
  if (ng == 0) ng = 1;
  std::vector<BatchView> bvs(ng);
  std::vector<int> caps(ng);
  std::vector<unsigned> masks(ng, 1u << SC_MISS);
  for (int e = 0; e < ng; ++e) {
    const int slots = (int)std::min<unsigned long long>((unsigned long long)ctx->default_batch_slots,
                                                         std::max<unsigned long long>(gtotal[e], 1024ULL));
    if ((rc = prepare_engine(ctx, e, (int)group[e].size(), slots, &bvs[e], &caps[e])) != ORION_OK) return rc;
    for (const DevJob& J : group[e]) masks[e] |= J.scene.class_mask;
    if (!ctx->profiling && (rc = build_batch_graph(ctx, e, ORION_BATCH_POOLED, bvs[e], caps[e], masks[e])) != ORION_OK)
      return rc;
  }
  cudaStream_t s = ctx->stream;
  std::memset(&ctx->stage_times, 0, sizeof(ctx->stage_times));
  CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  if (ng > 1) {
    CUDA_TRY(cudaEventRecord(ctx->ev_fork, s));
    for (int e = 1; e < ng; ++e) CUDA_TRY(cudaStreamWaitEvent(engine_stream(ctx, e), ctx->ev_fork, 0));
  }
  std::vector<BatchCtl> init(ng);
  for (int e = 0; e < ng; ++e) {
    cudaStream_t es = engine_stream(ctx, e);
    init[e] = initial_ctl(gtotal[e], (int)group[e].size(), caps[e], max_depth_all, ctx->cfg.test_batch_iterations);
    if (!group[e].empty())
      CUDA_TRY(cudaMemcpyAsync(bvs[e].jobs, group[e].data(), group[e].size() * sizeof(DevJob),
                               cudaMemcpyHostToDevice, es));
    CUDA_TRY(cudaMemcpyAsync(bvs[e].ctl, &init[e], sizeof(BatchCtl), cudaMemcpyHostToDevice, es));
    launch_batch_init(engine_wave(ctx, e).view, bvs[e], caps[e], es);
    CUDA_TRY(cudaGetLastError());
  }
  if (ctx->profiling) {
    // Profiling: the same iterations driven from the host, every stage timed
    // (one host round trip per iteration, so device_ms includes those gaps).
    const int per_iter = 8;
    const int need = (int)std::min<int64_t>((int64_t)init[0].max_iterations * per_iter, 200000);
    while ((int)ctx->prof_events.size() < 2 * need) {
      cudaEvent_t e;
      CUDA_TRY(cudaEventCreate(&e));
      ctx->prof_events.push_back(e);
    }
    ctx->prof_stage.resize(need);
    StageTimer timer{ctx->prof_events.data(), ctx->prof_stage.data(), need, 0};
    int more = 1;
    for (int it = 0; more && it < init[0].max_iterations; ++it) {
      launch_batch_iteration(ctx->wave.view, bvs[0], ctx->sobol.as<uint32_t>(), ctx->cfg, masks[0], false, s,
                             &timer);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(&more, &bvs[0].ctl->more, sizeof(int), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
    }
    CUDA_TRY(cudaEventRecord(ctx->ev1, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    for (int i = 0; i < std::min(timer.used, timer.capacity); ++i) {
      float e = 0.f;
      CUDA_TRY(cudaEventElapsedTime(&e, timer.events[2 * i], timer.events[2 * i + 1]));
      ctx->stage_times.ms[timer.stage[i]] += e;
      ctx->stage_times.launches[timer.stage[i]] += 1;
    }
  } else {
    for (int e = 0; e < ng; ++e)
      CUDA_TRY(cudaGraphLaunch(ctx->beng[e].loop[ORION_BATCH_POOLED].exec, engine_stream(ctx, e)));
    for (int e = 1; e < ng; ++e) {
      CUDA_TRY(cudaEventRecord(ctx->ev_join[e - 1], engine_stream(ctx, e)));
      CUDA_TRY(cudaStreamWaitEvent(s, ctx->ev_join[e - 1], 0));
    }
    CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  }
  std::vector<BatchCtl> outs(ng);
  for (int e = 0; e < ng; ++e)
    CUDA_TRY(cudaMemcpyAsync(&outs[e], bvs[e].ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_out = ms;
  BatchCtl& out = *out_ctl;
  out = outs[0];
  int64_t launches = 0;
  int error_bits = 0;
  for (int e = 0; e < ng; ++e) {
    const BatchCtl& o = outs[e];
    if (e > 0) {
      out.paths_done += o.paths_done;
      for (int k = 0; k < 3; ++k) out.rays[k] += o.rays[k];
      out.iterations = std::max(out.iterations, o.iterations);
    }
    error_bits |= o.error;
    // Per iteration: plan, regen, 4 traces, one shade per class, resolve, retire, control; plus the init.
    const unsigned launched = ctx->profiling ? masks[e] : ctx->beng[e].loop[ORION_BATCH_POOLED].mask;
    launches += (9LL + __builtin_popcount(launched)) * o.iterations + 1;
  }
  out.error = error_bits;
  ctx->last.paths = (int64_t)out.paths_done;
  ctx->last.ext_rays = (int64_t)out.rays[0];
  ctx->last.shadow_rays = (int64_t)out.rays[1];
  ctx->last.mis_rays = (int64_t)out.rays[2];
  ctx->last.rays = (int64_t)(out.rays[0] + out.rays[1] + out.rays[2]);
  ctx->last.kernel_launches = launches;
  ctx->last.device_ms = ms;
  if (out.error) return fail(ORION_ERR_DEVICE, batch_error(out.error));
  if (out.paths_done != total)
    return fail(ORION_ERR_DEVICE, "batch finished " + std::to_string(out.paths_done) + " of " + std::to_string(total) +
                                      " paths");
  return ORION_OK;
}

// Wave mode: the concatenated work list in waves of up to `wave_paths`
// paths, consecutive waves on the engines in turn (concurrently, one stream
// each). Films take FP64 atomics, so waves may finish in any order.
static int run_batch_waves_locked(orion_gpu_ctx* ctx, std::vector<DevJob>& dj, unsigned long long total,
                                  int max_depth_all, BatchCtl* out_ctl, float* ms_out) {
  const int njobs = (int)dj.size();
  int rc;
  const int64_t wave = std::max<int64_t>(1024, std::min<int64_t>(ctx->default_batch_slots, (int64_t)total));
  const int64_t nwaves = std::max<int64_t>(1, ((int64_t)total + wave - 1) / wave);
  const int ne = ctx->profiling ? 1 : (int)std::min<int64_t>(std::min(ctx->batch_engines, (int)orion_gpu_ctx::kBatchEngines),
                                                            nwaves);
  std::vector<BatchView> bvs(ne);
  std::vector<int> caps(ne);
  unsigned mask = 1u << SC_MISS;
  for (const DevJob& J : dj) mask |= J.scene.class_mask;
  for (int e = 0; e < ne; ++e) {
    if ((rc = prepare_engine(ctx, e, njobs, (int)wave, &bvs[e], &caps[e])) != ORION_OK) return rc;
    if (!ctx->profiling && (rc = build_batch_graph(ctx, e, ORION_BATCH_WAVES, bvs[e], caps[e], mask)) != ORION_OK)
      return rc;
  }
  cudaStream_t s = ctx->stream;
  std::memset(&ctx->stage_times, 0, sizeof(ctx->stage_times));
  CUDA_TRY(cudaEventRecord(ctx->ev0, s));
  if (ne > 1) {
    CUDA_TRY(cudaEventRecord(ctx->ev_fork, s));
    for (int e = 1; e < ne; ++e) CUDA_TRY(cudaStreamWaitEvent(engine_stream(ctx, e), ctx->ev_fork, 0));
  }
  BatchCtl zero;
  std::memset(&zero, 0, sizeof(zero));
  zero.njobs = njobs;
  for (int e = 0; e < ne; ++e) {
    cudaStream_t es = engine_stream(ctx, e);
    CUDA_TRY(cudaMemcpyAsync(bvs[e].jobs, dj.data(), (size_t)njobs * sizeof(DevJob), cudaMemcpyHostToDevice, es));
    CUDA_TRY(cudaMemcpyAsync(bvs[e].ctl, &zero, sizeof(BatchCtl), cudaMemcpyHostToDevice, es));
    // The queue-compaction bytes start clear (other entry points share the slots' memory).
    CUDA_TRY(cudaMemsetAsync(engine_wave(ctx, e).view.qflags, 0, (size_t)caps[e], es));
  }
  // Every live path advances one bounce per iteration: a bound on each wave's loop.
  const int iteration_cap =
      ctx->cfg.test_batch_iterations > 0 ? ctx->cfg.test_batch_iterations : 2 * (max_depth_all + 2) + 8;
  StageTimer timer{nullptr, nullptr, 0, 0};
  if (ctx->profiling) {
    const int need = (int)std::min<int64_t>(nwaves * iteration_cap * 10, 200000);
    while ((int)ctx->prof_events.size() < 2 * need) {
      cudaEvent_t e;
      CUDA_TRY(cudaEventCreate(&e));
      ctx->prof_events.push_back(e);
    }
    ctx->prof_stage.resize(need);
    timer = StageTimer{ctx->prof_events.data(), ctx->prof_stage.data(), need, 0};
  }
  for (int64_t k = 0; k < nwaves; ++k) {
    const int e = (int)(k % ne);
    cudaStream_t es = engine_stream(ctx, e);
    const WaveView& wv = engine_wave(ctx, e).view;
    const unsigned long long base = (unsigned long long)(k * wave);
    const int n = (int)std::min<unsigned long long>((unsigned long long)wave, total - base);
    if (ctx->profiling) timer.begin(ST_CAMERA, es);
    launch_batch_wave_begin(wv, bvs[e], ctx->sobol.as<uint32_t>(), base, n, iteration_cap, ctx->num_sms, es);
    if (ctx->profiling) timer.end(es);
    if (ctx->profiling) {
      int more = 1;
      for (int it = 0; more && it < iteration_cap; ++it) {
        launch_batch_iteration(wv, bvs[e], ctx->sobol.as<uint32_t>(), ctx->cfg, mask, true, es, &timer);
        CUDA_TRY(cudaGetLastError());
        CUDA_TRY(cudaMemcpyAsync(&more, &bvs[e].ctl->more, sizeof(int), cudaMemcpyDeviceToHost, es));
        CUDA_TRY(cudaStreamSynchronize(es));
      }
    } else {
      CUDA_TRY(cudaGraphLaunch(ctx->beng[e].loop[ORION_BATCH_WAVES].exec, es));
    }
    if (ctx->profiling) timer.begin(ST_FILM, es);
    launch_batch_wave_film(wv, bvs[e], n, ctx->num_sms, es);
    if (ctx->profiling) timer.end(es);
    CUDA_TRY(cudaGetLastError());
  }
  for (int e = 1; e < ne; ++e) {
    CUDA_TRY(cudaEventRecord(ctx->ev_join[e - 1], engine_stream(ctx, e)));
    CUDA_TRY(cudaStreamWaitEvent(s, ctx->ev_join[e - 1], 0));
  }
  CUDA_TRY(cudaEventRecord(ctx->ev1, s));
  std::vector<BatchCtl> outs(ne);
  for (int e = 0; e < ne; ++e)
    CUDA_TRY(cudaMemcpyAsync(&outs[e], bvs[e].ctl, sizeof(BatchCtl), cudaMemcpyDeviceToHost, s));
  CUDA_TRY(cudaStreamSynchronize(s));
  float ms = 0.f;
  CUDA_TRY(cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1));
  *ms_out = ms;
  for (int i = 0; i < std::min(timer.used, timer.capacity); ++i) {
    float e = 0.f;
    CUDA_TRY(cudaEventElapsedTime(&e, timer.events[2 * i], timer.events[2 * i + 1]));
    ctx->stage_times.ms[timer.stage[i]] += e;
    ctx->stage_times.launches[timer.stage[i]] += 1;
  }
  BatchCtl& out = *out_ctl;
  out = outs[0];
  int64_t launches = 0;
  int error_bits = 0;
  for (int e = 0; e < ne; ++e) {
    const BatchCtl& o = outs[e];
    if (e > 0) {
      out.paths_done += o.paths_done;
      for (int j = 0; j < 3; ++j) out.rays[j] += o.rays[j];
      out.iterations += o.iterations;
    }
    error_bits |= o.error;
    // Per iteration: plan, 4 traces, 2 queue compactions, one shade per class, resolve, control.
    const unsigned launched = ctx->profiling ? mask : ctx->beng[e].loop[ORION_BATCH_WAVES].mask;
    launches += (9LL + __builtin_popcount(launched)) * o.iterations;
  }
  launches += 3 * nwaves;  // begin, camera, film per wave
  out.error = error_bits;
  ctx->last.paths = (int64_t)out.paths_done;
  ctx->last.ext_rays = (int64_t)out.rays[0];
  ctx->last.shadow_rays = (int64_t)out.rays[1];
  ctx->last.mis_rays = (int64_t)out.rays[2];
  ctx->last.rays = (int64_t)(out.rays[0] + out.rays[1] + out.rays[2]);
  ctx->last.kernel_launches = launches;
  ctx->last.device_ms = ms;
  if (out.error) return fail(ORION_ERR_DEVICE, batch_error(out.error));
  if (out.paths_done != total)
    return fail(ORION_ERR_DEVICE, "batch finished " + std::to_string(out.paths_done) + " of " + std::to_string(total) +
                                      " paths");
  return ORION_OK;
}

static int run_batch_locked(orion_gpu_ctx* ctx, std::vector<DevJob>& dj, unsigned long long total, int max_depth_all,
                            BatchCtl* out_ctl, float* ms_out) {
  return ctx->batch_mode == ORION_BATCH_WAVES ? run_batch_waves_locked(ctx, dj, total, max_depth_all, out_ctl, ms_out)
                                              : run_batch_pooled_locked(ctx, dj, total, max_depth_all, out_ctl, ms_out);
}

// Job table and film layout of a batch (films packed into one device block).
static int plan_batch(orion_gpu_ctx* ctx, int32_t njobs, const orion_job* jobs, int spp_cap, std::vector<DevJob>& dj,
                      std::vector<size_t>& film_off, size_t* film_bytes_out, unsigned long long* total_out,
                      int* max_depth_out) {
  dj.assign(njobs, DevJob{});
  film_off.assign(njobs, 0);
  size_t film_bytes = 0;
  unsigned long long total = 0;
  int max_depth_all = 0;
  for (int i = 0; i < njobs; ++i) {
    auto it = ctx->scenes.find(jobs[i].scene);
    if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "job " + std::to_string(i) + ": unknown scene id");
    const DeviceScene& d = *it->second;
    const orion_render_params& p = jobs[i].params;
    DevJob& J = dj[i];
    std::memset(&J, 0, sizeof(J));
    J.scene = d.view;
    if (jobs[i].camera) {
      if (jobs[i].camera->width <= 0 || jobs[i].camera->height <= 0)
        return fail(ORION_ERR_INVALID, "job " + std::to_string(i) + ": film size must be positive");
      J.scene.cam = prepare_camera(*jobs[i].camera);
    }
    J.width = J.scene.cam.width;
    J.height = J.scene.cam.height;
    int spp = p.spp > 0 ? p.spp : d.spp;
    if (spp_cap > 0) spp = std::min(spp, spp_cap);
    J.max_depth = p.max_depth >= 0 ? p.max_depth : d.max_depth;
    J.rr_depth = p.rr_depth;
    if (J.max_depth > 120 || 17 + 8 * (int64_t)J.max_depth > 1024)
      return fail(ORION_ERR_INVALID, "job " + std::to_string(i) + ": max_depth out of range");
    const long long wh = (long long)J.width * J.height;
    J.first_index = p.first_pass * wh;
    J.num_paths = wh * spp;
    J.work_begin = (long long)total;
    total += (unsigned long long)J.num_paths;
    max_depth_all = std::max(max_depth_all, J.max_depth);
    film_off[i] = film_bytes;
    film_bytes += (size_t)((wh * (3 * 8 * 2 + 4) + 255) & ~255LL);
  }
  *film_bytes_out = film_bytes;
  *total_out = total;
  *max_depth_out = max_depth_all;
  return ORION_OK;
}

extern "C" int orion_gpu_render_batch(orion_gpu_ctx* ctx, int32_t njobs, const orion_job* jobs,
                                      orion_batch_stats* stats) {
  if (!ctx || njobs < 0 || (njobs > 0 && !jobs)) return fail(ORION_ERR_INVALID, "bad argument");
  NvtxRange range("orion_gpu_render_batch");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  if (njobs == 0) {
    if (stats) std::memset(stats, 0, sizeof(*stats));
    return ORION_OK;
  }
  std::vector<DevJob> dj;
  std::vector<size_t> film_off;
  size_t film_bytes = 0;
  unsigned long long total = 0;
  int max_depth_all = 0;
  RC(plan_batch(ctx, njobs, jobs, 0, dj, film_off, &film_bytes, &total, &max_depth_all));
  int rc;
  if (ctx->b_films.bytes < film_bytes && (rc = ctx->b_films.alloc(film_bytes)) != ORION_OK) return rc;
  char* fb = ctx->b_films.as<char>();
  for (int i = 0; i < njobs; ++i) {
    const long long wh = (long long)dj[i].width * dj[i].height;
    dj[i].sum = reinterpret_cast<double*>(fb + film_off[i]);
    // Every pixel of a finished job has exactly its spp samples, so counts are
    // written on the host, not counted on the device (one atomic per path less).
    dj[i].count = nullptr;
    // Sums of squares only for callers that want them (they cost 3 FP64 atomics per path).
    dj[i].sumsq = jobs[i].sumsq ? dj[i].sum + 3 * wh : nullptr;
  }
  cudaStream_t s = ctx->stream;
  CUDA_TRY(cudaMemsetAsync(ctx->b_films.p, 0, film_bytes, s));
  BatchCtl out;
  float ms = 0.f;
  rc = run_batch_locked(ctx, dj, total, max_depth_all, &out, &ms);
  if (rc != ORION_OK) return rc;
  // FP32 read-back: every requested film rounded on the device into one
  // staging block, then one copy per film.
  size_t f32_bytes = 0;
  for (int i = 0; i < njobs; ++i)
    if (jobs[i].sum32) f32_bytes += (size_t)dj[i].width * dj[i].height * 12;
  if (f32_bytes && ctx->b_films32.bytes < f32_bytes && (rc = ctx->b_films32.alloc(f32_bytes)) != ORION_OK) return rc;
  size_t f32_off = 0;
  for (int i = 0; i < njobs; ++i) {
    const size_t wh = (size_t)dj[i].width * dj[i].height;
    if (jobs[i].sum) CUDA_TRY(cudaMemcpyAsync(jobs[i].sum, dj[i].sum, wh * 24, cudaMemcpyDeviceToHost, s));
    if (jobs[i].sumsq) CUDA_TRY(cudaMemcpyAsync(jobs[i].sumsq, dj[i].sumsq, wh * 24, cudaMemcpyDeviceToHost, s));
    if (jobs[i].sum32) {
      float* dst = reinterpret_cast<float*>(ctx->b_films32.as<char>() + f32_off);
      launch_film_to_f32(dj[i].sum, dst, (long long)wh * 3, ctx->num_sms, s);
      CUDA_TRY(cudaGetLastError());
      CUDA_TRY(cudaMemcpyAsync(jobs[i].sum32, dst, wh * 12, cudaMemcpyDeviceToHost, s));
      f32_off += wh * 12;
    }
  }
  for (int i = 0; i < njobs; ++i)
    if (jobs[i].count) {
      const size_t wh = (size_t)dj[i].width * dj[i].height;
      std::fill(jobs[i].count, jobs[i].count + wh, (uint32_t)(dj[i].num_paths / (long long)wh));
    }
  CUDA_TRY(cudaStreamSynchronize(s));
  if (stats) {
    stats->paths = (int64_t)out.paths_done;
    stats->rays = (int64_t)(out.rays[0] + out.rays[1] + out.rays[2]);
    stats->iterations = out.iterations;
    stats->capacity = ctx->wave.capacity;
    stats->device_ms = ms;
  }
  return ORION_OK;
}

extern "C" int orion_gpu_set_batch_mode(orion_gpu_ctx* ctx, int32_t mode) {
  if (!ctx) return fail(ORION_ERR_INVALID, "null context");
  if (mode != ORION_BATCH_POOLED && mode != ORION_BATCH_WAVES) return fail(ORION_ERR_INVALID, "unknown batch mode");
  std::lock_guard<std::mutex> g(ctx->mu);
  ctx->batch_mode = mode;
  return ORION_OK;
}

extern "C" int orion_gpu_autotune_batch(orion_gpu_ctx* ctx, int32_t njobs, const orion_job* jobs, int32_t spp_cap,
                                        double budget_ms, orion_launch_config* best_out, double* best_mpaths) {
  if (!ctx || njobs <= 0 || !jobs) return fail(ORION_ERR_INVALID, "bad argument");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  std::vector<DevJob> dj;
  std::vector<size_t> film_off;
  size_t film_bytes = 0;
  unsigned long long total = 0;
  int max_depth_all = 0;
  RC(plan_batch(ctx, njobs, jobs, spp_cap, dj, film_off, &film_bytes, &total, &max_depth_all));
  DevBuf films;  // trial films: accumulated into and discarded
  RC(films.alloc(film_bytes));
  char* fb = films.as<char>();
  for (int i = 0; i < njobs; ++i) {
    const long long wh = (long long)dj[i].width * dj[i].height;
    dj[i].sum = reinterpret_cast<double*>(fb + film_off[i]);
    dj[i].sumsq = dj[i].sum + 3 * wh;
    dj[i].count = reinterpret_cast<unsigned int*>(dj[i].sumsq + 3 * wh);
  }
  CUDA_TRY(cudaMemsetAsync(films.p, 0, film_bytes, ctx->stream));
  // batch_slots is the pool size (pooled mode) or the wave size (wave mode).
  LaunchConfig best = ctx->cfg;
  int best_slots = ctx->default_batch_slots;
  int best_streams = ctx->batch_engines, best_mode = ctx->batch_mode;
  double best_ms = 1e30, used = 0;
  auto trial = [&](const LaunchConfig& c, int slots, int streams, int mode, double* ms) -> int {
    LaunchConfig saved = ctx->cfg;
    int saved_slots = ctx->default_batch_slots, saved_streams = ctx->batch_engines;
    int saved_mode = ctx->batch_mode;
    ctx->cfg = c;
    ctx->default_batch_slots = slots;
    ctx->batch_engines = streams;
    ctx->batch_mode = mode;
    BatchCtl out;
    float fms = 0.f;
    int rc = run_batch_locked(ctx, dj, total, max_depth_all, &out, &fms);
    ctx->cfg = saved;
    ctx->default_batch_slots = saved_slots;
    ctx->batch_engines = saved_streams;
    ctx->batch_mode = saved_mode;
    *ms = fms;
    used += fms;
    return rc;
  };
  double ms;
  RC(trial(best, best_slots, best_streams, best_mode, &ms));  // warm-up (graph instantiation)
  RC(trial(best, best_slots, best_streams, best_mode, &best_ms));
  const int trace_blocks[] = {64, 128, 256};
  const int stacks[] = {8, 16, 32};
  const int shade_blocks[] = {64, 128, 256};
  const int bpsm[] = {4, 6, 8, 12};
  const int slot_counts[] = {1 << 22, 1 << 23, 1 << 24, 1 << 25};
  const int refills[] = {8, 16, 24, 32};
  const int engine_counts[] = {1, 2};
  const int modes[] = {ORION_BATCH_POOLED, ORION_BATCH_WAVES};
  for (int knob = 0; knob < 8 && used < budget_ms; ++knob) {
    const int n = knob >= 6 ? 2 : (knob >= 3 ? 4 : 3);
    for (int v = 0; v < n && used < budget_ms; ++v) {
      LaunchConfig c = best;
      int slots = best_slots, streams = best_streams, mode = best_mode;
      if (knob == 0) c.trace_block = trace_blocks[v];
      if (knob == 1) c.smem_stack = stacks[v];
      if (knob == 2) c.shade_block = shade_blocks[v];
      if (knob == 3) c.blocks_per_sm = bpsm[v];
      if (knob == 4) slots = slot_counts[v];
      if (knob == 5) c.refill_below = refills[v];
      if (knob == 6) streams = engine_counts[v];
      if (knob == 7) mode = modes[v];
      if (std::memcmp(&c, &best, sizeof(c)) == 0 && slots == best_slots && streams == best_streams &&
          mode == best_mode)
        continue;
      if (!config_problem(ctx, c).empty()) continue;
      int rc = trial(c, slots, streams, mode, &ms);
      if (rc == ORION_ERR_NOMEM) continue;
      if (rc != ORION_OK) return rc;
      if (ms < best_ms) {
        best_ms = ms;
        best = c;
        best_slots = slots;
        best_streams = streams;
        best_mode = mode;
      }
    }
  }
  ctx->cfg = best;
  ctx->default_batch_slots = best_slots;
  ctx->batch_engines = best_streams;
  ctx->batch_mode = best_mode;
  if (best_out) {
    best_out->trace_block = best.trace_block;
    best_out->shade_block = best.shade_block;
    best_out->smem_stack = best.smem_stack;
    best_out->blocks_per_sm = best.blocks_per_sm;
    best_out->wave_paths = ctx->default_wave;
    best_out->batch_slots = best_slots;
    best_out->refill_below = best.refill_below;
    best_out->streams = ctx->batch_engines;
  }
  if (best_mpaths) *best_mpaths = (double)total / (best_ms * 1e-3) / 1e6;
  return ORION_OK;
}

// ------------------------------------------------------ internal hooks

namespace orion_gb300 {

int ctx_run_device_jobs(orion_gpu_ctx* ctx, const DeviceFilmJob* jobs, int njobs, double* device_ms,
                        int64_t* paths) {
  NvtxRange range("orion_server launch");
  std::lock_guard<std::mutex> g(ctx->mu);
  CUDA_TRY(cudaSetDevice(ctx->device));
  std::vector<DevJob> dj(njobs);
  unsigned long long total = 0;
  int max_depth_all = 0;
  for (int i = 0; i < njobs; ++i) {
    auto it = ctx->scenes.find(jobs[i].scene);
    if (it == ctx->scenes.end()) return fail(ORION_ERR_INVALID, "unknown scene id");
    const DeviceScene& d = *it->second;
    const orion_render_params& p = jobs[i].params;
    DevJob& J = dj[i];
    std::memset(&J, 0, sizeof(J));
    J.scene = d.view;
    if (jobs[i].camera) J.scene.cam = prepare_camera(*jobs[i].camera);
    J.width = J.scene.cam.width;
    J.height = J.scene.cam.height;
    const int spp = p.spp > 0 ? p.spp : d.spp;
    J.max_depth = p.max_depth >= 0 ? p.max_depth : d.max_depth;
    J.rr_depth = p.rr_depth;
    if (J.max_depth > 120) return fail(ORION_ERR_INVALID, "max_depth out of range");
    const long long wh = (long long)J.width * J.height;
    J.first_index = p.first_pass * wh;
    J.num_paths = wh * spp;
    J.work_begin = (long long)total;
    total += (unsigned long long)J.num_paths;
    max_depth_all = std::max(max_depth_all, J.max_depth);
    J.sum = jobs[i].sum;
    J.sumsq = jobs[i].sumsq;
    J.count = jobs[i].count;
  }
  BatchCtl out;
  float ms = 0.f;
  int rc = run_batch_locked(ctx, dj, total, max_depth_all, &out, &ms);
  if (device_ms) *device_ms = ms;
  if (paths) *paths = (int64_t)out.paths_done;
  return rc;
}

}  // namespace orion_gb300
