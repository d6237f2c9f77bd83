// Batched wavefront path tracing: many render jobs per device-side loop.
//
// The jobs' sample ranges are concatenated into one work list. One
// iteration of the device-side loop
//
//   k_b_plan     take = min(free slots, work left); reset this iteration's queues
//   k_b_regen    pooled mode: start `take` new camera paths in free slots
//   k_b_trace    closest hit for every live path (each against its job's scene)
//   k_b_shade    one bounce of PathTracing::Li per path (shared shade_one)
//   k_b_trace    shadow rays (any hit) and MIS rays (closest hit)
//   k_b_resolve  direct-light estimate into the path radiance
//   k_b_retire   pooled mode: finished paths' radiance into the job's FP64
//                film, slot freed
//   k_b_control  flip queues; keep looping while work or live paths remain
//
// runs inside a CUDA graph while-node. Pooled mode shares one pool of path
// slots among all jobs and refills finished slots every iteration. Wave mode
// starts a wave of contiguous work items on slots 0..n-1
// (k_b_wave_begin / k_b_wave_camera), loops until none is alive and writes
// the film once (k_b_wave_film). Paths of different jobs, depths and bounces
// share every launch. Each path runs the plain path's device functions on
// the same samples; the film's order of accumulation differs (FP64 atomics).
#include <cuda_runtime.h>

#include "kernels.h"
#include "shade.cuh"

namespace orion_gb300 {

namespace {

__global__ void k_b_init(BatchView b, int capacity) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < capacity; i += gridDim.x * blockDim.x) b.q_free[i] = i;
}

__global__ void k_b_plan(BatchView b) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  BatchCtl& c = *b.ctl;
  unsigned long long rem = c.total - c.cursor;
  int nfree = c.counters[CNT_FREE];
  int take = (unsigned long long)nfree < rem ? nfree : (int)rem;
  c.take = take;
  c.take_base = c.cursor;
  c.cursor += (unsigned long long)take;
  c.counters[CNT_FREE] = nfree - take;
  c.counters[CNT_NEE] = 0;
  c.counters[CNT_SH] = 0;
  c.counters[CNT_MIS] = 0;
  c.counters[CNT_RETIRE] = 0;
  c.counters[CNT_EXT0 + (c.cur ^ 1)] = 0;
  c.counters[CNT_FETCH_EXT] = 0;
  c.counters[CNT_FETCH_SH] = 0;
  c.counters[CNT_FETCH_MIS] = 0;
  c.counters[CNT_MIS_ENV] = 0;
  c.counters[CNT_FETCH_MIS_ENV] = 0;
  for (int k = 0; k < kShadeClasses; ++k) c.counters[CNT_CLS0 + k] = 0;
}

__device__ __forceinline__ int job_of_work(const DevJob* jobs, int njobs, unsigned long long work) {
  int lo = 0, hi = njobs - 1;
  while (lo < hi) {  // last job with work_begin <= work
    int mid = (lo + hi + 1) >> 1;
    if ((unsigned long long)jobs[mid].work_begin <= work)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

__global__ void k_b_regen(WaveView w, BatchView b, const uint32_t* sobol) {
  BatchCtl& c = *b.ctl;
  const int take = c.take;
  const int free_after = c.counters[CNT_FREE];
  const int cur = c.cur;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < take; i += gridDim.x * blockDim.x) {
    const int slot = b.q_free[free_after + i];
    const unsigned long long work = c.take_base + (unsigned long long)i;
    const int job = job_of_work(b.jobs, c.njobs, work);
    const DevJob& J = b.jobs[job];
    const long long index = J.first_index + (long long)(work - (unsigned long long)J.work_begin);
    const long long wh = (long long)J.width * J.height;
    const long long pix = index % wh;
    PathSampler smp{sobol, (uint64_t)index, 5u};
    V3 o, d;
    camera_ray(J.scene.cam, smp, (int)(pix % J.width), (int)(pix / J.width), &o, &d);
    // The whole 96-byte record in one go: three full sectors at a scattered slot.
    PathRec r;
    r.o = f4(o, 0.f);
    r.d = f4(d, 0.f);
    r.beta = make_float4(1.f, 1.f, 1.f, 0.f);
    r.L = make_float4(0.f, 0.f, 0.f, __uint_as_float((uint32_t)(unsigned long long)index));
    r.hit = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    r.meta = make_int4((int)smp.dim, job, 0, (int)((unsigned long long)index >> 32));
    w.rec[slot] = r;
    queue_append(&c.counters[CNT_EXT0 + cur], w.q_ext[cur], slot, true);
  }
}

// kind 0: extension rays (current queue), 1: shadow rays, 2: MIS rays towards
// area lights, 3: MIS rays towards environment lights (occlusion).
// cls_flags (wave mode): extension hits mark their slot's shading class there
// for k_b_compact instead of appending to the class queues.
template <int SMEM>
__global__ void __launch_bounds__(512, 2) k_b_trace(WaveView w, BatchView b, int kind, int refill_below,
                                                     uint8_t* cls_flags) {
  extern __shared__ int2 stack_smem[];
  BatchCtl& c = *b.ctl;
  JobScene js{b.jobs, w.job};
  int n;
  if (kind == 0) {
    n = c.counters[CNT_EXT0 + c.cur];
    trace_persistent<false, SMEM>(js, w.q_ext[c.cur], n, &c.counters[CNT_FETCH_EXT], w.ray_o, w.ray_d, w.hit,
                                  nullptr, stack_smem, refill_below, &c.error, &c.counters[CNT_CLS0], w.q_cls,
                                  w.capacity, nullptr, cls_flags);
  } else if (kind == 1) {
    n = c.counters[CNT_SH];
    trace_persistent<true, SMEM>(js, w.q_sh, n, &c.counters[CNT_FETCH_SH], w.sh_o, w.sh_d,
                                 F4{nullptr}, w.occluded, stack_smem, refill_below, &c.error);
  } else if (kind == 2) {
    n = c.counters[CNT_MIS];
    trace_persistent<false, SMEM>(js, w.q_mis, n, &c.counters[CNT_FETCH_MIS], w.mis_o, w.mis_d,
                                  F4{w.mis_hit}, nullptr, stack_smem, refill_below, &c.error);
  } else {  // 3: MIS rays towards environment lights, occlusion only
    n = c.counters[CNT_MIS_ENV];
    trace_persistent<true, SMEM>(js, w.q_mis_env, n, &c.counters[CNT_FETCH_MIS_ENV], w.mis_o, w.mis_d,
                                 F4{nullptr}, w.mis_occluded, stack_smem, refill_below, &c.error);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c.rays[kind < 3 ? kind : 2], (unsigned long long)n);
}

// Shading of the slots whose extension ray hit a material of class SC (or
// missed, SC_MISS), each against its job's scene.
// waves: a wave's paths are never retired one by one, and the queues they go
// to are marked in the slots' qflags bytes for k_b_compact (slot order, as in
// plain renders); pooled mode appends to the queues directly.
template <int SC>
__global__ void __launch_bounds__(128, 5) k_b_shade(WaveView w, BatchView b, const uint32_t* sobol,
                                                    int waves) {
  BatchCtl& c = *b.ctl;
  const int cur = c.cur;
  const int n = c.counters[CNT_CLS0 + SC];
  const int* in_q = w.q_cls + (size_t)SC * w.capacity;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = in_q[q];
    const int4 meta = w.rec[pid].meta;
    const DevJob& J = b.jobs[meta.y];
    const int bounce = meta.z;
    ShadeResult r = shade_one<lobes_of_class(SC), SC == SC_TEXTURED>(
        J.scene, w, sobol, pid, (uint64_t)slot_index(w, pid), bounce, J.max_depth, J.rr_depth);
    if (r.alive) w.bounce[pid] = bounce + 1;
    if (waves) {
      w.qflags[pid] = (uint8_t)((r.alive ? kQfExt : 0) | (r.did_nee ? kQfNee : 0) | (r.want_sh ? kQfShadow : 0) |
                                (r.want_mis ? kQfMis : 0) | (r.want_mis_env ? kQfMisEnv : 0));
      continue;
    }
    queue_append(&c.counters[CNT_NEE], w.q_nee, pid, r.did_nee);
    queue_append(&c.counters[CNT_SH], w.q_sh, pid, r.want_sh);
    queue_append(&c.counters[CNT_MIS], w.q_mis, pid, r.want_mis);
    queue_append(&c.counters[CNT_MIS_ENV], w.q_mis_env, pid, r.want_mis_env);
    queue_append(&c.counters[CNT_EXT0 + (cur ^ 1)], w.q_ext[cur ^ 1], pid, r.alive);
    queue_append(&c.counters[CNT_RETIRE], b.q_retire, pid, !r.alive);
  }
}

// Wave mode: the slots' qflags bytes into queues in slot order (plain
// renders' compaction, compact_queues). which 0: shading classes, after the
// extension trace; 1: the queues the shading sent paths to (next extension
// queue by the current parity, which only the device knows inside a graph).
__global__ void __launch_bounds__(kCompactThreads) k_b_compact(WaveView w, BatchView b, int which) {
  BatchCtl& c = *b.ctl;
  const int cur = c.cur;
  CompactTargets tg{};
  if (which == 0) {
    for (int k = 0; k < kShadeClasses; ++k) {
      tg.queue[k] = w.q_cls + (size_t)k * w.capacity;
      tg.counter[k] = &c.counters[CNT_CLS0 + k];
    }
    compact_queues<kShadeClasses>(w.qflags, w.q_ext[cur], &c.counters[CNT_EXT0 + cur], tg);
  } else {
    const int next = cur ^ 1;
    int* qs[5] = {w.q_ext[next], w.q_nee, w.q_sh, w.q_mis, w.q_mis_env};
    int* cs[5] = {&c.counters[CNT_EXT0 + next], &c.counters[CNT_NEE], &c.counters[CNT_SH], &c.counters[CNT_MIS],
                  &c.counters[CNT_MIS_ENV]};
    for (int k = 0; k < 5; ++k) tg.queue[k] = qs[k], tg.counter[k] = cs[k];
    compact_queues<5>(w.qflags, w.q_ext[cur], &c.counters[CNT_EXT0 + cur], tg);
  }
}

__global__ void k_b_resolve(WaveView w, BatchView b) {
  const int n = b.ctl->counters[CNT_NEE];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = w.q_nee[q];
    resolve_one(b.jobs[w.job[pid]].scene, w, pid);
  }
}

__global__ void k_b_retire(WaveView w, BatchView b) {
  BatchCtl& c = *b.ctl;
  const int n = c.counters[CNT_RETIRE];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = b.q_retire[q];
    const float4 l = w.L[pid];
    const int4 meta = w.rec[pid].meta;
    const DevJob& J = b.jobs[meta.y];
    const long long index =
        (long long)(((unsigned long long)(unsigned)meta.w << 32) | (unsigned long long)__float_as_uint(l.w));
    const long long pix = index % ((long long)J.width * J.height);
    atomicAdd(&J.sum[3 * pix], (double)l.x);
    atomicAdd(&J.sum[3 * pix + 1], (double)l.y);
    atomicAdd(&J.sum[3 * pix + 2], (double)l.z);
    if (J.sumsq) {
      atomicAdd(&J.sumsq[3 * pix], (double)l.x * l.x);
      atomicAdd(&J.sumsq[3 * pix + 1], (double)l.y * l.y);
      atomicAdd(&J.sumsq[3 * pix + 2], (double)l.z * l.z);
    }
    if (J.count) atomicAdd(&J.count[pix], 1u);  // null: the caller knows every pixel gets spp samples
    queue_append(&c.counters[CNT_FREE], b.q_free, pid, true);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&c.paths_done, (unsigned long long)n);
}

// ------------------------------------------------------------ wave mode
//
// A batch can also run as waves over its concatenated work list: wave k
// takes work items [base, base + n) onto slots 0..n-1 in order, its paths
// bounce until none is alive (no refills), and the radiance of all n paths
// goes to the jobs' films at the end, slot after slot, so neighbouring slots
// add to neighbouring pixels of one job.

// Resets the per-wave control fields (rays, paths and iterations stay
// cumulative over the batch's waves).
__global__ void k_b_wave_begin(BatchView b, int n, int iteration_cap) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  BatchCtl& c = *b.ctl;
  c.cursor = c.total = c.take_base = 0ULL;
  c.take = 0;
  c.cur = 0;
  for (int k = 0; k < kCounterSlots; ++k) c.counters[k] = 0;
  c.counters[CNT_EXT0] = n;
  c.max_iterations = c.iterations + iteration_cap;
  c.more = 1;
}

__global__ void k_b_wave_camera(WaveView w, BatchView b, const uint32_t* sobol, unsigned long long base, int n) {
  const int njobs = b.ctl->njobs;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned long long work = base + (unsigned long long)i;
    const int job = job_of_work(b.jobs, njobs, work);
    const DevJob& J = b.jobs[job];
    const long long index = J.first_index + (long long)(work - (unsigned long long)J.work_begin);
    const long long wh = (long long)J.width * J.height;
    const long long pix = index % wh;
    V3 o, d;
    const uint32_t dim = camera_ray_block(J.scene.cam, sobol, (uint64_t)index, (int)(pix % J.width),
                                          (int)(pix / J.width), &o, &d);
    PathRec r;
    r.o = f4(o, 0.f);
    r.d = f4(d, 0.f);
    r.beta = make_float4(1.f, 1.f, 1.f, 0.f);
    r.L = make_float4(0.f, 0.f, 0.f, __uint_as_float((uint32_t)(unsigned long long)index));
    r.hit = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    r.meta = make_int4((int)dim, job, 0, (int)((unsigned long long)index >> 32));
    w.rec[i] = r;
    w.q_ext[0][i] = i;
    w.qflags[i] = 0;
  }
}

__global__ void k_b_wave_film(WaveView w, BatchView b, int n) {
  for (int pid = blockIdx.x * blockDim.x + threadIdx.x; pid < n; pid += gridDim.x * blockDim.x) {
    const float4 l = w.L[pid];
    const int4 meta = w.rec[pid].meta;
    const DevJob& J = b.jobs[meta.y];
    const long long index =
        (long long)(((unsigned long long)(unsigned)meta.w << 32) | (unsigned long long)__float_as_uint(l.w));
    const long long pix = index % ((long long)J.width * J.height);
    atomicAdd(&J.sum[3 * pix], (double)l.x);
    atomicAdd(&J.sum[3 * pix + 1], (double)l.y);
    atomicAdd(&J.sum[3 * pix + 2], (double)l.z);
    if (J.sumsq) {
      atomicAdd(&J.sumsq[3 * pix], (double)l.x * l.x);
      atomicAdd(&J.sumsq[3 * pix + 1], (double)l.y * l.y);
      atomicAdd(&J.sumsq[3 * pix + 2], (double)l.z * l.z);
    }
    if (J.count) atomicAdd(&J.count[pix], 1u);
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(&b.ctl->paths_done, (unsigned long long)n);
}

// in_graph: sets the while-node's condition; otherwise leaves the decision in
// ctl->more for a host-driven loop (profiling runs).
__global__ void k_b_control(BatchView b, cudaGraphConditionalHandle cond, int in_graph) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  BatchCtl& c = *b.ctl;
  c.cur ^= 1;
  c.iterations += 1;
  bool more = c.cursor < c.total || c.counters[CNT_EXT0 + c.cur] > 0;
  if (more && c.iterations >= c.max_iterations) {
    c.error |= kErrIterationCap;  // bounded loop: report instead of spinning on
    more = false;
  }
  if (in_graph)
    cudaGraphSetConditional(cond, more ? 1u : 0u);
  else
    c.more = more ? 1 : 0;
}

template <int SMEM>
void launch_b_trace(const WaveView& w, const BatchView& b, int kind, int grid, int block, int refill,
                    uint8_t* cls_flags, cudaStream_t s) {
  k_b_trace<SMEM><<<grid, block, trace_smem_bytes(SMEM, block), s>>>(w, b, kind, refill, cls_flags);
}

void b_trace(const LaunchConfig& cfg, const WaveView& w, const BatchView& b, int kind, int grid, uint8_t* cls_flags,
             cudaStream_t s) {
  const int block = cfg.trace_block;
  const int refill = cfg.refill_below < 1 ? 1 : (cfg.refill_below > 32 ? 32 : cfg.refill_below);
  switch (cfg.smem_stack) {
    case 0: launch_b_trace<0>(w, b, kind, grid, block, refill, cls_flags, s); break;
    case 8: launch_b_trace<8>(w, b, kind, grid, block, refill, cls_flags, s); break;
    case 24: launch_b_trace<24>(w, b, kind, grid, block, refill, cls_flags, s); break;
    case 32: launch_b_trace<32>(w, b, kind, grid, block, refill, cls_flags, s); break;
    default: launch_b_trace<16>(w, b, kind, grid, block, refill, cls_flags, s); break;
  }
}

cudaError_t batch_limit_of(const void* f, int smem_bytes, int* max_block) {
  if (smem_bytes > 0) {
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
  }
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, f);
  if (e != cudaSuccess) return e;
  *max_block = *max_block < a.maxThreadsPerBlock ? *max_block : a.maxThreadsPerBlock;
  return cudaSuccess;
}

int grid_cap(int64_t n, int block, int cap) {
  int64_t g = (n + block - 1) / block;
  return (int)(g < 1 ? 1 : (g > cap ? cap : g));
}

}  // namespace

cudaError_t configure_batch_kernels(int smem_bytes, KernelLimits* lim) {
  const void* trace[] = {(const void*)k_b_trace<0>, (const void*)k_b_trace<8>, (const void*)k_b_trace<16>,
                         (const void*)k_b_trace<24>, (const void*)k_b_trace<32>};
  const void* shade[] = {(const void*)k_b_shade<SC_DIFFUSE>,    (const void*)k_b_shade<SC_CONDUCTOR>,
                         (const void*)k_b_shade<SC_SPECULAR>,   (const void*)k_b_shade<SC_DIELECTRIC>,
                         (const void*)k_b_shade<SC_PLASTIC>,    (const void*)k_b_shade<SC_GENERAL>,
                         (const void*)k_b_shade<SC_TEXTURED>,
                         (const void*)k_b_shade<SC_MISS>,       (const void*)k_b_resolve,
                         (const void*)k_b_retire};
  for (const void* f : trace) {
    cudaError_t e = batch_limit_of(f, smem_bytes, &lim->max_trace_block);
    if (e != cudaSuccess) return e;
  }
  for (const void* f : shade) {
    cudaError_t e = batch_limit_of(f, 0, &lim->max_shade_block);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void launch_batch_init(const WaveView& w, const BatchView& b, int capacity, cudaStream_t stream) {
  k_b_init<<<grid_cap(capacity, 256, 4096), 256, 0, stream>>>(b, capacity);
}

namespace {

// One loop iteration's kernels on `stream`, optionally timed per stage.
void enqueue_iteration(const WaveView& w, const BatchView& b, const uint32_t* sobol,
                       const LaunchConfig& cfg, unsigned class_mask, bool waves, cudaGraphConditionalHandle cond,
                       int in_graph, cudaStream_t stream, StageTimer* timer) {
  const int cap = w.capacity;
  const int persistent = cfg.num_sms * cfg.blocks_per_sm;
  const int tgrid = grid_cap(cap, cfg.trace_block, persistent);
  const int sgrid = grid_cap(cap, cfg.shade_block, persistent * 2);
  auto begin = [&](int st) {
    if (timer) timer->begin(st, stream);
  };
  auto end = [&]() {
    if (timer) timer->end(stream);
  };
  begin(ST_CAMERA);
  k_b_plan<<<1, 32, 0, stream>>>(b);  // wave mode: counters reset, nothing to take
  if (!waves) k_b_regen<<<grid_cap(cap, 256, persistent * 4), 256, 0, stream>>>(w, b, sobol);
  end();
  const int cgrid = grid_cap(cap, kCompactSpan, cfg.num_sms * 8);
  begin(ST_TRACE_EXT);
  b_trace(cfg, w, b, 0, tgrid, waves ? w.qflags : nullptr, stream);
  end();
  if (waves) {  // the trace marked the slots' shading classes: list them in slot order
    begin(ST_OTHER);
    k_b_compact<<<cgrid, kCompactThreads, 0, stream>>>(w, b, 0);
    end();
  }
  begin(ST_SHADE);
  for (int sc = 0; sc < kShadeClasses; ++sc) {
    if (!((class_mask >> sc) & 1u)) continue;
    switch (sc) {
      case SC_DIFFUSE: k_b_shade<SC_DIFFUSE><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_CONDUCTOR: k_b_shade<SC_CONDUCTOR><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_SPECULAR: k_b_shade<SC_SPECULAR><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_DIELECTRIC: k_b_shade<SC_DIELECTRIC><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_PLASTIC: k_b_shade<SC_PLASTIC><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_GENERAL: k_b_shade<SC_GENERAL><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_TEXTURED: k_b_shade<SC_TEXTURED><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
      case SC_MISS: k_b_shade<SC_MISS><<<sgrid, cfg.shade_block, 0, stream>>>(w, b, sobol, waves); break;
    }
  }
  end();
  if (waves) {  // the shading marked the queues its paths go to
    begin(ST_OTHER);
    k_b_compact<<<cgrid, kCompactThreads, 0, stream>>>(w, b, 1);
    end();
  }
  begin(ST_TRACE_SHADOW);
  b_trace(cfg, w, b, 1, tgrid, nullptr, stream);
  end();
  begin(ST_TRACE_MIS);
  b_trace(cfg, w, b, 2, tgrid, nullptr, stream);
  b_trace(cfg, w, b, 3, tgrid, nullptr, stream);
  end();
  begin(ST_RESOLVE);
  k_b_resolve<<<sgrid, cfg.shade_block, 0, stream>>>(w, b);
  end();
  if (!waves) {  // wave mode: the film is written once the wave is done
    begin(ST_FILM);
    k_b_retire<<<sgrid, cfg.shade_block, 0, stream>>>(w, b);
    end();
  }
  begin(ST_OTHER);
  k_b_control<<<1, 32, 0, stream>>>(b, cond, in_graph);
  end();
}

}  // namespace

cudaError_t capture_batch_iteration(const WaveView& w, const BatchView& b, const uint32_t* sobol,
                                    const LaunchConfig& cfg, unsigned class_mask, bool waves, cudaGraphConditionalHandle cond, cudaStream_t stream,
                                    cudaGraph_t body) {
  cudaError_t e = cudaStreamBeginCaptureToGraph(stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal);
  if (e != cudaSuccess) return e;
  enqueue_iteration(w, b, sobol, cfg, class_mask, waves, cond, 1, stream, nullptr);
  cudaGraph_t out = body;
  cudaError_t e2 = cudaStreamEndCapture(stream, &out);
  cudaError_t e3 = cudaGetLastError();
  return e2 != cudaSuccess ? e2 : e3;
}

void launch_batch_iteration(const WaveView& w, const BatchView& b, const uint32_t* sobol, const LaunchConfig& cfg,
                            unsigned class_mask, bool waves, cudaStream_t stream, StageTimer* timer) {
  enqueue_iteration(w, b, sobol, cfg, class_mask, waves, cudaGraphConditionalHandle{}, 0, stream, timer);
}

void launch_batch_wave_begin(const WaveView& w, const BatchView& b, const uint32_t* sobol,
                             unsigned long long base, int n, int iteration_cap, int num_sms, cudaStream_t stream) {
  k_b_wave_begin<<<1, 32, 0, stream>>>(b, n, iteration_cap);
  k_b_wave_camera<<<grid_cap(n, 256, num_sms * 32), 256, 0, stream>>>(w, b, sobol, base, n);
}

// FP64 film sums rounded to FP32 (orion_job.sum32).
__global__ void k_film_to_f32(const double* __restrict__ src, float* __restrict__ dst, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}

void launch_film_to_f32(const double* src, float* dst, long long n, int num_sms, cudaStream_t stream) {
  const long long blocks = std::min<long long>((n + 255) / 256, (long long)num_sms * 8);
  k_film_to_f32<<<(int)std::max<long long>(blocks, 1), 256, 0, stream>>>(src, dst, n);
}

void launch_batch_wave_film(const WaveView& w, const BatchView& b, int n, int num_sms, cudaStream_t stream) {
  k_b_wave_film<<<grid_cap(n, 256, num_sms * 32), 256, 0, stream>>>(w, b, n);
}

}  // namespace orion_gb300
