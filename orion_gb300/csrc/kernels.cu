// Wavefront path tracer kernels for sm_103a.
//
// PathTracing::Li (src/integrator/path.cpp:50-99) is split into stages that
// each run over a device queue of path slots:
//
//   k_camera      Pinhole::generateRay for every path of the wave
//   k_trace       closest hit for the extension rays
//   k_shade       emission, BSDF construction, light sampling
//                 (uniformSampleOneLight / estimateDirect,
//                 src/core/integrator.cpp:8-90), BSDF sampling, Russian
//                 roulette; appends shadow / MIS / next-bounce work
//   k_trace_sh    occlusion for the light-sample shadow rays
//   k_trace       closest hit for the BSDF-sampled MIS rays (traced once;
//                 the reference traces that ray twice, once inside
//                 Triangle::pdf and once in estimateDirect)
//   k_film        per-pixel sums in sample order (RenderTarget::acumulate)
//
// A path's direct-lighting estimate is added to its radiance by its next
// k_shade, before anything else of that bounce, or by k_film if the path
// ended after sampling the light (shade_one, DEFER).
//
// Sample dimensions are consumed in exactly the reference's order, so every
// path sees the same Sobol numbers as the reference path with the same index.
#include <cuda_runtime.h>

#include "kernels.h"
#include "shade.cuh"

namespace orion_gb300 {

namespace {

__global__ void k_camera(SceneView s, WaveView w, WaveArgs a) {
  const int64_t wh = (int64_t)a.width * a.height;
  for (int pid = blockIdx.x * blockDim.x + threadIdx.x; pid < a.n_paths; pid += gridDim.x * blockDim.x) {
    int64_t index = a.base_index + pid;
    int64_t pix = index % wh;
    int i = (int)(pix % a.width), j = (int)(pix / a.width);
    V3 o, d;
    const uint32_t dim = camera_ray_block(s.cam, a.sobol, (uint64_t)index, i, j, &o, &d);
    // Whole 32-byte sectors only (a partly written sector costs L2 a DRAM
    // read): the ray, then the hit and meta sector. The throughput and
    // radiance sector is left out: bounce 0's shading takes 1 and 0 for them
    // (shade_one, FRESH) and writes them.
    PathRec& r = w.rec[pid];
    r.o = f4(o, 0.f);
    r.d = f4(d, 0.f);
    r.hit = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    r.meta = make_int4((int)dim, 0, 0, 0);
    w.q_ext[0][pid] = pid;
    w.qflags[pid] = 0;
  }
}

// Closest hit: extension rays (RayView = RecF4, hits into the path records,
// slots sorted by shading class) or MIS rays (NeeF4, hits into mis_hit).
// COUNT: the same traversal, adding its node visits and triangle tests to
// work[0] and work[3] (a diagnostic render; see WaveView::trace_work).
// CAP: traversal stack capacity (kTestStackEntries only in the kernels that
// exercise the overflow report); overflows set bits of *err.
template <int SMEM, class RayView, class HitView, bool COUNT = false, int CAP = kMaxStack>
__global__ void __launch_bounds__(512, 2)
    k_trace(SceneView s, const int* queue, const int* count, int* fetch, RayView ray_o, RayView ray_d, HitView hit,
            unsigned long long* stat, int refill_below, int* cls_counters, int* q_cls, int cls_stride,
            unsigned long long* work, int* err, uint8_t* cls_flags) {
  extern __shared__ int2 stack_smem[];
  const int n = *count;
  trace_persistent<false, SMEM, COUNT, CAP>(SingleScene{&s}, queue, n, fetch, ray_o, ray_d, hit, nullptr, stack_smem,
                                            refill_below, err, cls_counters, q_cls, cls_stride, work, cls_flags);
  if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stat, (unsigned long long)n);
}

template <int SMEM, bool COUNT = false, int CAP = kMaxStack>
__global__ void __launch_bounds__(512, 2)
    k_trace_sh(SceneView s, const int* queue, const int* count, int* fetch, NeeF4 ray_o, NeeF4 ray_d, int* occluded,
               unsigned long long* stat, int refill_below, unsigned long long* work, int* err) {
  extern __shared__ int2 stack_smem[];
  const int n = *count;
  trace_persistent<true, SMEM, COUNT, CAP>(SingleScene{&s}, queue, n, fetch, ray_o, ray_d, F4{nullptr}, occluded,
                                           stack_smem, refill_below, err, nullptr, nullptr, 0, work);
  if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stat, (unsigned long long)n);
}

// One bounce for every path whose extension ray hit a material of shading
// class SC (or, for SC_MISS, left the scene), with that class's BSDF code only.
// Launch bounds: at most 96 registers (5 blocks of 128 threads per SM).
// The queues a path goes to next (light-sample resolution, shadow ray, MIS
// rays, next extension ray) are recorded as bits of its qflags byte, and
// k_compact_queues lists them in slot order: the next trace launches then
// take rays of neighbouring pixels together instead of in the order the
// shading finished them.
template <int SC>
__global__ void __launch_bounds__(128, 5) k_shade(SceneView s, WaveView w, WaveArgs a, int bounce, int cur) {
  const int n = w.counters[CNT_CLS0 + SC];
  const int* in_q = w.q_cls + (size_t)SC * w.capacity;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = in_q[q];
    ShadeResult r = shade_one<lobes_of_class(SC), SC == SC_TEXTURED, true, true>(
        s, w, a.sobol, pid, (uint64_t)(a.base_index + pid), bounce, a.max_depth, a.rr_depth);
    w.qflags[pid] = (uint8_t)((r.alive ? kQfExt : 0) | (r.want_sh ? kQfShadow : 0) |
                              (r.want_mis ? kQfMis : 0) | (r.want_mis_env ? kQfMisEnv : 0));
  }
}

// Per-pixel accumulation in sample order: thread t owns the pixel of sample
// base + t and walks that pixel's samples of the wave in index order.
// A path whose last light sample is still pending (it ended right after
// sampling it) gets it added here, before its radiance is summed.
__global__ void k_film(SceneView s, WaveView w, WaveArgs a, FilmView film) {
  const int64_t wh = (int64_t)a.width * a.height;
  const int64_t nt = a.n_paths < wh ? a.n_paths : wh;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t pix = (a.base_index + t) % wh;
    float r = film.sum[3 * pix], g = film.sum[3 * pix + 1], b = film.sum[3 * pix + 2];
    double r64 = 0, g64 = 0, b64 = 0, rr = 0, gg = 0, bb = 0;
    uint32_t c = 0;
    for (int64_t k = t; k < a.n_paths; k += wh) {
      float4 l = w.L[k];
      if (w.dim[k] & kNeePending) {
        const V3 e = xyz(l) + nee_estimate(s, w, (int)k);
        l.x = e.x;
        l.y = e.y;
        l.z = e.z;
      }
      r += l.x;
      g += l.y;
      b += l.z;
      ++c;
      if (film.sum64) {
        r64 += l.x;
        g64 += l.y;
        b64 += l.z;
        rr += (double)l.x * l.x;
        gg += (double)l.y * l.y;
        bb += (double)l.z * l.z;
      }
    }
    film.sum[3 * pix] = r;
    film.sum[3 * pix + 1] = g;
    film.sum[3 * pix + 2] = b;
    if (film.count) film.count[pix] += c;
    if (film.sum64) {
      film.sum64[3 * pix] += r64;
      film.sum64[3 * pix + 1] += g64;
      film.sum64[3 * pix + 2] += b64;
      film.sumsq64[3 * pix] += rr;
      film.sumsq64[3 * pix + 1] += gg;
      film.sumsq64[3 * pix + 2] += bb;
    }
  }
}

template <int NQ>
__global__ void __launch_bounds__(kCompactThreads) k_compact_queues(uint8_t* flags, const int* list, const int* count,
                                                                    CompactTargets tg) {
  compact_queues<NQ>(flags, list, count, tg);
}

__global__ void k_reset_counters(int* counters, int slots, int keep_slot, int keep_value) {
  int i = threadIdx.x;
  if (i < slots) counters[i] = (i == keep_slot) ? keep_value : 0;
}

// Start of a bounce: empty the queues this bounce fills, zero the fetch counters.
__global__ void k_reset_bounce_counters(int* counters, int next_ext) {
  int i = threadIdx.x;
  if (i == 0) counters[next_ext] = 0;
  if (i == 1) counters[CNT_NEE] = 0;
  if (i == 2) counters[CNT_SH] = 0;
  if (i == 3) counters[CNT_MIS] = 0;
  if (i == 4) counters[CNT_FETCH_EXT] = 0;
  if (i == 5) counters[CNT_FETCH_SH] = 0;
  if (i == 6) counters[CNT_FETCH_MIS] = 0;
  if (i == CNT_MIS_ENV || i == CNT_FETCH_MIS_ENV) counters[i] = 0;
  if (i >= CNT_CLS0 && i < CNT_CLS0 + kShadeClasses) counters[i] = 0;
}

// ------------------------------------------------------------ test hooks

__global__ void k_sobol(const uint32_t* sobol, int64_t n, const uint64_t* index, const uint32_t* dim, float* out) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    out[i] = sobol_sample(sobol, index[i], dim[i]);
}

template <int SMEM>
__global__ void k_trace_rays(SceneView s, int64_t n, const float* rays, int any_hit, float* t, float* u, float* v,
                             int* prim) {
  extern __shared__ int2 stack_smem[];
  TraceScene ts = trace_scene(s);
  TraversalStack<SMEM> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float* r = rays + 8 * i;
    V3 o = V3{r[0], r[1], r[2]}, d = V3{r[3], r[4], r[5]};
    RayHit h = any_hit ? traverse<true, SMEM>(ts, o, d, r[6], r[7], st) : traverse<false, SMEM>(ts, o, d, r[6], r[7], st);
    t[i] = h.tri >= 0 ? h.t : 0.f;
    u[i] = h.u;
    v[i] = h.v;
    prim[i] = h.tri >= 0 ? __ldg(s.tri_prim + h.tri) : -1;
  }
}

// Production-traversal hook: n rays (o, d, tnear = 0, tfar) placed in a
// wave's records as extension rays (closest hit) or shadow rays (occlusion,
// tmax = tfar), so that the renderer's own persistent trace kernels trace them.
__global__ void k_load_rays(WaveView w, int n, const float* rays, int any_hit) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float* r = rays + 8 * (size_t)i;
    if (any_hit) {
      w.sh_o[i] = make_float4(r[0], r[1], r[2], r[7]);
      w.sh_d[i] = make_float4(r[3], r[4], r[5], 0.f);
      w.q_sh[i] = i;
    } else {
      w.ray_o[i] = make_float4(r[0], r[1], r[2], 0.f);
      w.ray_d[i] = make_float4(r[3], r[4], r[5], 0.f);
      w.q_ext[0][i] = i;
    }
  }
}

__global__ void k_store_hits(WaveView w, int n, int any_hit, float* t, float* u, float* v, int* prim) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (any_hit) {
      t[i] = u[i] = v[i] = 0.f;
      prim[i] = w.occluded[i] ? 1 : -1;
    } else {
      const float4 h = w.hit[i];
      const int p = __float_as_int(h.w);
      t[i] = p >= 0 ? h.x : 0.f;
      u[i] = h.y;
      v[i] = h.z;
      prim[i] = p;
    }
  }
}

__global__ void k_camera_rays(SceneView s, const uint32_t* sobol, int64_t n, const int64_t* index, float* rays) {
  const int64_t wh = (int64_t)s.cam.width * s.cam.height;
  for (int64_t q = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; q < n; q += (int64_t)gridDim.x * blockDim.x) {
    int64_t idx = index[q];
    int64_t pix = idx % wh;
    PathSampler smp{sobol, (uint64_t)idx, 5u};
    V3 o, d;
    camera_ray(s.cam, smp, (int)(pix % s.cam.width), (int)(pix / s.cam.width), &o, &d);
    float* r = rays + 6 * q;
    r[0] = o.x;
    r[1] = o.y;
    r[2] = o.z;
    r[3] = d.x;
    r[4] = d.y;
    r[5] = d.z;
  }
}

__global__ void k_bsdf_eval(const DevMaterial* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                            const float* rnd, int type, float* f, float* pdf, float* sf, float* swi, float* spdf,
                            int* stype, int* nbxdf) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float* fr = frame + 12 * i;
    Frame F{ld3(fr), ld3(fr + 3), ld3(fr + 6), ld3(fr + 9)};
    V3 o = ld3(wo + 3 * i), in = ld3(wi + 3 * i);
    V3 fv = bsdf_f(*mat, F, in, o, type);
    f[3 * i] = fv.x;
    f[3 * i + 1] = fv.y;
    f[3 * i + 2] = fv.z;
    pdf[i] = bsdf_pdf(*mat, F, in, o, type);
    V3 w = V3{0, 0, 0};
    float p = 0.f;
    int st = 0;
    V3 s = bsdf_sample_f(*mat, F, o, rnd[2 * i], rnd[2 * i + 1], type, &w, &p, &st);
    sf[3 * i] = s.x;
    sf[3 * i + 1] = s.y;
    sf[3 * i + 2] = s.z;
    swi[3 * i] = w.x;
    swi[3 * i + 1] = w.y;
    swi[3 * i + 2] = w.z;
    spdf[i] = p;
    stype[i] = st;
    nbxdf[i] = bsdf_num_matching(*mat, kNonSpecular);
  }
}

int grid_for(int64_t n, int block, int max_blocks) {
  int64_t g = (n + block - 1) / block;
  if (g > max_blocks) g = max_blocks;
  return (int)(g < 1 ? 1 : g);
}

enum TraceKind { TK_EXT = 0, TK_SHADOW = 1, TK_MIS = 2, TK_MIS_ENV = 3 };

template <int SMEM, bool COUNT = false, int CAP = kMaxStack>
void launch_trace_kernels(int kind, const SceneView& s, const WaveView& w, int cur, const LaunchConfig& cfg,
                          int grid, cudaStream_t stream) {
  const int block = cfg.trace_block;
  const int refill = cfg.refill_below < 1 ? 1 : (cfg.refill_below > 32 ? 32 : cfg.refill_below);
  // Any-hit rays end early and unevenly; their warps refill at 4 lanes more
  // (1024x1024 x 64 spp displaced sphere: 804 Mpaths/s against 798 at the
  // closest-hit threshold of 20, 787 at 16).
  const int refill_any = refill + 4 > 32 ? 32 : refill + 4;
  const size_t smem = trace_smem_bytes(SMEM, block);
  unsigned long long* work = w.trace_work;  // nodes[ext, shadow, mis], then tris[ext, shadow, mis]
  int* err = w.error_word;
  if (kind == TK_EXT)
    k_trace<SMEM, RecF4, RecF4, COUNT, CAP><<<grid, block, smem, stream>>>(
        s, w.q_ext[cur], w.counters + cur, w.counters + CNT_FETCH_EXT, w.ray_o, w.ray_d, w.hit, w.ray_stats, refill,
        w.counters + CNT_CLS0, w.q_cls, w.capacity, work, err, w.qflags);
  else if (kind == TK_SHADOW)
    k_trace_sh<SMEM, COUNT, CAP><<<grid, block, smem, stream>>>(s, w.q_sh, w.counters + CNT_SH,
                                                                w.counters + CNT_FETCH_SH, w.sh_o, w.sh_d, w.occluded,
                                                                w.ray_stats + 1, refill_any,
                                                                COUNT ? work + 1 : nullptr, err);
  else if (kind == TK_MIS_ENV)
    k_trace_sh<SMEM, COUNT, CAP><<<grid, block, smem, stream>>>(s, w.q_mis_env, w.counters + CNT_MIS_ENV,
                                                                w.counters + CNT_FETCH_MIS_ENV, w.mis_o, w.mis_d,
                                                                w.mis_occluded, w.ray_stats + 2, refill_any,
                                                                COUNT ? work + 2 : nullptr, err);
  else
    k_trace<SMEM, NeeF4, F4, COUNT, CAP><<<grid, block, smem, stream>>>(s, w.q_mis, w.counters + CNT_MIS,
                                                                        w.counters + CNT_FETCH_MIS, w.mis_o, w.mis_d,
                                                                        F4{w.mis_hit}, w.ray_stats + 2, refill,
                                                                        nullptr, nullptr, 0,
                                                                        COUNT ? work + 2 : nullptr, err, nullptr);
}

void trace_dispatch(int kind, const SceneView& s, const WaveView& w, int cur, const LaunchConfig& cfg, int grid,
                    cudaStream_t stream) {
  if (w.trace_work) {  // counting render: the stack's split between shared and local memory is irrelevant
    launch_trace_kernels<0, true>(kind, s, w, cur, cfg, grid, stream);
    return;
  }
  if (cfg.test_stack_entries) {  // orion_gpu_set_test_limits: kernels with a kTestStackEntries-entry stack
    launch_trace_kernels<0, false, kTestStackEntries>(kind, s, w, cur, cfg, grid, stream);
    return;
  }
  switch (cfg.smem_stack) {
    case 0: launch_trace_kernels<0>(kind, s, w, cur, cfg, grid, stream); break;
    case 8: launch_trace_kernels<8>(kind, s, w, cur, cfg, grid, stream); break;
    case 24: launch_trace_kernels<24>(kind, s, w, cur, cfg, grid, stream); break;
    case 32: launch_trace_kernels<32>(kind, s, w, cur, cfg, grid, stream); break;
    default: launch_trace_kernels<16>(kind, s, w, cur, cfg, grid, stream); break;
  }
}

}  // namespace

void launch_wave(const SceneView& s, const WaveView& w, const WaveArgs& a, const FilmView& film,
                 const LaunchConfig& cfg, cudaStream_t stream, int* launches, StageTimer* timer,
                 cudaEvent_t film_wait, cudaEvent_t film_done) {
  const int persistent = cfg.num_sms * cfg.blocks_per_sm;
  int nl = 0;
  auto begin = [&](int st) {
    if (timer) timer->begin(st, stream);
  };
  auto end = [&]() {
    if (timer) timer->end(stream);
    ++nl;
  };
  begin(ST_OTHER);
  k_reset_counters<<<1, 32, 0, stream>>>(w.counters, kCounterSlots, CNT_EXT0, a.n_paths);
  end();
  begin(ST_CAMERA);
  k_camera<<<grid_for(a.n_paths, 256, persistent * 4), 256, 0, stream>>>(s, w, a);
  end();
  // The persistent trace grids leave room on each SM for the other stream's
  // shading blocks (6 of 128 threads per SM: 24 of 64 warps; 1012 -> 1023
  // Mpaths/s on the displaced sphere, 2433 -> 2525 on eight spheres, against
  // grids that fill the register file).
  const int tgrid = grid_for(a.n_paths, cfg.trace_block, persistent);
  const int sgrid = grid_for(a.n_paths, cfg.shade_block, persistent * 2);
  const int compact_grid = grid_for(a.n_paths, kCompactSpan, cfg.num_sms * 8);
  CompactTargets class_tg{};
  for (int c = 0; c < kShadeClasses; ++c)
    class_tg.queue[c] = w.q_cls + (size_t)c * w.capacity, class_tg.counter[c] = w.counters + CNT_CLS0 + c;
  int cur = 0;
  for (int bounce = 0; bounce <= a.max_depth; ++bounce) {
    begin(ST_OTHER);
    k_reset_bounce_counters<<<1, 32, 0, stream>>>(w.counters, cur ^ 1);
    end();
    begin(ST_TRACE_EXT);
    trace_dispatch(TK_EXT, s, w, cur, cfg, tgrid, stream);
    end();
    // The trace marked each finished ray's shading class; list them by class in slot order.
    begin(ST_OTHER);
    k_compact_queues<kShadeClasses><<<compact_grid, kCompactThreads, 0, stream>>>(w.qflags, w.q_ext[cur],
                                                                                  w.counters + cur, class_tg);
    end();
    begin(ST_SHADE);
    for (int sc = 0; sc < kShadeClasses; ++sc) {
      if (!((a.class_mask >> sc) & 1u)) continue;
      switch (sc) {
        case SC_DIFFUSE: k_shade<SC_DIFFUSE><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_CONDUCTOR: k_shade<SC_CONDUCTOR><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_SPECULAR: k_shade<SC_SPECULAR><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_DIELECTRIC: k_shade<SC_DIELECTRIC><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_PLASTIC: k_shade<SC_PLASTIC><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_GENERAL: k_shade<SC_GENERAL><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_TEXTURED: k_shade<SC_TEXTURED><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        case SC_MISS: k_shade<SC_MISS><<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur); break;
        default: break;
      }
      ++nl;  // one launch per class present
    }
    --nl;  // end() counts one of them
    end();
    if (bounce < a.max_depth) {  // after the last bounce no path goes on and no queue is read
      begin(ST_OTHER);
      CompactTargets tg{};
      int* qs[5] = {w.q_ext[cur ^ 1], w.q_nee, w.q_sh, w.q_mis, w.q_mis_env};
      int* cs[5] = {w.counters + (cur ^ 1), w.counters + CNT_NEE, w.counters + CNT_SH, w.counters + CNT_MIS,
                    w.counters + CNT_MIS_ENV};
      for (int q = 0; q < 5; ++q) tg.queue[q] = qs[q], tg.counter[q] = cs[q];
      k_compact_queues<5><<<compact_grid, kCompactThreads, 0, stream>>>(w.qflags, w.q_ext[cur], w.counters + cur,
                                                                           tg);
      end();
    }
    if (bounce < a.max_depth) {
      begin(ST_TRACE_SHADOW);
      trace_dispatch(TK_SHADOW, s, w, cur, cfg, tgrid, stream);
      end();
      // MIS rays exist only towards area lights (closest hit) and environment
      // lights (occlusion); a scene without one kind skips its launch.
      begin(ST_TRACE_MIS);
      int mis = 0;
      if (s.num_area_lights > 0) {
        trace_dispatch(TK_MIS, s, w, cur, cfg, tgrid, stream);
        ++mis;
      }
      if (s.num_env > 0) {
        trace_dispatch(TK_MIS_ENV, s, w, cur, cfg, tgrid, stream);
        ++mis;
      }
      nl += mis - 1;  // end() counts one
      end();
      // No resolve pass: each path's light sample is added to its radiance by
      // its next shading, or by k_film if the path ends here (shade_one, DEFER).
    }
    cur ^= 1;
  }
  if (film_wait) cudaStreamWaitEvent(stream, film_wait, 0);
  begin(ST_FILM);
  k_film<<<grid_for(a.n_paths, 256, persistent * 4), 256, 0, stream>>>(s, w, a, film);
  end();
  if (film_done) cudaEventRecord(film_done, stream);
  if (launches) *launches += nl;
}

void launch_sobol(const uint32_t* sobol, int64_t n, const uint64_t* index, const uint32_t* dim, float* out,
                  cudaStream_t stream) {
  k_sobol<<<grid_for(n, 256, 4096), 256, 0, stream>>>(sobol, n, index, dim, out);
}

void launch_trace(const SceneView& s, int64_t n, const float* rays, int any_hit, float* t, float* u, float* v,
                  int* prim, const LaunchConfig& cfg, cudaStream_t stream) {
  int block = cfg.trace_block;
  int grid = grid_for(n, block, cfg.num_sms * cfg.blocks_per_sm * 2);
  k_trace_rays<16><<<grid, block, (size_t)16 * block * sizeof(int2), stream>>>(s, n, rays, any_hit, t, u, v, prim);
}

void launch_trace_wave(const SceneView& s, const WaveView& w, int n, const float* rays, int any_hit, float* t,
                       float* u, float* v, int* prim, const LaunchConfig& cfg, cudaStream_t stream) {
  k_reset_counters<<<1, 32, 0, stream>>>(w.counters, kCounterSlots, any_hit ? CNT_SH : CNT_EXT0, n);
  k_load_rays<<<grid_for(n, 256, 4096), 256, 0, stream>>>(w, n, rays, any_hit);
  const int tgrid = grid_for(n, cfg.trace_block, cfg.num_sms * cfg.blocks_per_sm);
  trace_dispatch(any_hit ? TK_SHADOW : TK_EXT, s, w, 0, cfg, tgrid, stream);
  k_store_hits<<<grid_for(n, 256, 4096), 256, 0, stream>>>(w, n, any_hit, t, u, v, prim);
}

namespace {

cudaError_t limit_of(const void* f, int smem_bytes, int* max_block) {
  if (smem_bytes > 0) {
    cudaError_t e = cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, smem_bytes);
    if (e != cudaSuccess) return e;
  }
  cudaFuncAttributes a;
  cudaError_t e = cudaFuncGetAttributes(&a, f);
  if (e != cudaSuccess) return e;
  *max_block = std::min(*max_block, a.maxThreadsPerBlock);
  return cudaSuccess;
}

}  // namespace

cudaError_t configure_kernels(int smem_bytes, KernelLimits* lim) {
  const void* trace[] = {
      (const void*)k_trace<0, RecF4, RecF4>,  (const void*)k_trace<8, RecF4, RecF4>,
      (const void*)k_trace<16, RecF4, RecF4>, (const void*)k_trace<24, RecF4, RecF4>,
      (const void*)k_trace<32, RecF4, RecF4>, (const void*)k_trace<0, NeeF4, F4>,
      (const void*)k_trace<8, NeeF4, F4>,     (const void*)k_trace<16, NeeF4, F4>,
      (const void*)k_trace<24, NeeF4, F4>,    (const void*)k_trace<32, NeeF4, F4>,
      (const void*)k_trace_sh<0>,             (const void*)k_trace_sh<8>,
      (const void*)k_trace_sh<16>,            (const void*)k_trace_sh<24>,
      (const void*)k_trace_sh<32>,            (const void*)k_trace_rays<16>,
      (const void*)k_trace<0, RecF4, RecF4, true>, (const void*)k_trace<0, NeeF4, F4, true>,
      (const void*)k_trace_sh<0, true>};
  const void* shade[] = {(const void*)k_shade<SC_DIFFUSE>, (const void*)k_shade<SC_CONDUCTOR>,
                         (const void*)k_shade<SC_SPECULAR>, (const void*)k_shade<SC_DIELECTRIC>,
                         (const void*)k_shade<SC_PLASTIC>, (const void*)k_shade<SC_GENERAL>, (const void*)k_shade<SC_TEXTURED>,
                         (const void*)k_shade<SC_MISS>};
  for (const void* f : trace) {
    cudaError_t e = limit_of(f, smem_bytes, &lim->max_trace_block);
    if (e != cudaSuccess) return e;
  }
  for (const void* f : shade) {
    cudaError_t e = limit_of(f, 0, &lim->max_shade_block);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

void launch_camera_rays(const SceneView& s, const uint32_t* sobol, int64_t n, const int64_t* index, float* rays,
                        cudaStream_t stream) {
  k_camera_rays<<<grid_for(n, 256, 4096), 256, 0, stream>>>(s, sobol, n, index, rays);
}

void launch_bsdf_eval(const DevMaterial* mat, int64_t n, const float* frame, const float* wo, const float* wi,
                      const float* rnd, int type, float* f, float* pdf, float* sf, float* swi, float* spdf,
                      int* stype, int* nbxdf, cudaStream_t stream) {
  k_bsdf_eval<<<grid_for(n, 128, 4096), 128, 0, stream>>>(mat, n, frame, wo, wi, rnd, type, f, pdf, sf, swi, spdf,
                                                           stype, nbxdf);
}

}  // namespace orion_gb300
