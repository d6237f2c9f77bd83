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
//   k_resolve     adds the direct-lighting estimate to the path radiance
//   k_film        per-pixel sums in sample order (RenderTarget::acumulate)
//
// Sample dimensions are consumed in exactly the reference's order, so every
// path sees the same Sobol numbers as the reference path with the same index.
#include <cuda_runtime.h>

#include "bsdf.cuh"
#include "dmath.cuh"
#include "kernels.h"
#include "light.cuh"
#include "traverse.cuh"

namespace orion_gb300 {

namespace {

constexpr int kNonSpecular = BXDF_ALL & ~BXDF_SPECULAR;
constexpr int kFlagShadow = 1, kFlagMis = 2, kFlagEnv = 4;

__device__ __forceinline__ void queue_append(int* counter, int* queue, int value, bool pred) {
  unsigned active = __activemask();
  unsigned m = __ballot_sync(active, pred);
  if (!pred) return;
  int lane = threadIdx.x & 31;
  int leader = __ffs(m) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counter, __popc(m));
  base = __shfl_sync(m, base, leader);
  queue[base + __popc(m & ((1u << lane) - 1u))] = value;
}

struct Hit {
  V3 p, ng, ns, su, sv;
};

// Post-hit reconstruction (src/core/kernel.cpp:127-169).
__device__ __forceinline__ Hit reconstruct(const PrimShade& sh, float u, float v) {
  Hit h;
  V3 p0 = ld3(sh.p), p1 = ld3(sh.p + 3), p2 = ld3(sh.p + 6);
  float w = 1.f - u - v;
  h.p = w * p0 + u * p1 + v * p2;
  h.ns = ld3(sh.n) * w + ld3(sh.n + 3) * u + ld3(sh.n + 6) * v;
  h.ng = normalize(cross(p1 - p0, p2 - p0));
  V3 su = normalize(p1 - p0);
  h.sv = normalize(cross(h.ns, su));
  h.su = normalize(cross(h.sv, h.ns));
  return h;
}

__device__ __forceinline__ V3 geometric_normal(const PrimShade& sh) {
  V3 p0 = ld3(sh.p), p1 = ld3(sh.p + 3), p2 = ld3(sh.p + 6);
  return normalize(cross(p1 - p0, p2 - p0));
}

__device__ __forceinline__ V3 point_on(const PrimShade& sh, float u, float v) {
  V3 p0 = ld3(sh.p), p1 = ld3(sh.p + 3), p2 = ld3(sh.p + 6);
  float w = 1.f - u - v;
  return w * p0 + u * p1 + v * p2;
}

__device__ __forceinline__ TraceScene trace_scene(const SceneView& s) { return TraceScene{s.nodes, s.woop, s.tri_prim}; }

// Pinhole::generateRay (src/camera/pinhole.cpp:8-33).
// Sampler::next2() builds Point2f(next(), next()) (src/core/sampler.h:29); the
// two calls are unsequenced and the compiled reference evaluates the second
// first, so .x holds the later dimension. All 2-D samples follow that order.
__device__ __forceinline__ void camera_ray(const DevCamera& c, PathSampler& smp, int i, int j, V3* o, V3* d) {
  float s0 = smp.next(), s1 = smp.next();
  float rx = (float)i + s1;
  float ry = (float)j + s0;
  float xx = (2.f * rx / (float)c.width - 1.f) * c.aspect * c.tan_half_fov;
  float yy = (1.f - 2.f * ry / (float)c.height) * c.tan_half_fov;
  V3 dir = normalize(V3{xx, yy, -1.f});
  V3 org = V3{0.f, 0.f, 0.f};
  if (c.lens_radius > 0.f) {
    V3 target = org + dir * c.focal_distance;
    float lx, ly;
    float l0 = smp.next(), l1 = smp.next();
    concentric_sample_disk(l1, l0, &lx, &ly);
    org = V3{lx * c.lens_radius, ly * c.lens_radius, 0.f};
    dir = normalize(target - org);
  }
  const float* m = c.c2w;
  float xp = m[0] * org.x + m[1] * org.y + m[2] * org.z + m[3];
  float yp = m[4] * org.x + m[5] * org.y + m[6] * org.z + m[7];
  float zp = m[8] * org.x + m[9] * org.y + m[10] * org.z + m[11];
  float wp = m[12] * org.x + m[13] * org.y + m[14] * org.z + m[15];
  if (wp == 1.f)
    *o = V3{xp, yp, zp};
  else
    *o = vdiv(V3{xp, yp, zp}, wp);
  *d = V3{m[0] * dir.x + m[1] * dir.y + m[2] * dir.z, m[4] * dir.x + m[5] * dir.y + m[6] * dir.z,
          m[8] * dir.x + m[9] * dir.y + m[10] * dir.z};
}

__global__ void k_camera(SceneView s, WaveView w, WaveArgs a) {
  const int64_t wh = (int64_t)a.width * a.height;
  for (int pid = blockIdx.x * blockDim.x + threadIdx.x; pid < a.n_paths; pid += gridDim.x * blockDim.x) {
    int64_t index = a.base_index + pid;
    int64_t pix = index % wh;
    int i = (int)(pix % a.width), j = (int)(pix / a.width);
    PathSampler smp{a.sobol, (uint64_t)index, 5u};
    V3 o, d;
    camera_ray(s.cam, smp, i, j, &o, &d);
    w.ray_o[pid] = f4(o, 0.f);
    w.ray_d[pid] = f4(d, 0.f);
    w.beta[pid] = make_float4(1.f, 1.f, 1.f, 0.f);
    w.L[pid] = make_float4(0.f, 0.f, 0.f, 0.f);
    w.dim[pid] = (int)smp.dim;
    w.q_ext[0][pid] = pid;
  }
}

template <int SMEM>
__device__ __forceinline__ void trace_queue(const SceneView& s, const int* queue, const int* count,
                                            const float4* ray_o, const float4* ray_d, float4* hit, int2* stack_smem,
                                            unsigned long long* stat) {
  TraceScene ts = trace_scene(s);
  TraversalStack<SMEM> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  int n = *count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int pid = queue[q];
    float4 o4 = ray_o[pid], d4 = ray_d[pid];
    RayHit h = traverse<false, SMEM>(ts, xyz(o4), xyz(d4), 0.f, kFloatMax, st);
    hit[pid] = make_float4(h.t, h.u, h.v, __int_as_float(h.tri));
  }
  if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stat, (unsigned long long)n);
}

template <int SMEM>
__global__ void k_trace(SceneView s, const int* queue, const int* count, const float4* ray_o, const float4* ray_d,
                        float4* hit, unsigned long long* stat) {
  extern __shared__ int2 stack_smem[];
  trace_queue<SMEM>(s, queue, count, ray_o, ray_d, hit, stack_smem, stat);
}

template <int SMEM>
__global__ void k_trace_sh(SceneView s, const int* queue, const int* count, const float4* ray_o,
                           const float4* ray_d, int* occluded, unsigned long long* stat) {
  extern __shared__ int2 stack_smem[];
  TraceScene ts = trace_scene(s);
  TraversalStack<SMEM> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  int n = *count;
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    int pid = queue[q];
    float4 o4 = ray_o[pid], d4 = ray_d[pid];
    RayHit h = traverse<true, SMEM>(ts, xyz(o4), xyz(d4), 0.f, o4.w, st);
    occluded[pid] = h.tri >= 0;
  }
  if (stat && blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(stat, (unsigned long long)n);
}

// One bounce of PathTracing::Li for every path in the queue.
__global__ void k_shade(SceneView s, WaveView w, WaveArgs a, int bounce, int cur) {
  const int* in_q = w.q_ext[cur];
  int* out_q = w.q_ext[cur ^ 1];
  int* out_cnt = w.counters + (cur ^ 1);
  const int n = w.counters[cur];
  LightDistrib distrib{s.light_func, s.light_cdf, s.light_func_int, s.num_lights};
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = in_q[q];
    const float4 hv = w.hit[pid];
    const int tri = __float_as_int(hv.w);
    const V3 ro = xyz(w.ray_o[pid]);
    const V3 rd = xyz(w.ray_d[pid]);
    float4 b4 = w.beta[pid];
    V3 beta = xyz(b4);
    const bool spec_prev = b4.w != 0.f;
    V3 L = xyz(w.L[pid]);
    const int prim = tri >= 0 ? __ldg(s.tri_prim + tri) : -1;

    // Emission on the first hit or after a specular bounce (path.cpp:61-69).
    if (bounce == 0 || spec_prev) {
      if (prim >= 0) {
        int li = __ldg(&s.prims[prim].light);
        if (li >= 0) {
          V3 ng = geometric_normal(s.prims[prim]);
          if (dot(ng, -rd) > 0.f) L = L + mul(beta, ld3(s.lights[li].L));
        }
      } else {
        for (int e = 0; e < s.num_env; ++e) L = L + mul(beta, ld3(s.lights[s.env_idx[e]].L));
      }
    }
    bool alive = prim >= 0 && bounce < a.max_depth;
    bool did_nee = false, want_sh = false, want_mis = false;
    if (alive) {
      const PrimShade& sh = s.prims[prim];
      Hit h = reconstruct(sh, hv.y, hv.z);
      const DevMaterial& m = s.mats[sh.material];
      Frame fr{h.ng, h.ns, h.su, h.sv};
      PathSampler smp{a.sobol, (uint64_t)(a.base_index + pid), (uint32_t)w.dim[pid]};

      // uniformSampleOneLight (integrator.cpp:8-27) when a non-specular lobe exists.
      if (m.num_nonspecular > 0 && s.num_lights > 0) {
        float sel_pdf;
        int li = sample_discrete(distrib, smp.next(), &sel_pdf);
        if (sel_pdf != 0.f) {
          float ul1 = smp.next(), ul0 = smp.next();  // next2(): .x is the later dimension
          float ub1 = smp.next(), ub0 = smp.next();
          const DevLight& lt = s.lights[li];
          V3 wo = normalize(-rd);
          // estimateDirect, light-sampling half (integrator.cpp:39-60).
          LightSample ls = sample_li(lt, s.prims, h.p, ul0, ul1, s.world_radius);
          V3 ld = V3{0, 0, 0};
          if (ls.pdf > 0.f && !is_black(ls.Li)) {
            V3 f = bsdf_f(m, fr, ls.wi, wo, kNonSpecular) * absdot(ls.wi, h.ns);
            float bpdf = bsdf_pdf(m, fr, ls.wi, wo, kNonSpecular);
            if (!is_black(f)) {
              if (is_delta_light(lt.kind)) {
                ld = sdiv(mul(f, ls.Li), ls.pdf);
              } else {
                float wgt = power_heuristic(ls.pdf, bpdf);
                ld = sdiv(mul(f, ls.Li) * wgt, ls.pdf);
              }
              // ShadowTester::unoccluded (light.h:26-29): Intersection::spawnRay to a point.
              V3 so = offset_ray_origin(h.p, h.ng, ls.p_light - h.p);
              w.sh_o[pid] = f4(so, 1.f - kShadowEpsilon);
              w.sh_d[pid] = f4(ls.p_light - so, 0.f);
              want_sh = true;
            }
          }
          // estimateDirect, BSDF-sampling half (integrator.cpp:62-89).
          int flags = want_sh ? kFlagShadow : 0;
          float mis_pdf = 0.f, env_w = 0.f;
          V3 fb = V3{0, 0, 0};
          if (!is_delta_light(lt.kind)) {
            V3 wib;
            int st;
            fb = bsdf_sample_f(m, fr, wo, ub0, ub1, kNonSpecular, &wib, &mis_pdf, &st);
            fb = fb * absdot(wib, h.ns);
            if (!is_black(fb) && mis_pdf > 0.f) {
              bool ok = true;
              if (lt.kind == DL_ENV) {
                float lpdf = env_pdf_li(lt, wib);
                if (lpdf == 0.f)
                  ok = false;
                else {
                  env_w = power_heuristic(mis_pdf, lpdf);
                  flags |= kFlagEnv;
                }
              }
              if (ok) {
                V3 mo = offset_ray_origin(h.p, h.ng, wib);
                w.mis_o[pid] = f4(mo, 0.f);
                w.mis_d[pid] = f4(wib, 0.f);
                want_mis = true;
                flags |= kFlagMis;
              }
            }
          }
          w.nee_p[pid] = f4(h.p, sel_pdf);
          w.nee_beta[pid] = f4(beta, __int_as_float(flags | (li << 8)));
          w.nee_ld[pid] = f4(ld, mis_pdf);
          w.nee_f[pid] = f4(fb, env_w);
          did_nee = true;
        }
      }

      // Continuation: BSDF sample, throughput, spawn, Russian roulette (path.cpp:81-96).
      float u1 = smp.next(), u0 = smp.next();  // next2(): .x is the later dimension
      V3 wi;
      float pdf;
      int stype;
      V3 f = bsdf_sample_f(m, fr, -rd, u0, u1, BXDF_ALL, &wi, &pdf, &stype);
      if (is_black(f) || pdf == 0.f) {
        alive = false;
      } else {
        beta = mul(beta, sdiv(f * absdot(wi, h.ns), pdf));
        bool spec = (stype & BXDF_SPECULAR) != 0;
        V3 no = offset_ray_origin(h.p, h.ng, wi);
        if (bounce > a.rr_depth) {
          float qq = fmaxf(0.05f, 1.f - max_comp(beta));
          if (smp.next() < qq)
            alive = false;
          else
            beta = sdiv(beta, 1.f - qq);
        }
        if (alive) {
          w.ray_o[pid] = f4(no, 0.f);
          w.ray_d[pid] = f4(wi, 0.f);
          w.beta[pid] = f4(beta, spec ? 1.f : 0.f);
        }
      }
      w.dim[pid] = (int)smp.dim;
    }
    w.L[pid] = f4(L, 0.f);
    queue_append(w.counters + CNT_NEE, w.q_nee, pid, did_nee);
    queue_append(w.counters + CNT_SH, w.q_sh, pid, want_sh);
    queue_append(w.counters + CNT_MIS, w.q_mis, pid, want_mis);
    queue_append(out_cnt, out_q, pid, alive);
  }
}

// Adds beta * Ld / selPdf for every path that sampled a light this bounce.
__global__ void k_resolve(SceneView s, WaveView w) {
  const int n = w.counters[CNT_NEE];
  for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
    const int pid = w.q_nee[q];
    float4 pb = w.nee_beta[pid];
    int fl = __float_as_int(pb.w);
    int li = fl >> 8;
    float4 np = w.nee_p[pid];
    float4 ldv = w.nee_ld[pid];
    V3 Ld = V3{0, 0, 0};
    if ((fl & kFlagShadow) && !w.occluded[pid]) Ld = Ld + xyz(ldv);
    if (fl & kFlagMis) {
      const DevLight& lt = s.lights[li];
      float4 fv = w.nee_f[pid];
      V3 fb = xyz(fv);
      float bpdf = ldv.w;
      float4 mh = w.mis_hit[pid];
      int tri = __float_as_int(mh.w);
      V3 wi = xyz(w.mis_d[pid]);
      if (fl & kFlagEnv) {
        if (tri < 0) Ld = Ld + sdiv(mul(fb, ld3(lt.L)) * fv.w, bpdf);
      } else if (tri >= 0) {
        int prim = __ldg(s.tri_prim + tri);
        if (prim == lt.prim) {
          // Triangle::pdf (src/core/triangle.cpp:123-135) on the traced hit.
          const PrimShade& sh = s.prims[prim];
          V3 ip = point_on(sh, mh.y, mh.z);
          V3 ing = geometric_normal(sh);
          float lpdf = length_sq(xyz(np) - ip) / (absdot(ing, -wi) * lt.area);
          if (isinf(lpdf)) lpdf = 0.f;
          if (lpdf != 0.f) {
            float wgt = power_heuristic(bpdf, lpdf);
            V3 Li = dot(ing, -wi) > 0.f ? ld3(lt.L) : V3{0, 0, 0};
            if (!is_black(Li)) Ld = Ld + sdiv(mul(fb, Li) * wgt, bpdf);
          }
        }
      }
    }
    V3 L = xyz(w.L[pid]);
    L = L + mul(xyz(pb), sdiv(Ld, np.w));
    w.L[pid] = f4(L, 0.f);
  }
}

// Per-pixel accumulation in sample order: thread t owns the pixel of sample
// base + t and walks that pixel's samples of the wave in index order.
__global__ void k_film(WaveView w, WaveArgs a, FilmView film) {
  const int64_t wh = (int64_t)a.width * a.height;
  const int64_t nt = a.n_paths < wh ? a.n_paths : wh;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < nt; t += (int64_t)gridDim.x * blockDim.x) {
    int64_t pix = (a.base_index + t) % wh;
    float r = film.sum[3 * pix], g = film.sum[3 * pix + 1], b = film.sum[3 * pix + 2];
    double r64 = 0, g64 = 0, b64 = 0, rr = 0, gg = 0, bb = 0;
    uint32_t c = 0;
    for (int64_t k = t; k < a.n_paths; k += wh) {
      float4 l = w.L[k];
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

__global__ void k_reset_counters(int* counters, int slots, int keep_slot, int keep_value) {
  int i = threadIdx.x;
  if (i < slots) counters[i] = (i == keep_slot) ? keep_value : 0;
}

__global__ void k_reset_nee_counters(int* counters, int next_ext) {
  int i = threadIdx.x;
  if (i == 0) counters[next_ext] = 0;
  if (i == 1) counters[CNT_NEE] = 0;
  if (i == 2) counters[CNT_SH] = 0;
  if (i == 3) counters[CNT_MIS] = 0;
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

template <int SMEM>
void launch_trace_kernels(bool shadow, const SceneView& s, const int* queue, const int* count, const float4* o,
                          const float4* d, float4* hit, int* occl, unsigned long long* stat, int grid, int block,
                          cudaStream_t stream) {
  size_t smem = (size_t)SMEM * block * sizeof(int2);
  if (shadow)
    k_trace_sh<SMEM><<<grid, block, smem, stream>>>(s, queue, count, o, d, occl, stat);
  else
    k_trace<SMEM><<<grid, block, smem, stream>>>(s, queue, count, o, d, hit, stat);
}

void trace_dispatch(int smem_stack, bool shadow, const SceneView& s, const int* queue, const int* count,
                    const float4* o, const float4* d, float4* hit, int* occl, unsigned long long* stat, int grid,
                    int block, cudaStream_t stream) {
  switch (smem_stack) {
    case 0: launch_trace_kernels<0>(shadow, s, queue, count, o, d, hit, occl, stat, grid, block, stream); break;
    case 8: launch_trace_kernels<8>(shadow, s, queue, count, o, d, hit, occl, stat, grid, block, stream); break;
    case 24: launch_trace_kernels<24>(shadow, s, queue, count, o, d, hit, occl, stat, grid, block, stream); break;
    case 32: launch_trace_kernels<32>(shadow, s, queue, count, o, d, hit, occl, stat, grid, block, stream); break;
    default: launch_trace_kernels<16>(shadow, s, queue, count, o, d, hit, occl, stat, grid, block, stream); break;
  }
}

}  // namespace

void launch_wave(const SceneView& s, const WaveView& w, const WaveArgs& a, const FilmView& film,
                 const LaunchConfig& cfg, cudaStream_t stream, int* launches, StageTimer* timer) {
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
  const int tgrid = grid_for(a.n_paths, cfg.trace_block, persistent * 2);
  const int sgrid = grid_for(a.n_paths, cfg.shade_block, persistent * 2);
  int cur = 0;
  for (int bounce = 0; bounce <= a.max_depth; ++bounce) {
    begin(ST_TRACE_EXT);
    trace_dispatch(cfg.smem_stack, false, s, w.q_ext[cur], w.counters + cur, w.ray_o, w.ray_d, w.hit, nullptr,
                   w.ray_stats, tgrid, cfg.trace_block, stream);
    end();
    begin(ST_OTHER);
    k_reset_nee_counters<<<1, 32, 0, stream>>>(w.counters, cur ^ 1);
    end();
    begin(ST_SHADE);
    k_shade<<<sgrid, cfg.shade_block, 0, stream>>>(s, w, a, bounce, cur);
    end();
    if (bounce < a.max_depth) {
      begin(ST_TRACE_SHADOW);
      trace_dispatch(cfg.smem_stack, true, s, w.q_sh, w.counters + CNT_SH, w.sh_o, w.sh_d, nullptr, w.occluded,
                     w.ray_stats + 1, tgrid, cfg.trace_block, stream);
      end();
      begin(ST_TRACE_MIS);
      trace_dispatch(cfg.smem_stack, false, s, w.q_mis, w.counters + CNT_MIS, w.mis_o, w.mis_d, w.mis_hit, nullptr,
                     w.ray_stats + 2, tgrid, cfg.trace_block, stream);
      end();
      begin(ST_RESOLVE);
      k_resolve<<<sgrid, cfg.shade_block, 0, stream>>>(s, w);
      end();
    }
    cur ^= 1;
  }
  begin(ST_FILM);
  k_film<<<grid_for(a.n_paths, 256, persistent * 4), 256, 0, stream>>>(w, a, film);
  end();
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
