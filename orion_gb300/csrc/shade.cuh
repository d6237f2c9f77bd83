// Per-path stages of the wavefront path tracer shared by the plain
// (one image per launch) and batched (many jobs per launch) drivers.
#pragma once
#include "bsdf.cuh"
#include "dmath.cuh"
#include "kernels.h"
#include "light.cuh"
#include "material_build.h"
#include "traverse.cuh"

#include <type_traits>

namespace orion_gb300 {

constexpr int kNonSpecular = BXDF_ALL & ~BXDF_SPECULAR;
constexpr int kFlagShadow = 1, kFlagMis = 2, kFlagEnv = 4;
// Plain waves: set in a path's Sobol dimension word (rec.meta.x) while its
// last light sample waits to be added to its radiance (shade_one, k_film).
constexpr int kNeePending = 1 << 30;

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

// Appends `value` to queue `cls` of `queues` (`stride` ints apart); the lanes
// of a warp that append to the same queue share one atomicAdd.
__device__ __forceinline__ void class_append(int* counters, int* queues, int stride, int cls, int value) {
  const unsigned active = __activemask();
  const unsigned peers = __match_any_sync(active, cls);
  const int lane = threadIdx.x & 31;
  const int leader = __ffs(peers) - 1;
  int base = 0;
  if (lane == leader) base = atomicAdd(counters + cls, __popc(peers));
  base = __shfl_sync(peers, base, leader);
  queues[(size_t)cls * stride + base + __popc(peers & ((1u << lane) - 1u))] = value;
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

// Texture coordinates at barycentrics (u, v) (src/core/kernel.cpp:138-142),
// rounded without contraction: the texel choice is discontinuous in them.
__device__ __forceinline__ void hit_uv(const float* uv, float u, float v, float* x, float* y) {
  const float w = __fsub_rn(__fsub_rn(1.f, u), v);
  *x = __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(uv + 0)), __fmul_rn(u, __ldg(uv + 2))), __fmul_rn(v, __ldg(uv + 4)));
  *y = __fadd_rn(__fadd_rn(__fmul_rn(w, __ldg(uv + 1)), __fmul_rn(u, __ldg(uv + 3))), __fmul_rn(v, __ldg(uv + 5)));
}

// Texture::evaluate -> ImageTexture::sample(int, int) with the wrap filter
// (src/core/texture.cpp:8-29, src/texture/imagetexture.cpp:4-12): texel
// (int)(u * width), (int)(v * height), wrapped. The reference wraps a
// negative multiple of the size to the size itself and reads the texel that
// follows in memory (the next row's first); past the last texel, undefined
// there, the last texel is read here.
__device__ __forceinline__ V3 texture_eval(const DevTexture& t, float x, float y) {
  const int w = t.width, h = t.height;
  int ix = __float2int_rz(__fmul_rn(x, (float)w)), iy = __float2int_rz(__fmul_rn(y, (float)h));
  ix = ix >= 0 ? ix % w : w - (int)((0u - (unsigned)ix) % (unsigned)w);
  iy = iy >= 0 ? iy % h : h - (int)((0u - (unsigned)iy) % (unsigned)h);
  int64_t off = (int64_t)iy * w + ix;
  const int64_t last = (int64_t)w * h - 1;
  off = off > last ? last : off;
  const float* p = t.texels + 3 * off;
  return V3{__ldg(p), __ldg(p + 1), __ldg(p + 2)};
}

// Material::getBSDF of a textured material at texture coordinates (x, y):
// its image inputs looked up, then the lobe list built as the host builds
// constant materials.
static __device__ __noinline__ void textured_material(const SceneView& s, int mi, float x, float y, DevMaterial* m) {
  const DevMaterialSrc& src = s.mat_src[mi];
  MaterialInputs in = src.in;
#pragma unroll
  for (int t = 0; t < kTexSlots; ++t) {
    const int ti = src.tex[t];
    if (ti < 0) continue;
    const V3 c = texture_eval(s.textures[ti], x, y);
    float* d = t == ORION_TEX_KD ? in.Kd
               : t == ORION_TEX_KS ? in.Ks
               : t == ORION_TEX_KR ? in.Kr
               : t == ORION_TEX_KT ? in.Kt
               : t == ORION_TEX_OPACITY ? in.opacity
               : t == ORION_TEX_ETA ? in.eta_rgb
                                    : in.k;
    d[0] = c.x;
    d[1] = c.y;
    d[2] = c.z;
  }
  build_material(in, m);
}

__device__ __forceinline__ TraceScene trace_scene(const SceneView& s) { return TraceScene{s.nodes, s.woop, s.tri_prim, s.tri_class}; }

// Pinhole::generateRay (src/camera/pinhole.cpp:8-33).
// Sampler::next2() builds Point2f(next(), next()) (src/core/sampler.h:29); the
// two calls are unsequenced and the compiled reference evaluates the second
// first, so .x holds the later dimension. All 2-D samples follow that order.
// u: the path's sample dimensions 5..8 in order (pixel jitter, then lens).
__device__ __forceinline__ void camera_ray_u(const DevCamera& c, const float u[4], int i, int j, V3* o, V3* d) {
  float s0 = u[0], s1 = u[1];
  float rx = (float)i + s1;
  float ry = (float)j + s0;
  float xx = (2.f * rx / (float)c.width - 1.f) * c.aspect * c.tan_half_fov;
  float yy = (1.f - 2.f * ry / (float)c.height) * c.tan_half_fov;
  V3 dir = normalize(V3{xx, yy, -1.f});
  V3 org = V3{0.f, 0.f, 0.f};
  if (c.lens_radius > 0.f) {
    V3 target = org + dir * c.focal_distance;
    float lx, ly;
    float l0 = u[2], l1 = u[3];
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

// Pinhole::generateRay from a path's sampler (dimensions consumed in order).
__device__ __forceinline__ void camera_ray(const DevCamera& c, PathSampler& smp, int i, int j, V3* o, V3* d) {
  float u[4];
  u[0] = smp.next();
  u[1] = smp.next();
  if (c.lens_radius > 0.f) {
    u[2] = smp.next();
    u[3] = smp.next();
  }
  camera_ray_u(c, u, i, j, o, d);
}

// The same with its 2 (pinhole) or 4 (thin lens) sample dimensions drawn
// together; returns the next sample dimension (7 or 9).
__device__ __forceinline__ uint32_t camera_ray_block(const DevCamera& c, const uint32_t* __restrict__ tables,
                                                     uint64_t index, int i, int j, V3* o, V3* d) {
  float u[4];
  if (c.lens_radius > 0.f) {
    sobol_dims<4>(tables, index, 5u, u);
  } else {
    sobol_dims<2>(tables, index, 5u, u);
    u[2] = u[3] = 0.f;
  }
  camera_ray_u(c, u, i, j, o, d);
  return c.lens_radius > 0.f ? 9u : 7u;
}

// One bounce of PathTracing::Li (src/integrator/path.cpp:56-97) for path slot
// `pid`: emission, BSDF, light sample (uniformSampleOneLight /
// estimateDirect, src/core/integrator.cpp:8-90), continuation, roulette.
// Writes the path state and NEE records; the caller appends the slot to the
// queues the result asks for.
struct ShadeResult {
  bool alive, did_nee, want_sh, want_mis, want_mis_env;
};

// Lobe kinds a shading class's materials can hold (see prepare_material).
__host__ __device__ constexpr unsigned lobes_of_class(int sc) {
  return sc == SC_DIFFUSE      ? (1u << LOBE_LAMBERT_R)
         : sc == SC_CONDUCTOR  ? (1u << LOBE_MICROFACET_R)
         : sc == SC_SPECULAR   ? ((1u << LOBE_SPECULAR_R) | (1u << LOBE_SPECULAR_T) | (1u << LOBE_FRESNEL_SPECULAR))
         : sc == SC_DIELECTRIC ? ((1u << LOBE_MICROFACET_R) | (1u << LOBE_MICROFACET_T))
         : sc == SC_PLASTIC    ? ((1u << LOBE_LAMBERT_R) | (1u << LOBE_MICROFACET_R))
         : sc == SC_MISS       ? 0u
                               : kLobeAll;
}

// beta * Ld / selPdf of the light sample a path's shading left in its NEE
// record (path.cpp:77-80), once its shadow and MIS rays are traced; the
// radiance adds it next (resolve_one, or the next bounce's shading).
__device__ __forceinline__ V3 nee_estimate(const SceneView& s, const WaveView& w, int pid) {
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
      if (fl & kFlagEnv) {
        if (!w.mis_occluded[pid]) Ld = Ld + sdiv(mul(fb, env_le(lt, s.envmaps, xyz(w.mis_d[pid]))) * fv.w, bpdf);
      } else {
        const float4 mh = w.mis_hit[pid];
        const int prim = __float_as_int(mh.w);  // primitive hit by the MIS ray, -1 for a miss
        const V3 wi = xyz(w.mis_d[pid]);
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
    return mul(xyz(pb), sdiv(Ld, np.w));
}

// One bounce of PathTracing::Li for the path in slot `pid`, whose material
// (if it hit one) holds only lobe kinds in KM; TEX: the material is textured.
// FRESH: at bounce 0 the path's throughput is 1 and its radiance 0, and its
// record does not hold them (plain waves: k_camera leaves them out).
// DEFER (plain waves): the light sample of the path's previous bounce is
// added to its radiance here, first, as a separate resolve pass would have
// added it before this bounce; this bounce's sample is left pending
// (kNeePending) for the next shading or, if the path ends, for k_film.
template <unsigned KM = kLobeAll, bool TEX = false, bool FRESH = false, bool DEFER = false>
__device__ __forceinline__ ShadeResult shade_one(const SceneView& s, const WaveView& w, const uint32_t* sobol,
                                                 int pid, uint64_t index, int bounce, int max_depth, int rr_depth) {
  LightDistrib distrib{s.light_func, s.light_cdf, s.light_func_int, s.num_lights};
    const float4 hv = w.hit[pid];
    const int prim = __float_as_int(hv.w);  // the trace stores the primitive, -1 for a miss
    const V3 ro = xyz(w.ray_o[pid]);
    const V3 rd = xyz(w.ray_d[pid]);
    const bool fresh = FRESH && bounce == 0;
    float4 b4 = fresh ? make_float4(1.f, 1.f, 1.f, 0.f) : w.beta[pid];
    V3 beta = xyz(b4);
    const bool spec_prev = b4.w != 0.f;
    const float4 L4 = fresh ? make_float4(0.f, 0.f, 0.f, 0.f) : w.L[pid];
    V3 L = xyz(L4);
    const int dimw = DEFER ? w.dim[pid] : 0;
    if (DEFER && (dimw & kNeePending)) L = L + nee_estimate(s, w, pid);

    // Emission on the first hit or after a specular bounce (path.cpp:61-69).
    if (bounce == 0 || spec_prev) {
      if (prim >= 0) {
        int li = __ldg(&s.prims[prim].light);
        if (li >= 0) {
          V3 ng = geometric_normal(s.prims[prim]);
          if (dot(ng, -rd) > 0.f) L = L + mul(beta, ld3(s.lights[li].L));
        }
      } else {
        for (int e = 0; e < s.num_env; ++e) L = L + mul(beta, env_le(s.lights[s.env_idx[e]], s.envmaps, rd));
      }
    }
    bool alive = prim >= 0 && bounce < max_depth;
    bool did_nee = false, want_sh = false, want_mis = false, want_mis_env = false;
    if (alive) {
      const PrimShade& sh = s.prims[prim];
      Hit h = reconstruct(sh, hv.y, hv.z);
      DevMaterial tm;  // a textured material's lobes at this hit
      const DevMaterial* mp = &s.mats[sh.material];
      if constexpr (TEX) {
        float x, y;
        hit_uv(s.prim_uv + 6 * (size_t)prim, hv.y, hv.z, &x, &y);
        textured_material(s, sh.material, x, y, &tm);
        mp = &tm;
      }
      const DevMaterial& m = *mp;
      Frame fr{h.ng, h.ns, h.su, h.sv};
      // This bounce consumes at most 8 sample dimensions (light choice 1,
      // light point 2, BSDF for MIS 2, continuation 2, roulette 1), drawn
      // together: their table lookups are independent.
      const uint32_t d0 = DEFER ? (uint32_t)(dimw & ~kNeePending) : (uint32_t)w.dim[pid];
      float u[8];
      sobol_dims<8>(sobol, index, d0, u);
      int used = 0;

      // uniformSampleOneLight (integrator.cpp:8-27) when a non-specular lobe exists.
      if (m.num_nonspecular > 0 && s.num_lights > 0) {
        float sel_pdf;
        int li = sample_discrete(distrib, u[0], &sel_pdf);
        used = 1;
        if (sel_pdf != 0.f) {
          used = 5;
          float ul1 = u[1], ul0 = u[2];  // next2(): .x is the later dimension
          float ub1 = u[3], ub0 = u[4];
          const DevLight& lt = s.lights[li];
          V3 wo = normalize(-rd);
          // estimateDirect, light-sampling half (integrator.cpp:39-60).
          LightSample ls = sample_li(lt, s.prims, s.envmaps, h.p, ul0, ul1, s.world_radius);
          V3 ld = V3{0, 0, 0};
          if (ls.pdf > 0.f && !is_black(ls.Li)) {
            V3 f = bsdf_f<KM>(m, fr, ls.wi, wo, kNonSpecular) * absdot(ls.wi, h.ns);
            float bpdf = bsdf_pdf<KM>(m, fr, ls.wi, wo, kNonSpecular);
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
            fb = bsdf_sample_f<KM>(m, fr, wo, ub0, ub1, kNonSpecular, &wib, &mis_pdf, &st);
            fb = fb * absdot(wib, h.ns);
            if (!is_black(fb) && mis_pdf > 0.f) {
              bool ok = true;
              if (lt.kind == DL_ENV) {
                float lpdf = env_pdf_li(lt, s.envmaps, wib);
                if (lpdf == 0.f)
                  ok = false;
                else {
                  env_w = power_heuristic(mis_pdf, lpdf);
                  flags |= kFlagEnv;
                }
              }
              if (ok) {
                // Towards an environment light only an escape counts, so that
                // ray is an occlusion query over (0, FLT_MAX] (tmax in o.w);
                // towards an area light the closest hit is needed.
                V3 mo = offset_ray_origin(h.p, h.ng, wib);
                const bool env = (flags & kFlagEnv) != 0;
                w.mis_o[pid] = f4(mo, env ? kFloatMax : 0.f);
                w.mis_d[pid] = f4(wib, 0.f);
                want_mis = !env;
                want_mis_env = env;
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
      float u1 = used == 0 ? u[0] : (used == 1 ? u[1] : u[5]);  // next2(): .x is the later dimension
      float u0 = used == 0 ? u[1] : (used == 1 ? u[2] : u[6]);
      used += 2;
      V3 wi;
      float pdf;
      int stype;
      V3 f = bsdf_sample_f<KM>(m, fr, -rd, u0, u1, BXDF_ALL, &wi, &pdf, &stype);
      if (is_black(f) || pdf == 0.f) {
        alive = false;
      } else {
        beta = mul(beta, sdiv(f * absdot(wi, h.ns), pdf));
        bool spec = (stype & BXDF_SPECULAR) != 0;
        V3 no = offset_ray_origin(h.p, h.ng, wi);
        if (bounce > rr_depth) {
          float qq = fmaxf(0.05f, 1.f - max_comp(beta));
          float rr = used == 2 ? u[2] : (used == 3 ? u[3] : u[7]);
          used += 1;
          if (rr < qq)
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
      w.dim[pid] = (int)(d0 + used) | (DEFER && did_nee ? kNeePending : 0);
    } else if (DEFER && (dimw & kNeePending)) {
      w.dim[pid] = dimw & ~kNeePending;  // added above
    }
    w.L[pid] = f4(L, L4.w);  // w holds batched mode's sample index bits
  return ShadeResult{alive, did_nee, want_sh, want_mis, want_mis_env};
}

// The scene a path slot traces against: one scene for a plain wave, the
// slot's job's scene in batched mode.
struct SingleScene {
  const SceneView* s;
  __device__ __forceinline__ const SceneView& operator()(int) const { return *s; }
};
struct JobScene {
  const DevJob* jobs;
  RecI job;
  __device__ __forceinline__ const SceneView& operator()(int pid) const { return jobs[job[pid]].scene; }
};

// Persistent-warp tracing of `n` queued rays (see traverse.cuh): warps stay
// in the kernel and refill idle lanes from the queue through `fetch`, a
// counter that must be zero at launch. Block size must be a multiple of 32.
// With `q_cls` (closest hit only), each finished ray's slot is also appended
// to the queue of the shading class of what it hit (SC_MISS for a miss), or,
// given `cls_flags`, that class's bit is set in the slot's byte there for a
// compaction pass to list the slots in slot order. COUNT adds the kernel's node visits to work[0] and its triangle tests to
// work[3]. A ray whose traversal overflowed its stack (capacity CAP) is
// reported as a miss (not occluded) and sets kErrTraversalStack in *err.
template <bool ANY, int SMEM, bool COUNT = false, int CAP = kMaxStack, class SceneOf, class RayView, class HitView>
__device__ __forceinline__ void trace_persistent(const SceneOf& scene_of, const int* queue, int n, int* fetch,
                                                 RayView ray_o, RayView ray_d, HitView hit, int* occluded,
                                                 int2* stack_smem, int refill_below, int* err,
                                                 int* cls_counters = nullptr, int* q_cls = nullptr,
                                                 int cls_stride = 0, unsigned long long* work = nullptr,
                                                 uint8_t* cls_flags = nullptr) {
  constexpr unsigned kFull = 0xffffffffu;
  constexpr bool kUniform = std::is_same<SceneOf, SingleScene>::value;
  const int lane = threadIdx.x & 31;
  TraversalStack<SMEM, CAP> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  TriScratch* tsc = reinterpret_cast<TriScratch*>(stack_smem + (size_t)SMEM * blockDim.x) + (threadIdx.x >> 5);
  LaneRay r;
  r.tg = make_uint2(0u, 0u);
  // Every lane may test triangles for the others (warp_triangles): with one
  // scene for all rays, a lane holds its arrays before its first ray.
  TraceScene ts{nullptr, nullptr, nullptr, nullptr};
  if constexpr (kUniform) {
    const SceneView& s0 = scene_of(0);
    ts = TraceScene{s0.nodes, s0.woop, s0.tri_prim, s0.tri_class};
  }
  int pid = -1;
  bool active = false, exhausted = false;
  TraceWork wk;
  while (true) {
    unsigned act = __ballot_sync(kFull, active);
    if (!exhausted && __popc(act) < refill_below) {
      const unsigned idle = ~act;
      const int cnt = __popc(idle);
      int base = 0;
      if (lane == 0) base = atomicAdd(fetch, cnt);
      base = __shfl_sync(kFull, base, 0);
      if (base + cnt >= n) exhausted = true;
      if (!active) {
        const int my = base + __popc(idle & ((1u << lane) - 1u));
        if (my < n) {
          pid = queue[my];
          const SceneView& s = scene_of(pid);
          ts = TraceScene{s.nodes, s.woop, s.tri_prim, s.tri_class};
          // The ray and its result pass through once: streaming (evict-first) accesses
          // leave L1 and L2 to the BVH nodes and triangles (displaced sphere +1.2%).
          const float4 o4 = __ldcs(&ray_o[pid]), d4 = __ldcs(&ray_d[pid]);
          st.sp = 0;
          lane_start(r, o4, d4, ANY ? o4.w : kFloatMax, ANY);
          active = true;
        }
      }
      act = __ballot_sync(kFull, active);
    }
    if (act == 0) {
      if (exhausted) break;
      continue;
    }
    if (active) lane_visit<ANY, SMEM, COUNT, CAP>(r, ts, st, &wk);
    const bool occl = warp_triangles<ANY, COUNT, kUniform>(r, ts, tsc, &wk);
    if (active) {
      if ((ANY && occl) || lane_pop(r, st)) {
        if constexpr (CAP < kMaxStack) {
          if (r.tmax < 0.f) {  // poisoned by a stack overflow
            r.tri = -1;
            atomicOr(err, kErrTraversalStack);
          }
        }
        if (ANY) {
          __stcs(&occluded[pid], r.tri >= 0 ? 1 : 0);
        } else {
          __stcs(&hit[pid], make_float4(r.tri >= 0 ? r.tmax : kFloatMax, r.u, r.v,
                                        __int_as_float(r.tri >= 0 ? __ldg(ts.tri_prim + r.tri) : -1)));
          if (q_cls) {
            const int cls = r.tri >= 0 ? (int)__ldg(ts.tri_class + r.tri) : SC_MISS;
            if (cls_flags)
              cls_flags[pid] = (uint8_t)(1u << cls);
            else
              class_append(cls_counters, q_cls, cls_stride, cls, pid);
          }
        }
        active = false;
      }
    }
  }
  if (COUNT) {  // the loop ends for the whole warp at once (act and exhausted are warp-uniform)
    for (int o = 16; o > 0; o >>= 1) {
      wk.nodes += __shfl_down_sync(kFull, wk.nodes, o);
      wk.tris += __shfl_down_sync(kFull, wk.tris, o);
    }
    if (lane == 0) {
      atomicAdd(work, wk.nodes);
      atomicAdd(work + 3, wk.tris);
    }
  }
}

// Lists slots in queues from their qflags bytes: bit b of a slot's byte puts
// the slot in queue b. The slots looked at are list[0 .. *count) (the bounce's
// extension queue: every slot traced and shaded this bounce), so the cost
// follows the live paths, not the wave. Blocks of kCompactThreads threads take
// spans of kCompactSpan list entries in turn: list order within a span (a
// block reserves its part of each queue with one atomicAdd, so spans land in
// any order), and the list is itself in slot order span by span, so the
// queues come out in slot order too. The bytes are cleared for the next pass.
// Used twice a bounce: the extension trace marks each slot's shading class
// (one queue per class), and the shading marks the queues a path goes to next.
constexpr int kCompactItems = 16, kCompactThreads = 256, kCompactSpan = kCompactItems * kCompactThreads;

struct CompactTargets {
  int* queue[8];
  int* counter[8];
};

template <int NQ>
__device__ __forceinline__ void compact_queues(uint8_t* flags, const int* list, const int* count,
                                               const CompactTargets& tg) {
  __shared__ int s_warp[kCompactThreads / 32][NQ];
  __shared__ int s_base[NQ];
  const int t = threadIdx.x, lane = t & 31, wid = t >> 5;
  const int n = *count;
  for (int span = blockIdx.x; span * kCompactSpan < n; span += gridDim.x) {
    const int p0 = span * kCompactSpan + t * kCompactItems;
    int slot[kCompactItems];
    uint32_t words[4] = {0u, 0u, 0u, 0u};
    if (p0 + kCompactItems <= n) {  // p0 is a multiple of 16: four aligned 16-byte loads of the list
      const int4* l4 = reinterpret_cast<const int4*>(list + p0);
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const int4 v = l4[k];
        slot[4 * k] = v.x, slot[4 * k + 1] = v.y, slot[4 * k + 2] = v.z, slot[4 * k + 3] = v.w;
      }
    } else {
#pragma unroll
      for (int j = 0; j < kCompactItems; ++j) slot[j] = p0 + j < n ? list[p0 + j] : -1;
    }
#pragma unroll
    for (int j = 0; j < kCompactItems; ++j)
      if (slot[j] >= 0) {
        const uint32_t f = flags[slot[j]];
        if (f) {
          words[j >> 2] |= f << (8 * (j & 3));
          flags[slot[j]] = 0;
        }
      }
    if (!__syncthreads_or((words[0] | words[1] | words[2] | words[3]) != 0u)) continue;
    int off[NQ];
#pragma unroll
    for (int b = 0; b < NQ; ++b) {
      int c = 0;
#pragma unroll
      for (int k = 0; k < 4; ++k) c += __popc(words[k] & (0x01010101u << b));
      int x = c;  // inclusive scan over the warp
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
      }
      off[b] = x - c;
      if (lane == 31) s_warp[wid][b] = x;
    }
    __syncthreads();
    if (t < NQ) {
      int total = 0;
      for (int k = 0; k < kCompactThreads / 32; ++k) {
        const int c = s_warp[k][t];
        s_warp[k][t] = total;
        total += c;
      }
      s_base[t] = total ? atomicAdd(tg.counter[t], total) : 0;
    }
    __syncthreads();
#pragma unroll
    for (int b = 0; b < NQ; ++b) {
      int o = s_base[b] + s_warp[wid][b] + off[b];
      int* q = tg.queue[b];
#pragma unroll
      for (int j = 0; j < kCompactItems; ++j)
        if ((words[j >> 2] >> (8 * (j & 3) + b)) & 1u) q[o++] = slot[j];
    }
    __syncthreads();  // s_warp and s_base are reused by the block's next span
  }
}

// Adds beta * Ld / selPdf for a path that sampled a light this bounce
// (path.cpp:77-80 with the shadow and MIS rays traced).
__device__ __forceinline__ void resolve_one(const SceneView& s, const WaveView& w, int pid) {
  const float4 L4 = w.L[pid];
  w.L[pid] = f4(xyz(L4) + nee_estimate(s, w, pid), L4.w);
}

}  // namespace orion_gb300
