// Stochastic progressive photon mapping (SPPM::render,
// src/integrator/sppm.cpp:58-322) on the GPU.
//
// One iteration is
//   k_sppm_camera    one thread per pixel: the camera path up to its first
//                    diffuse (or last glossy) hit, direct light at every hit
//                    (uniformSampleOneLight with uniform light choice,
//                    src/core/integrator.cpp:8-27), the visible point kept
//   k_sppm_bounds    bounds of the visible points' spheres, block partials
//   k_sppm_grid      the grid resolution (sppm.cpp:145-160)
//   k_sppm_photons   one thread per photon: Light::sample_Le, then a photon
//                    path with TransportMode::Photon BSDFs and throughput
//                    roulette; every hit after the first that falls inside
//                    the grid is recorded (point, wi, beta) and counted in
//                    its hash cell
//   k_scan_*         exclusive scan: each hash cell's first list entry
//   k_sppm_fill      the photon hits copied into hash-cell order
//   k_sppm_gather    one warp per visible point: for each hash cell its
//                    sphere overlaps, the recorded photons in that cell
//                    within its radius add beta * f(wi, wo) (sppm.cpp:226-247)
//   k_sppm_update    radius / N / tau update and the film (sppm.cpp:272-320)
// The reference walks, per photon hit, the visible points listed in the hit's
// hash cell; here each visible point walks the photon hits listed in the hash
// cells of its own sphere. Both consider a (visible point, photon) pair once
// per cell of the sphere whose hash equals the hash of the photon's cell, so
// the sums have the same terms; only their order differs. A visible point's
// material and frame are loaded once, and no flux atomics are needed.
// Paths and photons trace with the per-thread 8-wide traversal
// (traverse.cuh); the per-pixel and per-photon loops are short and their
// bounce counts vary, so a thread follows its own path to the end.
//
// Sample indices and dimensions follow the reference: the camera path of
// pixel (i, j) in iteration k uses index k*W*H + j*W + i, photon p uses
// iterations*W*H + k*photons + p, each from dimension 5.
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"
#include "shade.cuh"

namespace orion_gb300 {

namespace {

constexpr int kSppmBlock = 128;
constexpr int kSppmStack = 8;  // shared-memory traversal stack entries per thread

__device__ __forceinline__ void count_rays(unsigned long long* ctr, unsigned n) {
  const unsigned mask = __activemask();
  const unsigned total = __reduce_add_sync(mask, n);
  if ((int)(threadIdx.x & 31) == __ffs(mask) - 1) atomicAdd(ctr, (unsigned long long)total);
}

// The lobes of material `mi` at texture coordinates (x, y): the scene's
// record, or built at the hit for a textured material.
__device__ __forceinline__ const DevMaterial* material_at(const SceneView& s, int mi, float x, float y,
                                                          DevMaterial* tm) {
  if (s.mats[mi].shade_class != SC_TEXTURED) return &s.mats[mi];
  textured_material(s, mi, x, y, tm);
  return tm;
}

__device__ __forceinline__ int count_matching(const DevMaterial& m, int t) {
  int n = 0;
  for (int i = 0; i < m.num_lobes; ++i) n += (m.lobes[i].type & t) == m.lobes[i].type ? 1 : 0;
  return n;
}

// uniformSampleOneLight without a light distribution (integrator.cpp:8-27):
// the light chosen uniformly, estimateDirect (integrator.cpp:29-90) with
// its shadow and MIS rays traced here; returns estimateDirect / lightPdf.
template <int SMEM>
__device__ V3 sppm_direct(const SceneView& s, const TraceScene& ts, TraversalStack<SMEM>& st, const DevMaterial& m,
                          const Frame& fr, const Hit& h, V3 rd, PathSampler& smp, unsigned* rays) {
  const int n = s.num_lights;
  if (n == 0) return V3{0, 0, 0};
  const int li = min((int)(smp.next() * n), n - 1);
  const float light_pdf = 1.f / n;
  const float a = smp.next(), b = smp.next(), c = smp.next(), d = smp.next();  // next2(): .x is the later one
  const DevLight& lt = s.lights[li];
  const V3 wo = normalize(-rd);
  V3 Ld = V3{0, 0, 0};
  const LightSample ls = sample_li(lt, s.prims, s.envmaps, h.p, b, a, s.world_radius);
  if (ls.pdf > 0.f && !is_black(ls.Li)) {
    const V3 f = bsdf_f<kLobeAll>(m, fr, ls.wi, wo, kNonSpecular) * absdot(ls.wi, h.ns);
    const float bpdf = bsdf_pdf<kLobeAll>(m, fr, ls.wi, wo, kNonSpecular);
    if (!is_black(f)) {
      // ShadowTester::unoccluded (light.h:26-29): Intersection::spawnRay to a point.
      const V3 so = offset_ray_origin(h.p, h.ng, ls.p_light - h.p);
      ++*rays;
      if (traverse<true, SMEM>(ts, so, ls.p_light - so, 0.f, 1.f - kShadowEpsilon, st).tri < 0) {
        if (is_delta_light(lt.kind))
          Ld = sdiv(mul(f, ls.Li), ls.pdf);
        else
          Ld = sdiv(mul(f, ls.Li) * power_heuristic(ls.pdf, bpdf), ls.pdf);
      }
    }
  }
  if (!is_delta_light(lt.kind)) {
    V3 wib;
    float mis_pdf = 0.f;
    int stype;
    V3 fb = bsdf_sample_f<kLobeAll>(m, fr, wo, d, c, kNonSpecular, &wib, &mis_pdf, &stype);
    fb = fb * absdot(wib, h.ns);
    if (!is_black(fb) && mis_pdf > 0.f) {
      const V3 mo = offset_ray_origin(h.p, h.ng, wib);
      if (lt.kind == DL_ENV) {
        const float lpdf = env_pdf_li(lt, s.envmaps, wib);
        if (lpdf != 0.f) {
          const float wgt = power_heuristic(mis_pdf, lpdf);
          ++*rays;
          if (traverse<true, SMEM>(ts, mo, wib, 0.f, kFloatMax, st).tri < 0)
            Ld = Ld + sdiv(mul(fb, env_le(lt, s.envmaps, wib)) * wgt, mis_pdf);
        }
      } else {
        ++*rays;
        const RayHit mh = traverse<false, SMEM>(ts, mo, wib, 0.f, kFloatMax, st);
        const int prim = mh.tri >= 0 ? __ldg(ts.tri_prim + mh.tri) : -1;
        if (prim >= 0 && prim == lt.prim) {
          // Triangle::pdf (src/core/triangle.cpp:123-135) on the traced hit.
          const PrimShade& sh = s.prims[prim];
          const V3 ip = point_on(sh, mh.u, mh.v);
          const V3 ing = geometric_normal(sh);
          float lpdf = length_sq(h.p - ip) / (absdot(ing, -wib) * lt.area);
          if (isinf(lpdf)) lpdf = 0.f;
          if (lpdf != 0.f) {
            const float wgt = power_heuristic(mis_pdf, lpdf);
            const V3 Li = dot(ing, -wib) > 0.f ? ld3(lt.L) : V3{0, 0, 0};
            if (!is_black(Li)) Ld = Ld + sdiv(mul(fb, Li) * wgt, mis_pdf);
          }
        }
      }
    }
  }
  return sdiv(Ld, light_pdf);
}

// Visible points (sppm.cpp:78-140).
template <int SMEM>
__global__ void __launch_bounds__(kSppmBlock) k_sppm_camera(SceneView s, SppmView v, int iter) {
  extern __shared__ int2 stack_smem[];
  TraversalStack<SMEM> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= v.npix) return;
  const TraceScene ts = trace_scene(s);
  const int i = pix % v.width, j = pix / v.width;
  PathSampler smp{v.sobol, (uint64_t)iter * v.npix + (uint64_t)v.width * j + i, 5u};
  V3 o, d;
  camera_ray(s.cam, smp, i, j, &o, &d);
  V3 beta = V3{1.f, 1.f, 1.f};
  bool specular = false;
  const float4 ld4 = v.ld[pix];
  V3 Ld = xyz(ld4);
  unsigned rays = 0;
  int vp_mat = -1;
  for (int depth = 0; depth < v.max_depth; ++depth) {
    ++rays;
    const RayHit rh = traverse<false, SMEM>(ts, o, d, 0.f, kFloatMax, st);
    if (rh.tri < 0) {
      for (int e = 0; e < s.num_env; ++e) Ld = Ld + mul(beta, env_le(s.lights[s.env_idx[e]], s.envmaps, d));
      break;
    }
    const int prim = __ldg(ts.tri_prim + rh.tri);
    const PrimShade& sh = s.prims[prim];
    const Hit h = reconstruct(sh, rh.u, rh.v);
    const int mi = sh.material;
    float tu = 0.f, tv = 0.f;
    if (s.prim_uv) hit_uv(s.prim_uv + 6 * (size_t)prim, rh.u, rh.v, &tu, &tv);
    DevMaterial tm;
    const DevMaterial& m = *material_at(s, mi, tu, tv, &tm);
    const Frame fr{h.ng, h.ns, h.su, h.sv};
    const V3 wo = -d;
    if (depth == 0 || specular) {
      const int li = sh.light;
      if (li >= 0 && dot(h.ng, wo) > 0.f) Ld = Ld + mul(beta, ld3(s.lights[li].L));
    }
    Ld = Ld + mul(beta, sppm_direct<SMEM>(s, ts, st, m, fr, h, d, smp, &rays));
    const bool diffuse = count_matching(m, BXDF_DIFFUSE | BXDF_REFLECTION | BXDF_TRANSMISSION) > 0;
    const bool glossy = count_matching(m, BXDF_GLOSSY | BXDF_REFLECTION | BXDF_TRANSMISSION) > 0;
    if (diffuse || (glossy && depth == v.max_depth - 1)) {
      if (!is_black(beta)) {
        vp_mat = mi;
        v.vp_pr[pix] = f4(h.p, v.vp_pr[pix].w);
        v.vp_wo[pix] = f4(wo, __int_as_float(mi));
        v.vp_beta[pix] = f4(beta, tu);
        v.vp_ns[pix] = f4(h.ns, tv);
        v.vp_ng[pix] = f4(h.ng, 0.f);
        v.vp_su[pix] = f4(h.su, 0.f);
        v.vp_sv[pix] = f4(h.sv, 0.f);
      }
      break;
    }
    if (depth < v.max_depth - 1) {
      const float a = smp.next(), b = smp.next();
      V3 wi;
      float pdf = 0.f;
      int stype = 0;
      const V3 f = bsdf_sample_f<kLobeAll>(m, fr, wo, b, a, BXDF_ALL, &wi, &pdf, &stype);
      if (pdf == 0.f || is_black(f)) break;
      specular = (stype & BXDF_SPECULAR) != 0;
      beta = mul(beta, sdiv(f * absdot(wi, h.ns), pdf));
      const float y = spectrum_intensity(beta);
      if (y < 0.25f) {
        const float cont = fminf(1.f, y);
        if (smp.next() > cont) break;
        beta = sdiv(beta, cont);
      }
      o = offset_ray_origin(h.p, h.ng, wi);
      d = wi;
    }
  }
  v.ld[pix] = f4(Ld, ld4.w);
  if (vp_mat < 0) v.vp_wo[pix].w = __int_as_float(-1);
  count_rays(v.rays, rays);
}

__device__ __forceinline__ bool has_vp(const SppmView& v, int pix) { return __float_as_int(v.vp_wo[pix].w) >= 0; }

// Bounds of every visible point's sphere and the largest radius: one
// partial per block.
__global__ void __launch_bounds__(256) k_sppm_bounds(SppmView v) {
  __shared__ float red[8][256];
  float lo[3] = {kFloatMax, kFloatMax, kFloatMax}, hi[3] = {-kFloatMax, -kFloatMax, -kFloatMax}, mr = 0.f, any = 0.f;
  for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < v.npix; pix += gridDim.x * blockDim.x) {
    if (!has_vp(v, pix)) continue;
    const float4 pr = v.vp_pr[pix];
    const float p[3] = {pr.x, pr.y, pr.z};
    for (int k = 0; k < 3; ++k) {
      const float a = p[k] - pr.w, b = p[k] + pr.w;  // expand(Bounds3f(p), radius)
      lo[k] = a < lo[k] ? a : lo[k];
      hi[k] = b > hi[k] ? b : hi[k];
    }
    mr = pr.w > mr ? pr.w : mr;
    any = 1.f;
  }
  const int t = threadIdx.x;
  red[0][t] = lo[0], red[1][t] = lo[1], red[2][t] = lo[2];
  red[3][t] = hi[0], red[4][t] = hi[1], red[5][t] = hi[2];
  red[6][t] = mr, red[7][t] = any;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      for (int k = 0; k < 3; ++k) red[k][t] = fminf(red[k][t], red[k][t + w]);
      for (int k = 3; k < 8; ++k) red[k][t] = fmaxf(red[k][t], red[k][t + w]);
    }
    __syncthreads();
  }
  if (t == 0) {
    v.part_lo[blockIdx.x] = make_float4(red[0][0], red[1][0], red[2][0], red[6][0]);
    v.part_hi[blockIdx.x] = make_float4(red[3][0], red[4][0], red[5][0], red[7][0]);
  }
}

// The grid over the visible points (sppm.cpp:145-160), from the partials.
__global__ void __launch_bounds__(256) k_sppm_grid(SppmView v, int nparts) {
  __shared__ float red[8][256];
  const int t = threadIdx.x;
  float r[8] = {kFloatMax, kFloatMax, kFloatMax, -kFloatMax, -kFloatMax, -kFloatMax, 0.f, 0.f};
  for (int b = t; b < nparts; b += blockDim.x) {
    const float4 l = v.part_lo[b], h = v.part_hi[b];
    r[0] = fminf(r[0], l.x), r[1] = fminf(r[1], l.y), r[2] = fminf(r[2], l.z);
    r[3] = fmaxf(r[3], h.x), r[4] = fmaxf(r[4], h.y), r[5] = fmaxf(r[5], h.z);
    r[6] = fmaxf(r[6], l.w), r[7] = fmaxf(r[7], h.w);
  }
  for (int k = 0; k < 8; ++k) red[k][t] = r[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (t < w) {
      for (int k = 0; k < 3; ++k) red[k][t] = fminf(red[k][t], red[k][t + w]);
      for (int k = 3; k < 8; ++k) red[k][t] = fmaxf(red[k][t], red[k][t + w]);
    }
    __syncthreads();
  }
  if (t == 0) {
    SppmGrid g;
    for (int k = 0; k < 3; ++k) {
      g.lo[k] = red[k][0];
      g.hi[k] = red[k + 3][0];
    }
    g.max_radius = red[6][0];
    g.any = red[7][0] != 0.f;
    g.res[0] = g.res[1] = g.res[2] = 1;
    if (g.any) {
      const float diag[3] = {g.hi[0] - g.lo[0], g.hi[1] - g.lo[1], g.hi[2] - g.lo[2]};
      const float max_diag = fmaxf(diag[0], fmaxf(diag[1], diag[2]));
      const int base = __float2int_rz(max_diag / g.max_radius);
      for (int k = 0; k < 3; ++k) g.res[k] = max(__float2int_rz(__fmul_rn((float)base, diag[k]) / max_diag), 1);
    }
    *v.grid = g;
  }
}

// ToGrid (sppm.cpp:41-51): Bounds3::offset, then the truncated cell, clamped.
__device__ __forceinline__ bool to_grid(const SppmGrid& g, V3 p, int* c) {
  float o[3] = {p.x - g.lo[0], p.y - g.lo[1], p.z - g.lo[2]};
  bool in = true;
  for (int k = 0; k < 3; ++k) {
    if (g.hi[k] > g.lo[k]) o[k] = o[k] / (g.hi[k] - g.lo[k]);
    int ck = __float2int_rz(__fmul_rn((float)g.res[k], o[k]));
    in = in && ck >= 0 && ck < g.res[k];
    c[k] = min(max(ck, 0), g.res[k] - 1);
  }
  return in;
}

// hash (sppm.cpp:53-57), the products modulo 2^32.
__device__ __forceinline__ unsigned cell_hash(int x, int y, int z, int size) {
  return (((unsigned)x * 73856093u) ^ ((unsigned)y * 19349663u) ^ ((unsigned)z * 83492791u)) % (unsigned)size;
}

// Copies the recorded photon hits into hash-cell order (cell_start holds
// each cell's first entry after the scan), so a gather reads a cell's hits
// from consecutive records.
__global__ void __launch_bounds__(256) k_sppm_fill(SppmView v) {
  const int n = min(*v.hit_count, v.hits_cap);
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4* src = v.hits + 3 * (size_t)i;
    const float4 a = src[0], b = src[1], c = src[2];
    const unsigned h = (unsigned)__float_as_int(a.w);
    float4* dst = v.by_cell + 3 * (size_t)(v.cell_start[h] + atomicAdd(v.cell_fill + h, 1));
    dst[0] = a;
    dst[1] = b;
    dst[2] = c;
  }
}

// Photon flux at each visible point (sppm.cpp:226-247, seen from the visible
// point): the cells its sphere overlaps (sppm.cpp:167-190), the photon hits
// listed under each cell's hash, those within the radius. One warp per
// visible point: the lanes take a cell's hits in turn, so every lane runs the
// same material's BSDF, and the lanes' sums are added at the end. Eight
// blocks per SM (64 registers, a few spilled to L1): 3% faster than 80
// registers at five blocks, the kernel waits on its L2 gathers.
__global__ void __launch_bounds__(128, 8) k_sppm_gather(SceneView s, SppmView v) {
  const int pix = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (pix >= v.npix || !has_vp(v, pix)) return;  // uniform across the warp
  const SppmGrid g = *v.grid;
  const float4 pr = v.vp_pr[pix], wo4 = v.vp_wo[pix], b4 = v.vp_beta[pix], ns4 = v.vp_ns[pix];
  const V3 p = xyz(pr), wo = xyz(wo4), r = V3{pr.w, pr.w, pr.w};
  const float rr = pr.w * pr.w;
  DevMaterial vm;
  const DevMaterial& m = *material_at(s, __float_as_int(wo4.w), b4.w, ns4.w, &vm);
  const Frame fr{xyz(v.vp_ng[pix]), xyz(ns4), xyz(v.vp_su[pix]), xyz(v.vp_sv[pix])};
  int lo[3], hi[3];
  to_grid(g, p - r, lo);
  to_grid(g, p + r, hi);
  V3 phi = V3{0, 0, 0};
  int count = 0;
  for (int z = lo[2]; z <= hi[2]; ++z)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int x = lo[0]; x <= hi[0]; ++x) {
        const unsigned h = cell_hash(x, y, z, v.npix);
        const int e1 = v.cell_start[h + 1];
        for (int e = v.cell_start[h] + lane; e < e1; e += 32) {
          const float4* rec = v.by_cell + 3 * (size_t)e;
          const float4 hp = rec[0];
          if (length_sq(p - xyz(hp)) > rr) continue;
          const float4 wi4 = rec[1], hb = rec[2];
          phi = phi + mul(xyz(hb), bsdf_f<kLobeAll>(m, fr, xyz(wi4), wo, BXDF_ALL));
          ++count;
        }
      }
  for (int off = 16; off > 0; off >>= 1) {
    phi.x += __shfl_xor_sync(0xffffffffu, phi.x, off);
    phi.y += __shfl_xor_sync(0xffffffffu, phi.y, off);
    phi.z += __shfl_xor_sync(0xffffffffu, phi.z, off);
    count += __shfl_xor_sync(0xffffffffu, count, off);
  }
  if (lane == 0) {
    float* ph = v.phi + 3 * (size_t)pix;
    ph[0] = phi.x;
    ph[1] = phi.y;
    ph[2] = phi.z;
    v.m[pix] = count;
  }
}

// Exclusive scan of n ints in place: per-block scans, a scan of the block
// sums, and the block offsets added back.
__global__ void __launch_bounds__(kScanBlock) k_scan_blocks(int* a, int n, int* part) {
  __shared__ int buf[kScanBlock];
  const int t = threadIdx.x, i = blockIdx.x * kScanBlock + t;
  const int x = i < n ? a[i] : 0;
  buf[t] = x;
  __syncthreads();
  for (int off = 1; off < kScanBlock; off <<= 1) {
    const int y = t >= off ? buf[t - off] : 0;
    __syncthreads();
    buf[t] += y;
    __syncthreads();
  }
  if (i < n) a[i] = buf[t] - x;
  if (t == kScanBlock - 1) part[blockIdx.x] = buf[t];
}

__global__ void __launch_bounds__(kScanBlock) k_scan_parts(int* part, int nparts) {
  __shared__ int buf[kScanBlock];
  __shared__ int carry;
  const int t = threadIdx.x;
  if (t == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < nparts; base += kScanBlock) {
    const int i = base + t;
    const int x = i < nparts ? part[i] : 0;
    buf[t] = x;
    __syncthreads();
    for (int off = 1; off < kScanBlock; off <<= 1) {
      const int y = t >= off ? buf[t - off] : 0;
      __syncthreads();
      buf[t] += y;
      __syncthreads();
    }
    if (i < nparts) part[i] = carry + buf[t] - x;
    __syncthreads();
    if (t == kScanBlock - 1) carry += buf[t];
    __syncthreads();
  }
}

__global__ void __launch_bounds__(kScanBlock) k_scan_add(int* a, int n, const int* part) {
  const int i = blockIdx.x * kScanBlock + threadIdx.x;
  if (i < n) a[i] += part[blockIdx.x];
}

// Photons (sppm.cpp:197-270). Eight blocks per SM (64 registers): 3% faster
// than 96 registers; the camera pass loses at any bound below 128.
template <int SMEM>
__global__ void __launch_bounds__(kSppmBlock, 8) k_sppm_photons(SceneView s, SppmView v, int iter) {
  extern __shared__ int2 stack_smem[];
  TraversalStack<SMEM> st;
  st.smem = stack_smem + threadIdx.x;
  st.stride = blockDim.x;
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= v.photons) return;
  const SppmGrid g = *v.grid;
  if (!g.any) return;
  const TraceScene ts = trace_scene(s);
  PathSampler smp{v.sobol, (uint64_t)v.iterations * v.npix + (uint64_t)iter * v.photons + (uint64_t)k, 5u};
  const LightDistrib distrib{s.light_func, s.light_cdf, s.light_func_int, s.num_lights};
  float light_pdf;
  const int ln = sample_discrete(distrib, smp.next(), &light_pdf);
  const float a = smp.next(), b = smp.next(), c = smp.next(), d = smp.next();  // next2(): .x is the later one
  const EmittedRay e = sample_le(s.lights[ln], s.prims, s.envmaps, s.world_center, s.world_radius, b, a, d, c);
  if (e.pdf_pos == 0.f || e.pdf_dir == 0.f || is_black(e.Le)) return;
  V3 beta = sdiv(absdot(e.n, e.d) * e.Le, light_pdf * e.pdf_pos * e.pdf_dir);
  if (is_black(beta)) return;
  V3 o = e.o, dir = e.d;
  unsigned rays = 0;
  for (int depth = 0; depth < v.max_depth; ++depth) {
    ++rays;
    const RayHit rh = traverse<false, SMEM>(ts, o, dir, 0.f, kFloatMax, st);
    if (rh.tri < 0) break;
    const int prim = __ldg(ts.tri_prim + rh.tri);
    const PrimShade& sh = s.prims[prim];
    const Hit h = reconstruct(sh, rh.u, rh.v);
    if (depth > 0) {  // recorded for the gather when inside the grid (sppm.cpp:226-229)
      int cell[3];
      const bool in = to_grid(g, h.p, cell);
      const unsigned hc = in ? cell_hash(cell[0], cell[1], cell[2], v.npix) : 0u;
      const unsigned act = __activemask();
      const unsigned want = __ballot_sync(act, in);
      if (in) {
        const int lane = threadIdx.x & 31, leader = __ffs(want) - 1;
        int base = 0;
        if (lane == leader) base = atomicAdd(v.hit_count, __popc(want));
        base = __shfl_sync(want, base, leader);
        const int slot = base + __popc(want & ((1u << lane) - 1u));
        if (slot < v.hits_cap) {
          float4* rec = v.hits + 3 * (size_t)slot;
          rec[0] = f4(h.p, __int_as_float((int)hc));
          rec[1] = f4(-dir, 0.f);
          rec[2] = f4(beta, 0.f);
          atomicAdd(v.cell_start + hc, 1);
        }
      }
    }
    // Intersection::calculateBSDF(TransportMode::Photon)
    const int mi = sh.material;
    float tu = 0.f, tv = 0.f;
    if (s.prim_uv) hit_uv(s.prim_uv + 6 * (size_t)prim, rh.u, rh.v, &tu, &tv);
    DevMaterial pm;
    if (s.mats[mi].shade_class == SC_TEXTURED)
      textured_material(s, mi, tu, tv, &pm);
    else
      pm = s.mats[mi];
    for (int l = 0; l < pm.num_lobes; ++l) pm.lobes[l].photon = 1;
    const Frame fr{h.ng, h.ns, h.su, h.sv};
    const float u1 = smp.next(), u0 = smp.next();
    V3 wi;
    float pdf = 0.f;
    int stype = 0;
    const V3 f = bsdf_sample_f<kLobeAll>(pm, fr, -dir, u0, u1, BXDF_ALL, &wi, &pdf, &stype);
    if (is_black(f) || pdf == 0.f) break;
    const V3 bnew = sdiv(mul(beta, f) * absdot(wi, h.ns), pdf);
    const float q = fmaxf(0.f, 1.f - spectrum_intensity(bnew) / spectrum_intensity(beta));
    if (smp.next() < q) break;
    beta = sdiv(bnew, 1.f - q);
    o = offset_ray_origin(h.p, h.ng, wi);
    dir = wi;
  }
  count_rays(v.rays, rays);
}

// Pixel update and film (sppm.cpp:272-320), in the reference's operation
// order without contraction.
__global__ void __launch_bounds__(256) k_sppm_update(SppmView v) {
  const int pix = blockIdx.x * blockDim.x + threadIdx.x;
  if (pix >= v.npix) return;
  float4 pr = v.vp_pr[pix];
  float4 ld4 = v.ld[pix];
  float4 tau4 = v.tau[pix];
  const int M = v.m[pix];
  if (M > 0) {
    const float gamma = 2.f / 3.f;
    const float N = ld4.w, r = pr.w;
    const float n_new = __fadd_rn(N, __fmul_rn(gamma, (float)M));
    const float r_new = __fmul_rn(r, __fsqrt_rn(__fdiv_rn(n_new, __fadd_rn(N, (float)M))));
    const float4 b4 = v.vp_beta[pix];
    const float* ph = v.phi + 3 * (size_t)pix;
    const float rr_new = __fmul_rn(r_new, r_new), rr = __fmul_rn(r, r);
    tau4.x = __fdiv_rn(__fmul_rn(__fadd_rn(tau4.x, __fmul_rn(b4.x, ph[0])), rr_new), rr);
    tau4.y = __fdiv_rn(__fmul_rn(__fadd_rn(tau4.y, __fmul_rn(b4.y, ph[1])), rr_new), rr);
    tau4.z = __fdiv_rn(__fmul_rn(__fadd_rn(tau4.z, __fmul_rn(b4.z, ph[2])), rr_new), rr);
    ld4.w = n_new;
    pr.w = r_new;
    v.m[pix] = 0;
    v.phi[3 * (size_t)pix] = v.phi[3 * (size_t)pix + 1] = v.phi[3 * (size_t)pix + 2] = 0.f;
    v.vp_pr[pix] = pr;
    v.ld[pix] = ld4;
    v.tau[pix] = tau4;
  }
  v.vp_wo[pix].w = __int_as_float(-1);  // the visible point is cleared
  const float np = (float)((unsigned long long)v.iterations * (unsigned long long)v.photons);
  const float den = __fmul_rn(__fmul_rn(__fmul_rn(np, kPi), pr.w), pr.w);
  const float fi = (float)v.iterations;
  float* f = v.film + 3 * (size_t)pix;
  f[0] = __fadd_rn(f[0], __fadd_rn(__fdiv_rn(ld4.x, fi), __fdiv_rn(tau4.x, den)));
  f[1] = __fadd_rn(f[1], __fadd_rn(__fdiv_rn(ld4.y, fi), __fdiv_rn(tau4.y, den)));
  f[2] = __fadd_rn(f[2], __fadd_rn(__fdiv_rn(ld4.z, fi), __fdiv_rn(tau4.z, den)));
  v.film_count[pix] += 1u;
}

__global__ void k_sppm_init(SppmView v, float radius0) {
  for (int pix = blockIdx.x * blockDim.x + threadIdx.x; pix < v.npix; pix += gridDim.x * blockDim.x) {
    v.vp_pr[pix] = make_float4(0.f, 0.f, 0.f, radius0);
    v.vp_wo[pix] = make_float4(0.f, 0.f, 0.f, __int_as_float(-1));
    v.ld[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
    v.tau[pix] = make_float4(0.f, 0.f, 0.f, 0.f);
    v.phi[3 * (size_t)pix] = v.phi[3 * (size_t)pix + 1] = v.phi[3 * (size_t)pix + 2] = 0.f;
    v.m[pix] = 0;
    v.film[3 * (size_t)pix] = v.film[3 * (size_t)pix + 1] = v.film[3 * (size_t)pix + 2] = 0.f;
    v.film_count[pix] = 0u;
  }
}

int blocks_for(int64_t n, int block) { return (int)((n + block - 1) / block); }

}  // namespace

void launch_sppm_init(const SppmView& v, float radius0, cudaStream_t stream) {
  k_sppm_init<<<std::min(blocks_for(v.npix, 256), 4096), 256, 0, stream>>>(v, radius0);
}

void launch_sppm_visible_points(const SceneView& s, const SppmView& v, int iter, cudaStream_t stream) {
  const size_t smem = (size_t)kSppmStack * kSppmBlock * sizeof(int2);
  k_sppm_camera<kSppmStack><<<blocks_for(v.npix, kSppmBlock), kSppmBlock, smem, stream>>>(s, v, iter);
  k_sppm_bounds<<<kSppmBoundsBlocks, 256, 0, stream>>>(v);
  k_sppm_grid<<<1, 256, 0, stream>>>(v, kSppmBoundsBlocks);
}

void launch_sppm_scan(const SppmView& v, cudaStream_t stream) {
  const int n = v.npix + 1;
  const int nb = blocks_for(n, kScanBlock);
  k_scan_blocks<<<nb, kScanBlock, 0, stream>>>(v.cell_start, n, v.scan_part);
  k_scan_parts<<<1, kScanBlock, 0, stream>>>(v.scan_part, nb);
  k_scan_add<<<nb, kScanBlock, 0, stream>>>(v.cell_start, n, v.scan_part);
}

void launch_sppm_photons(const SceneView& s, const SppmView& v, int iter, cudaStream_t stream) {
  cudaMemsetAsync(v.cell_start, 0, sizeof(int) * ((size_t)v.npix + 1), stream);
  cudaMemsetAsync(v.cell_fill, 0, sizeof(int) * (size_t)v.npix, stream);
  cudaMemsetAsync(v.hit_count, 0, sizeof(int), stream);
  const size_t smem = (size_t)kSppmStack * kSppmBlock * sizeof(int2);
  if (v.photons > 0)
    k_sppm_photons<kSppmStack><<<blocks_for(v.photons, kSppmBlock), kSppmBlock, smem, stream>>>(s, v, iter);
  launch_sppm_scan(v, stream);
  k_sppm_fill<<<std::min(blocks_for(v.hits_cap, 256), 8192), 256, 0, stream>>>(v);
  k_sppm_gather<<<blocks_for((int64_t)v.npix * 32, 128), 128, 0, stream>>>(s, v);
  k_sppm_update<<<blocks_for(v.npix, 256), 256, 0, stream>>>(v);
}

}  // namespace orion_gb300
