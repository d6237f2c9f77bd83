// BVH traversal: closest hit and occlusion over the host-built 8-wide BVH
// (80-byte nodes with quantised child boxes, Woop triangle records).
//
// Replaces rtcIntersect (src/core/kernel.cpp:111-125). Hit semantics match
// the reference's use of Embree: accept tnear < t <= tfar, barycentrics
// u, v >= 0, u + v <= 1, no culling; the closest hit is the least (t, primID).
//
// The traversal stack is short and lives in shared memory, laid out
// [entry][thread] so a warp's pushes hit 32 different banks; entries past the
// shared part spill to a per-thread local array. Each entry is an 8-byte
// node or triangle group, so popping needs no memory access.
//
// Capacity. A traversal holds at most one stack entry per tree level: an
// entry is the rest of one visited node's group of hit children, and popping
// it replaces it by at most one entry of the same level. So the stack never
// holds more entries than the wide tree has levels, which is at most the
// binary tree's depth; the builder bounds that below kMaxBvhDepth (48) and
// orion_gpu_scene_upload rejects any deeper tree, so kMaxStack (96) entries
// cannot overflow and the production kernels carry no per-push check (a
// checked push measured 2.7% slower on the 1024x1024 x 64 spp displaced
// sphere). Kernels built with a smaller capacity (kTestStackEntries, kernels.h:
// the failure-path tests) check every push: a push beyond the capacity writes
// nothing, the entry is dropped and the ray poisoned (tmax = -1, so no further
// box or triangle test passes and the traversal drains); the persistent trace
// kernels report a poisoned ray as a miss and set kErrTraversalStack in the
// launch's error word, and the render returns ORION_ERR_DEVICE.
#pragma once
#include "device_types.h"
#include "dmath.cuh"

namespace orion_gb300 {

constexpr int kMaxStack = 96;  // entries; >= the deepest tree a scene upload accepts
static_assert(kMaxStack > kMaxBvhDepth, "a traversal stack holds one entry per tree level");

struct TraceScene {
  const float4* __restrict__ nodes;  // 5 float4 per WideNode
  const float4* __restrict__ woop;   // 3 float4 per triangle, leaf order
  const int* __restrict__ tri_prim;  // leaf order -> primID
  const uint8_t* __restrict__ tri_class;  // leaf order -> ShadeClass
};

struct RayHit {
  float t, u, v;
  int tri;  // leaf-order triangle index, -1 for a miss
};

template <int SMEM, int CAP = kMaxStack>
struct TraversalStack {
  static_assert(CAP >= SMEM, "the shared part is within the capacity");
  int2* smem;  // SMEM entries for this thread, stride `stride`
  int stride;
  int sp;
  int2 local[CAP - SMEM > 0 ? CAP - SMEM : 1];
  // False (and nothing written) when a test-capacity stack already holds CAP
  // entries; a kMaxStack stack cannot overflow (see the file comment).
  __device__ __forceinline__ bool push(int2 e) {
    if constexpr (CAP < kMaxStack) {
      if (sp >= CAP) return false;
    }
    if (sp < SMEM)
      smem[sp * stride] = e;
    else
      local[sp - SMEM] = e;
    ++sp;
    return true;
  }
  __device__ __forceinline__ int2 pop() {
    --sp;
    return sp < SMEM ? smem[sp * stride] : local[sp - SMEM];
  }
};

__device__ __forceinline__ float safe_inv(float d) {
  return 1.f / (fabsf(d) > 1e-20f ? d : copysignf(1e-20f, d));
}

// Slab test; returns the entry distance or +inf when the box is missed.
__device__ __forceinline__ float box_entry(float4 lo, float4 hi, V3 idir, V3 oid, float tmin, float tmax) {
  float x0 = fmaf(lo.x, idir.x, -oid.x), x1 = fmaf(hi.x, idir.x, -oid.x);
  float y0 = fmaf(lo.y, idir.y, -oid.y), y1 = fmaf(hi.y, idir.y, -oid.y);
  float z0 = fmaf(lo.z, idir.z, -oid.z), z1 = fmaf(hi.z, idir.z, -oid.z);
  float tn = fmaxf(fmaxf(fminf(x0, x1), fminf(y0, y1)), fmaxf(fminf(z0, z1), tmin));
  float tf = fminf(fminf(fmaxf(x0, x1), fmaxf(y0, y1)), fminf(fmaxf(z0, z1), tmax));
  return tn <= tf ? tn : __int_as_float(0x7f800000);
}

// Woop unit-triangle test on an origin-relative record: rows (r2, r0, r1)
// of the inverse of [e1 e2 n] with v0 in the .w components. Returns true
// with t, u, v for a hit in (tnear, tfar].
__device__ __forceinline__ bool woop_hit(const float4* __restrict__ woop, int k, V3 o, V3 d, float tnear, float tfar,
                                         float* t, float* u, float* v) {
  float4 w0 = __ldg(woop + 3 * k);
  float4 w1 = __ldg(woop + 3 * k + 1);
  float4 w2 = __ldg(woop + 3 * k + 2);
  float cx = o.x - w0.w, cy = o.y - w1.w, cz = o.z - w2.w;
  float oz = -(cx * w0.x + cy * w0.y + cz * w0.z);
  float dz = d.x * w0.x + d.y * w0.y + d.z * w0.z;
  float tt = oz * __frcp_rn(dz);
  if (!(tt > tnear && tt <= tfar)) return false;
  float uu = (cx * w1.x + cy * w1.y + cz * w1.z) + tt * (d.x * w1.x + d.y * w1.y + d.z * w1.z);
  if (!(uu >= 0.f && uu <= 1.f)) return false;
  float vv = (cx * w2.x + cy * w2.y + cz * w2.z) + tt * (d.x * w2.x + d.y * w2.y + d.z * w2.z);
  if (!(vv >= 0.f && uu + vv <= 1.f)) return false;
  *t = tt;
  *u = uu;
  *v = vv;
  return true;
}

// ------------------------------------------------------- 8-wide traversal
//
// A node visit tests the ray against the eight quantised child boxes of one
// WideNode (five 16-byte loads) and yields two groups:
//   node group     (child_base, hits << 24 | imask): the hit internal
//                  children, one bit per child at position slot ^ octant,
//                  so taking the lowest bit first visits them roughly near
//                  to far;
//   triangle group (tri_base, mask): the triangles of the hit leaf children.
// A stack entry is a node group (top byte non-zero); an entry with a zero
// top byte would be taken as a triangle group. The root is the single
// internal child of a virtual group.


// Octant of a ray from the signs of its reciprocal direction (never zero,
// see safe_inv), so the near-plane choice agrees with the slab arithmetic
// even for a -0 direction component.
__device__ __forceinline__ uint32_t ray_octant(V3 idir) {
  return (idir.x < 0.f ? 1u : 0u) | (idir.y < 0.f ? 2u : 0u) | (idir.z < 0.f ? 4u : 0u);
}

__device__ __forceinline__ uint2 root_group(uint32_t oct) { return make_uint2(0u, (1u << (24 + oct)) | 1u); }

// Byte `b` of `w` as the float 1 + byte * 2^-15 (exact): one byte permute
// places the byte in mantissa bits 8..15 of 1.0.
__device__ __forceinline__ float q8(uint32_t w, int b) {
  return __uint_as_float(__byte_perm(w, 0x3f800000u, 0x7604u + ((uint32_t)b << 4)));
}

__device__ __forceinline__ float max3f(float a, float b, float c) {
  float d;
  asm("max.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

__device__ __forceinline__ float min3f(float a, float b, float c) {
  float d;
  asm("min.f32 %0, %1, %2, %3;" : "=f"(d) : "f"(a), "f"(b), "f"(c));
  return d;
}

// Moves bit s of an 8-bit mask to bit s ^ oct.
__device__ __forceinline__ uint32_t octant_permute(uint32_t x, uint32_t oct) {
  if (oct & 1u) x = ((x & 0x55u) << 1) | ((x >> 1) & 0x55u);
  if (oct & 2u) x = ((x & 0x33u) << 2) | ((x >> 2) & 0x33u);
  if (oct & 4u) x = ((x & 0x0fu) << 4) | ((x >> 4) & 0x0fu);
  return x;
}

// oct: the ray's octant (which box planes are near); ord: the octant whose
// near-to-far child order the node group lists (oct for closest hit, its
// opposite for occlusion: far children first).
__device__ __forceinline__ void wide_node(const float4* __restrict__ nodes, int idx, V3 o, V3 idir, uint32_t oct,
                                          float tnear, float tmax, uint2& ng, uint2& tg, uint32_t ord) {
  const float4* n = nodes + 5 * (size_t)idx;
  const float4 n0 = __ldg(n), n1 = __ldg(n + 1), n2 = __ldg(n + 2), n3 = __ldg(n + 3), n4 = __ldg(n + 4);
  // A child plane p + q * cell is met at ray distance (p - o + q * cell) / d,
  // computed as fma(1 + q * 2^-15, S, C) with S = 2^15 * cell / d (a power-of-
  // two scaling, exact) and C = (p - o) / d - S: one byte permute and one fma
  // per plane. C rounds once per node; beyond the rounding of (p - o) / d that
  // costs at most 2^-9 of a cell, well inside the outward quantisation. (The
  // builder keeps cells at or below 2^112, so S stays finite.)
  const uint32_t ew = __float_as_uint(n0.w);
  const float sx = __uint_as_float(((ew & 0xffu) + 15u) << 23) * idir.x;
  const float sy = __uint_as_float((((ew >> 8) & 0xffu) + 15u) << 23) * idir.y;
  const float sz = __uint_as_float((((ew >> 16) & 0xffu) + 15u) << 23) * idir.z;
  const uint32_t imask = ew >> 24;
  const float ox = fmaf(n0.x - o.x, idir.x, -sx), oy = fmaf(n0.y - o.y, idir.y, -sy);
  const float oz = fmaf(n0.z - o.z, idir.z, -sz);
  // Quantised bounds: lo x = (n2.x, n2.y), lo y = (n2.z, n2.w), lo z = (n3.x, n3.y),
  // hi x = (n3.z, n3.w), hi y = (n4.x, n4.y), hi z = (n4.z, n4.w); the near plane
  // along a negative direction is the upper bound.
  const uint32_t lx0 = __float_as_uint(n2.x), lx1 = __float_as_uint(n2.y);
  const uint32_t ly0 = __float_as_uint(n2.z), ly1 = __float_as_uint(n2.w);
  const uint32_t lz0 = __float_as_uint(n3.x), lz1 = __float_as_uint(n3.y);
  const uint32_t hx0 = __float_as_uint(n3.z), hx1 = __float_as_uint(n3.w);
  const uint32_t hy0 = __float_as_uint(n4.x), hy1 = __float_as_uint(n4.y);
  const uint32_t hz0 = __float_as_uint(n4.z), hz1 = __float_as_uint(n4.w);
  const bool fx = oct & 1u, fy = oct & 2u, fz = oct & 4u;
  const uint32_t nx[2] = {fx ? hx0 : lx0, fx ? hx1 : lx1}, xf[2] = {fx ? lx0 : hx0, fx ? lx1 : hx1};
  const uint32_t ny[2] = {fy ? hy0 : ly0, fy ? hy1 : ly1}, yf[2] = {fy ? ly0 : hy0, fy ? ly1 : hy1};
  const uint32_t nz[2] = {fz ? hz0 : lz0, fz ? hz1 : lz1}, zf[2] = {fz ? lz0 : hz0, fz ? lz1 : hz1};
  uint32_t hm = 0u;  // bit s: box of slot s hit (empty slots have inverted boxes)
#pragma unroll
  for (int s = 0; s < 8; ++s) {
    const int h = s >> 2, b = s & 3;
    const float tn = max3f(fmaf(q8(nx[h], b), sx, ox), fmaf(q8(ny[h], b), sy, oy),
                           fmaxf(fmaf(q8(nz[h], b), sz, oz), tnear));
    const float tf = min3f(fmaf(q8(xf[h], b), sx, ox), fmaf(q8(yf[h], b), sy, oy),
                           fminf(fmaf(q8(zf[h], b), sz, oz), tmax));
    hm |= (tn <= tf ? 1u : 0u) << s;
  }
  const uint32_t hits = octant_permute(hm & imask, ord);
  uint32_t tris = 0u;
  const uint32_t meta[2] = {__float_as_uint(n1.z), __float_as_uint(n1.w)};
  for (uint32_t lh = hm & ~imask; lh; lh &= lh - 1u) {
    const uint32_t s = (uint32_t)__ffs(lh) - 1u;
    const uint32_t m = (meta[s >> 2] >> (8u * (s & 3u))) & 0xffu;
    tris |= ((1u << (m >> 5)) - 1u) << (m & 31u);
  }
  ng = make_uint2(__float_as_uint(n1.x), hits ? (hits << 24) | imask : 0u);
  tg = make_uint2(__float_as_uint(n1.y), tris);
}

// Takes the nearest-first remaining child of a node group; returns its node index.
__device__ __forceinline__ int take_child(uint2& ng, uint32_t oct) {
  const uint32_t k = (uint32_t)__ffs(ng.y >> 24) - 1u;
  ng.y &= ~(1u << (24 + k));
  const uint32_t slot = k ^ oct;
  const int child = (int)ng.x + __popc((ng.y & 0xffu) & ((1u << slot) - 1u));
  if (ng.y <= 0x00ffffffu) ng.y = 0u;
  return child;
}

// ANY = false: closest hit over (tnear, tfar]. ANY = true: first hit found,
// children visited far to near (see lane_visit). A stack overflow ends the
// traversal with a miss (see the file comment).
template <bool ANY, int SMEM, int CAP>
__device__ __forceinline__ RayHit traverse(const TraceScene& s, V3 o, V3 d, float tnear, float tfar,
                                           TraversalStack<SMEM, CAP>& st) {
  RayHit h;
  h.t = tfar;
  h.u = h.v = 0.f;
  h.tri = -1;
  const V3 idir = V3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
  const uint32_t oct = ray_octant(idir);
  const uint32_t ord = ANY ? oct ^ 7u : oct;
  int best_prim = 0x7fffffff;
  st.sp = 0;
  uint2 ng = root_group(ord), tg = make_uint2(0u, 0u);
  while (true) {
    if (ng.y > 0x00ffffffu) {
      const int child = take_child(ng, ord);
      if (ng.y && !st.push(make_int2((int)ng.x, (int)ng.y))) {
        h.t = -1.f;  // poisoned: nothing passes a test against tmax < tnear
        h.tri = -1;
      }
      wide_node(s.nodes, child, o, idir, oct, tnear, h.t, ng, tg, ord);
    } else {
      tg = ng;
      ng = make_uint2(0u, 0u);
    }
    while (tg.y != 0u) {
      const int k = (int)tg.x + __ffs(tg.y) - 1;
      tg.y &= tg.y - 1u;
      float t, u, v;
      if (woop_hit(s.woop, k, o, d, tnear, h.t, &t, &u, &v)) {
        if (ANY) {
          h.t = t;
          h.u = u;
          h.v = v;
          h.tri = k;
          return h;
        }
        const int prim = __ldg(s.tri_prim + k);
        if (t < h.t || h.tri < 0 || prim < best_prim) {
          h.t = t;
          h.u = u;
          h.v = v;
          h.tri = k;
          best_prim = prim;
        }
      }
    }
    if (ng.y == 0u) {
      if (st.sp == 0) break;
      const int2 e = st.pop();
      ng = make_uint2((uint32_t)e.x, (uint32_t)e.y);
    }
  }
  if (h.t < 0.f) {  // stack overflow: reported as a miss
    h.t = tfar;
    h.tri = -1;
  }
  return h;
}

// ------------------------------------------------ persistent warp traversal
//
// The kernels below trace a queue of rays with warps that stay resident.
// Each loop iteration visits one node per lane; the triangles those visits
// yield are then tested by the whole warp together (warp_triangles), and
// each lane pops its next node group. (Postponing the triangles of lanes
// that are few in their warp, to keep descending with the rest, was measured
// 11% slower on the 8-wide tree: a leaf visit costs about as much as the
// node visits it waits for.) When fewer than `refill_below` lanes still hold
// a ray, the warp takes new rays for its idle lanes from the queue with one
// atomicAdd. Warp votes and the dealing of triangle tests only steer
// scheduling; each ray's result does not depend on them.

struct LaneRay {
  V3 o, d, idir;
  float tmax;  // shrinks to the closest hit found so far; the ray starts at t = 0
  float u, v;
  int tri, best_prim;
  uint32_t oct;
  uint2 ng, tg;
};

// any: an occlusion ray (its node groups list children far to near, lane_visit).
__device__ __forceinline__ void lane_start(LaneRay& r, float4 o4, float4 d4, float tmax, bool any) {
  r.o = xyz(o4);
  r.d = xyz(d4);
  r.idir = V3{safe_inv(r.d.x), safe_inv(r.d.y), safe_inv(r.d.z)};
  r.oct = ray_octant(r.idir);
  r.tmax = tmax;
  r.u = r.v = 0.f;
  r.tri = -1;
  r.best_prim = 0x7fffffff;
  r.ng = root_group(any ? r.oct ^ 7u : r.oct);
  r.tg = make_uint2(0u, 0u);
}

// Node visits and triangle tests of one lane (COUNT instantiations only).
struct TraceWork {
  unsigned long long nodes = 0, tris = 0;
};

// One node visit: the lane's next node group yields its hit children (r.ng)
// and the triangles of its hit leaves (r.tg). COUNT adds the visit to `wk`.
// A push beyond the stack's capacity poisons the ray (r.tmax = -1; see the
// file comment): the caller reports it when the ray is done.
template <bool ANY, int SMEM, bool COUNT = false, int CAP = kMaxStack>
__device__ __forceinline__ void lane_visit(LaneRay& r, const TraceScene& s, TraversalStack<SMEM, CAP>& st,
                                           TraceWork* wk) {
  if (r.ng.y > 0x00ffffffu) {
    // Occlusion rays take far children first: a shadow ray leaves the surface
    // it starts on, and the subtrees around its origin seldom hold its
    // occluder (shadow traversal of the 1024x1024 x 64 spp displaced sphere
    // 19.0 -> 15.5 ms against near first).
    const uint32_t ord = ANY ? (r.oct ^ 7u) : r.oct;
    const int child = take_child(r.ng, ord);
    if (r.ng.y && !st.push(make_int2((int)r.ng.x, (int)r.ng.y))) r.tmax = -1.f;
    wide_node(s.nodes, child, r.o, r.idir, r.oct, 0.f, r.tmax, r.ng, r.tg, ord);
    if (COUNT) ++wk->nodes;
  } else {
    r.tg = r.ng;
    r.ng = make_uint2(0u, 0u);
  }
}

// After a visit and its triangles: pops the lane's next node group. Returns
// true when the stack ran empty (the ray is done).
template <int SMEM, int CAP>
__device__ __forceinline__ bool lane_pop(LaneRay& r, TraversalStack<SMEM, CAP>& st) {
  if (r.ng.y == 0u) {
    if (st.sp == 0) return true;
    const int2 e = st.pop();
    r.ng = make_uint2((uint32_t)e.x, (uint32_t)e.y);
  }
  return false;
}

// Position of the n-th (from 0) set bit of m; n < popc(m).
__device__ __forceinline__ uint32_t nth_set_bit(uint32_t m, uint32_t n) {
  uint32_t p = 0u, c = (uint32_t)__popc(m & 0xffffu);
  if (n >= c) n -= c, m >>= 16, p += 16u;
  c = (uint32_t)__popc(m & 0xffu);
  if (n >= c) n -= c, m >>= 8, p += 8u;
  c = (uint32_t)__popc(m & 0xfu);
  if (n >= c) n -= c, m >>= 4, p += 4u;
  c = (uint32_t)__popc(m & 0x3u);
  if (n >= c) n -= c, m >>= 2, p += 2u;
  return p + (n >= (m & 1u) ? 1u : 0u);
}

// Shared scratch of one warp for warp_triangles.
struct TriScratch {
  unsigned long long key[32];  // owner lane -> least (t bits, primID) of its ray so far
  uint8_t owner[32];           // first pair of a segment -> its owner lane
};
static_assert(sizeof(TriScratch) == kTriScratchBytes, "per-warp triangle scratch");

// Dynamic shared memory of a persistent trace block: the stacks' shared
// entries, then one TriScratch per warp.
__host__ __device__ constexpr size_t trace_smem_bytes(int smem_entries, int block) {
  return (size_t)smem_entries * block * sizeof(int2) + (size_t)(block / 32) * kTriScratchBytes;
}

// Dealing a lane's triangle tests to the whole warp pays when one lane holds
// many more than the others: a dealt round costs about as much as this many
// one-by-one tests (closest hit: keeping the least hit takes shared-memory
// atomics; occlusion: one vote). Measured on the 1024x1024 x 64 spp displaced
// sphere: 986 Mpaths/s at 4 / 2, 985 at 3 / 2, 974 at 6 / 1, 971 dealing
// every step; occlusion at 3 a little ahead of 2.
constexpr int kDealClosest = 4, kDealAny = 3;

// Tests the triangles of every lane's r.tg (all 32 lanes call it; lanes
// without a ray have r.tg.y == 0), with the same result as each lane testing
// its own one by one, which it does when the warp's tests are even. When a
// few lanes hold most of them (the largest count at least kDealClosest /
// kDealAny times the rounds dealing takes), the warp's (ray, triangle) pairs,
// listed lane by lane in bit order, are dealt to the lanes 32 at a time: a
// lane tests its pair against the owning lane's ray (fetched by shuffles), and
// each owner keeps the least (t, primID) of its hits in (0, tmax] or, ANY,
// any hit. UNIFORM: every lane traces the same scene (otherwise each pair
// uses its owner's triangle arrays). Returns true for an ANY lane whose ray
// hit.
template <bool ANY, bool COUNT, bool UNIFORM>
__device__ __forceinline__ bool warp_triangles(LaneRay& r, const TraceScene& s, TriScratch* sc, TraceWork* wk) {
  constexpr unsigned kFull = 0xffffffffu;
  constexpr int kDeal = ANY ? kDealAny : kDealClosest;
  const int lane = threadIdx.x & 31;
  bool found = false;
  while (true) {
    const int c = __popc(r.tg.y);
    const int total = (int)__reduce_add_sync(kFull, (unsigned)c);
    if (total == 0) break;
    if ((int)__reduce_max_sync(kFull, (unsigned)c) < kDeal * ((total + 31) >> 5)) {
      while (r.tg.y != 0u) {  // one by one
        const int k = (int)r.tg.x + __ffs(r.tg.y) - 1;
        r.tg.y &= r.tg.y - 1u;
        float t, u, v;
        if (COUNT) ++wk->tris;
        if (woop_hit(s.woop, k, r.o, r.d, 0.f, r.tmax, &t, &u, &v)) {
          if (ANY) {
            r.tri = k;
            r.tg.y = 0u;
            found = true;
            break;
          }
          const int prim = __ldg(s.tri_prim + k);
          if (t < r.tmax || r.tri < 0 || prim < r.best_prim) {
            r.tmax = t;
            r.u = u;
            r.v = v;
            r.tri = k;
            r.best_prim = prim;
          }
        }
      }
      break;
    }
    // Dealt: this lane's pairs are [first, first + c) of the warp's list.
    int incl = c;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(kFull, incl, o);
      if (lane >= o) incl += y;
    }
    const int first = incl - c;
    const bool owns = c > 0 && first < 32;
    const int dealt = owns ? min(c, 32 - first) : 0;  // pairs of this lane tested this round
    const unsigned starts = __reduce_or_sync(kFull, owns ? 1u << first : 0u);
    if (owns) sc->owner[first] = (uint8_t)lane;
    __syncwarp();
    // The pair at position `lane`: segment start at or below it (position 0
    // always starts one), its owner, and the triangle's index there.
    const int seg = 31 - __clz(starts & (kFull >> (31 - lane)));
    const int ow = sc->owner[seg];
    const float ox = __shfl_sync(kFull, r.o.x, ow), oy = __shfl_sync(kFull, r.o.y, ow);
    const float oz = __shfl_sync(kFull, r.o.z, ow), dx = __shfl_sync(kFull, r.d.x, ow);
    const float dy = __shfl_sync(kFull, r.d.y, ow), dz = __shfl_sync(kFull, r.d.z, ow);
    const float tmax = __shfl_sync(kFull, r.tmax, ow);
    const uint32_t obase = __shfl_sync(kFull, r.tg.x, ow), omask = __shfl_sync(kFull, r.tg.y, ow);
    const float4* woop = s.woop;
    const int* tri_prim = s.tri_prim;
    if constexpr (!UNIFORM) {
      woop = (const float4*)__shfl_sync(kFull, (unsigned long long)s.woop, ow);
      tri_prim = (const int*)__shfl_sync(kFull, (unsigned long long)s.tri_prim, ow);
    }
    bool hit = false;
    float t = 0.f, u = 0.f, v = 0.f;
    int k = 0;
    if (lane < total) {
      k = (int)(obase + nth_set_bit(omask, (uint32_t)(lane - seg)));
      hit = woop_hit(woop, k, V3{ox, oy, oz}, V3{dx, dy, dz}, 0.f, tmax, &t, &u, &v);
    }
    const unsigned span = dealt == 32 ? kFull : (((1u << dealt) - 1u) << (first & 31));
    if (ANY) {
      if (__ballot_sync(kFull, hit) & span) {
        r.tri = 0;  // occluded; which triangle is not reported
        found = true;
      }
    } else {
      if (owns)
        sc->key[lane] = ((unsigned long long)__float_as_uint(r.tmax) << 32) |
                        (r.tri >= 0 ? (uint32_t)r.best_prim : 0xffffffffu);
      __syncwarp();
      unsigned long long key = 0ull;
      if (hit) {
        key = ((unsigned long long)__float_as_uint(t) << 32) | (uint32_t)__ldg(tri_prim + k);
        atomicMin(&sc->key[ow], key);
      }
      __syncwarp();
      const unsigned wins = __ballot_sync(kFull, hit && sc->key[ow] == key) & span;
      const int wl = wins ? __ffs(wins) - 1 : lane;
      const float wu = __shfl_sync(kFull, u, wl), wv = __shfl_sync(kFull, v, wl);
      const int wt = __shfl_sync(kFull, k, wl);
      if (wins) {
        const unsigned long long best = sc->key[lane];
        r.tmax = __uint_as_float((uint32_t)(best >> 32));
        r.best_prim = (int)(uint32_t)best;
        r.tri = wt;
        r.u = wu;
        r.v = wv;
      }
    }
    if (COUNT) wk->tris += (unsigned long long)dealt;
    if (found || dealt == c)
      r.tg.y = 0u;
    else if (dealt > 0)
      r.tg.y &= kFull << nth_set_bit(r.tg.y, (uint32_t)dealt);
    __syncwarp();
  }
  return found;
}

}  // namespace orion_gb300
