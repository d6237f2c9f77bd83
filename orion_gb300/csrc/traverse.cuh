// BVH traversal: closest hit and occlusion over the host-built BVH
// (32-byte nodes with adjacent child pairs, Woop triangle records).
//
// Replaces rtcIntersect (src/core/kernel.cpp:111-125). Hit semantics match
// the reference's use of Embree: accept tnear < t <= tfar, barycentrics
// u, v >= 0, u + v <= 1, no culling; the closest hit is the least (t, primID).
//
// The traversal stack is short and lives in shared memory, laid out
// [entry][thread] so a warp's pushes hit 32 different banks; entries past the
// shared part spill to a per-thread local array. Each entry is the (a, b)
// pair of a postponed node, so popping needs no memory access.
#pragma once
#include "device_types.h"
#include "dmath.cuh"

namespace orion_gb300 {

constexpr int kMaxStack = 64;  // >= BVH depth bound (the builder keeps depth < 64)

struct TraceScene {
  const float4* __restrict__ nodes;  // 2 float4 per node
  const float4* __restrict__ woop;   // 3 float4 per triangle, leaf order
  const int* __restrict__ tri_prim;  // leaf order -> primID
};

struct RayHit {
  float t, u, v;
  int tri;  // leaf-order triangle index, -1 for a miss
};

template <int SMEM>
struct TraversalStack {
  int2* smem;  // SMEM entries for this thread, stride `stride`
  int stride;
  int sp;
  int2 local[kMaxStack - SMEM > 0 ? kMaxStack - SMEM : 1];
  __device__ __forceinline__ void push(int2 e) {
    if (sp < SMEM)
      smem[sp * stride] = e;
    else
      local[sp - SMEM] = e;
    ++sp;
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

// ANY = false: closest hit over (tnear, tfar]. ANY = true: first hit found.
template <bool ANY, int SMEM>
__device__ __forceinline__ RayHit traverse(const TraceScene& s, V3 o, V3 d, float tnear, float tfar,
                                           TraversalStack<SMEM>& st) {
  RayHit h;
  h.t = tfar;
  h.u = h.v = 0.f;
  h.tri = -1;
  V3 idir = V3{safe_inv(d.x), safe_inv(d.y), safe_inv(d.z)};
  V3 oid = V3{o.x * idir.x, o.y * idir.y, o.z * idir.z};
  st.sp = 0;
  float4 rlo = __ldg(s.nodes), rhi = __ldg(s.nodes + 1);
  if (!(box_entry(rlo, rhi, idir, oid, tnear, tfar) < __int_as_float(0x7f800000))) return h;
  int a = __float_as_int(rlo.w), b = __float_as_int(rhi.w);
  int best_prim = 0x7fffffff;
  while (true) {
    if (b == 0) {
      float4 l0 = __ldg(s.nodes + 2 * a), h0 = __ldg(s.nodes + 2 * a + 1);
      float4 l1 = __ldg(s.nodes + 2 * a + 2), h1 = __ldg(s.nodes + 2 * a + 3);
      float t0 = box_entry(l0, h0, idir, oid, tnear, h.t);
      float t1 = box_entry(l1, h1, idir, oid, tnear, h.t);
      bool hit0 = t0 < __int_as_float(0x7f800000), hit1 = t1 < __int_as_float(0x7f800000);
      if (hit0 && hit1) {
        int2 n0 = make_int2(__float_as_int(l0.w), __float_as_int(h0.w));
        int2 n1 = make_int2(__float_as_int(l1.w), __float_as_int(h1.w));
        if (t1 < t0) {
          int2 tmp = n0;
          n0 = n1;
          n1 = tmp;
        }
        st.push(n1);
        a = n0.x;
        b = n0.y;
        continue;
      }
      if (hit0) {
        a = __float_as_int(l0.w);
        b = __float_as_int(h0.w);
        continue;
      }
      if (hit1) {
        a = __float_as_int(l1.w);
        b = __float_as_int(h1.w);
        continue;
      }
    } else {
      for (int k = a; k < a + b; ++k) {
        float t, u, v;
        if (woop_hit(s.woop, k, o, d, tnear, h.t, &t, &u, &v)) {
          if (ANY) {
            h.t = t;
            h.u = u;
            h.v = v;
            h.tri = k;
            return h;
          }
          int prim = __ldg(s.tri_prim + k);
          if (t < h.t || h.tri < 0 || prim < best_prim) {
            h.t = t;
            h.u = u;
            h.v = v;
            h.tri = k;
            best_prim = prim;
          }
        }
      }
    }
    if (st.sp == 0) break;
    int2 e = st.pop();
    a = e.x;
    b = e.y;
  }
  return h;
}

// ------------------------------------------------ persistent warp traversal
//
// The kernels below trace a queue of rays with warps that stay resident:
//  * while-while: each lane walks inner nodes until every active lane of the
//    warp has found a leaf (the first leaf a lane finds is postponed and the
//    lane keeps traversing), then all lanes test triangles together, so the
//    two phases do not interleave within a warp;
//  * dynamic fetch: when fewer than `refill_below` lanes still hold a ray,
//    the warp takes new rays for its idle lanes from the queue with one
//    atomicAdd, instead of idling until its slowest ray ends.
// Warp votes only steer scheduling; each ray's result does not depend on them.

struct LaneRay {
  V3 o, d, idir, oid;
  float tnear, tmax;  // tmax shrinks to the closest hit found so far
  float u, v;
  int tri, best_prim;
  int na, nb;  // node to visit: (a, b) fields; na < 0 when the stack is empty
  int la, lb;  // postponed leaf, lb == 0 when none
};

__device__ __forceinline__ void lane_start(LaneRay& r, const TraceScene& s, float4 o4, float4 d4, float tmax) {
  r.o = xyz(o4);
  r.d = xyz(d4);
  r.idir = V3{safe_inv(r.d.x), safe_inv(r.d.y), safe_inv(r.d.z)};
  r.oid = V3{r.o.x * r.idir.x, r.o.y * r.idir.y, r.o.z * r.idir.z};
  r.tnear = 0.f;
  r.tmax = tmax;
  r.u = r.v = 0.f;
  r.tri = -1;
  r.best_prim = 0x7fffffff;
  r.lb = 0;
  r.la = 0;
  float4 lo = __ldg(s.nodes), hi = __ldg(s.nodes + 1);
  if (box_entry(lo, hi, r.idir, r.oid, r.tnear, r.tmax) < __int_as_float(0x7f800000)) {
    r.na = __float_as_int(lo.w);
    r.nb = __float_as_int(hi.w);
  } else {
    r.na = -1;
    r.nb = 0;
  }
}

template <int SMEM>
__device__ __forceinline__ void lane_pop(LaneRay& r, TraversalStack<SMEM>& st) {
  if (st.sp == 0) {
    r.na = -1;
    r.nb = 0;
  } else {
    int2 e = st.pop();
    r.na = e.x;
    r.nb = e.y;
  }
}

// Inner nodes until this lane holds a postponed leaf and every active lane
// in the warp does too (or has no inner node left).
template <int SMEM>
__device__ __forceinline__ void lane_inner(LaneRay& r, const TraceScene& s, TraversalStack<SMEM>& st) {
  while (r.na >= 0 && r.nb == 0) {
    const int a = r.na;
    float4 l0 = __ldg(s.nodes + 2 * a), h0 = __ldg(s.nodes + 2 * a + 1);
    float4 l1 = __ldg(s.nodes + 2 * a + 2), h1 = __ldg(s.nodes + 2 * a + 3);
    float t0 = box_entry(l0, h0, r.idir, r.oid, r.tnear, r.tmax);
    float t1 = box_entry(l1, h1, r.idir, r.oid, r.tnear, r.tmax);
    bool hit0 = t0 < __int_as_float(0x7f800000), hit1 = t1 < __int_as_float(0x7f800000);
    if (hit0 && hit1) {
      int2 n0 = make_int2(__float_as_int(l0.w), __float_as_int(h0.w));
      int2 n1 = make_int2(__float_as_int(l1.w), __float_as_int(h1.w));
      if (t1 < t0) {
        int2 tmp = n0;
        n0 = n1;
        n1 = tmp;
      }
      st.push(n1);
      r.na = n0.x;
      r.nb = n0.y;
    } else if (hit0) {
      r.na = __float_as_int(l0.w);
      r.nb = __float_as_int(h0.w);
    } else if (hit1) {
      r.na = __float_as_int(l1.w);
      r.nb = __float_as_int(h1.w);
    } else {
      lane_pop(r, st);
    }
    if (r.nb > 0 && r.lb == 0) {  // first leaf: postpone it, keep traversing
      r.la = r.na;
      r.lb = r.nb;
      lane_pop(r, st);
    }
    if (!__any_sync(__activemask(), r.lb == 0)) break;
  }
}

// Triangles of the postponed leaf, then of any leaves the lane is standing on.
// Returns true when an occlusion query found its hit (ANY).
template <bool ANY, int SMEM>
__device__ __forceinline__ bool lane_leaves(LaneRay& r, const TraceScene& s, TraversalStack<SMEM>& st) {
  while (r.lb > 0) {
    for (int k = r.la; k < r.la + r.lb; ++k) {
      float t, u, v;
      if (woop_hit(s.woop, k, r.o, r.d, r.tnear, r.tmax, &t, &u, &v)) {
        if (ANY) {
          r.tmax = t;
          r.tri = k;
          return true;
        }
        int prim = __ldg(s.tri_prim + k);
        if (t < r.tmax || r.tri < 0 || prim < r.best_prim) {
          r.tmax = t;
          r.u = u;
          r.v = v;
          r.tri = k;
          r.best_prim = prim;
        }
      }
    }
    if (r.na >= 0 && r.nb > 0) {
      r.la = r.na;
      r.lb = r.nb;
      lane_pop(r, st);
    } else {
      r.lb = 0;
    }
  }
  return false;
}

}  // namespace orion_gb300
