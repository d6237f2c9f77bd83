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

}  // namespace orion_gb300
