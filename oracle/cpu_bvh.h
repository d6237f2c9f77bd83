// CPU closest-hit kernel for the oracle (test infrastructure, never shipped).
//
// The reference traces every ray through Embree 2.16.3 (`rtcIntersect`,
// src/core/kernel.cpp:111-125), a closed binary that is not available here.
// This header stands in for it, in two places:
//   * oracle/ref/embree_shim.cpp re-defines the reference's `EmbreeKernel`
//     methods with it, so the reference's own integrator can be compiled;
//   * oracle/port/ (the C++ restatement) traces with it.
//
// Semantics follow Embree 2's documented ray query (rtcore_ray.h: `tnear`,
// `tfar` shortened to the hit distance, barycentric `u`, `v` with
// p = (1-u-v) p0 + u p1 + v p2, `primID`): a hit is accepted when
// tnear < t <= tfar and u, v >= 0, u + v <= 1, with no back-face culling.
// The triangle test restates Embree 2's published Moeller-Trumbore variant
// (triangle_intersector_moeller.h in the Embree 2.16 sources): e1 = v0 - v1,
// e2 = v2 - v0, Ng = e1 x e2, C = v0 - o, R = d x C, U = R.e2, V = R.e1,
// T = Ng.C, all sign-corrected by den = Ng.d and divided by |den|.
//
// Closest hit is the minimum of (t, primID) in lexicographic order, so the
// result equals a brute-force loop over all triangles in primID order. Node
// bounds are padded and the slab test is inclusive so that the BVH never
// culls a triangle the brute-force loop would accept; `brute_force_closest`
// exists to check exactly that.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <vector>

namespace oracle_bvh {

struct Hit {
  float t = 0.f, u = 0.f, v = 0.f;
  int32_t prim = -1;
};

struct Tri {
  float v0[3], e1[3], e2[3], ng[3];  // e1 = v0 - v1, e2 = v2 - v0, ng = e1 x e2
};

inline void cross3(const float a[3], const float b[3], float out[3]) {
  out[0] = a[1] * b[2] - a[2] * b[1];
  out[1] = a[2] * b[0] - a[0] * b[2];
  out[2] = a[0] * b[1] - a[1] * b[0];
}
inline float dot3(const float a[3], const float b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

// Returns true and fills t,u,v when the ray hits the triangle in (tnear, tfar].
inline bool intersect_tri(const Tri& tr, const float o[3], const float d[3], float tnear, float tfar,
                          float* t, float* u, float* v) {
  float C[3] = {tr.v0[0] - o[0], tr.v0[1] - o[1], tr.v0[2] - o[2]};
  float R[3];
  cross3(d, C, R);
  float den = dot3(tr.ng, d);
  if (den == 0.f) return false;
  float absDen = std::fabs(den);
  float sgn = den < 0.f ? -1.f : 1.f;
  float U = dot3(R, tr.e2) * sgn;
  float V = dot3(R, tr.e1) * sgn;
  if (!(U >= 0.f && V >= 0.f && U + V <= absDen)) return false;
  float T = dot3(tr.ng, C) * sgn;
  if (!(absDen * tnear < T && T <= absDen * tfar)) return false;
  *t = T / absDen;
  *u = U / absDen;
  *v = V / absDen;
  return true;
}

class BVH {
 public:
  struct Node {
    float lo[3], hi[3];
    int32_t left_or_first;  // inner: index of left child (right = left + 1); leaf: first index into order
    int32_t count;          // 0 for inner nodes
  };

  // positions: T x 9 floats (p0, p1, p2 per triangle) in primID order.
  void build(const float* positions, int num_tris) {
    tris_.resize(num_tris);
    for (int i = 0; i < num_tris; ++i) {
      const float* p = positions + 9 * (size_t)i;
      Tri& tr = tris_[i];
      for (int k = 0; k < 3; ++k) {
        tr.v0[k] = p[k];
        tr.e1[k] = p[k] - p[3 + k];
        tr.e2[k] = p[6 + k] - p[k];
      }
      cross3(tr.e1, tr.e2, tr.ng);
    }
    order_.resize(num_tris);
    for (int i = 0; i < num_tris; ++i) order_[i] = i;
    nodes_.clear();
    if (num_tris == 0) return;
    std::vector<float> lo(3 * (size_t)num_tris), hi(3 * (size_t)num_tris), ce(3 * (size_t)num_tris);
    for (int i = 0; i < num_tris; ++i) {
      const float* p = positions + 9 * (size_t)i;
      for (int k = 0; k < 3; ++k) {
        float a = std::min(std::min(p[k], p[3 + k]), p[6 + k]);
        float b = std::max(std::max(p[k], p[3 + k]), p[6 + k]);
        lo[3 * i + k] = a;
        hi[3 * i + k] = b;
        ce[3 * i + k] = 0.5f * (a + b);
      }
    }
    nodes_.reserve(2 * (size_t)num_tris);
    nodes_.push_back(Node{});
    build_rec(0, 0, num_tris, lo, hi, ce, 0);
  }

  // Closest hit over (tnear, tfar]; ties in t resolve to the lowest primID.
  bool closest(const float o[3], const float d[3], float tnear, float tfar, Hit* out) const {
    Hit best;
    best.t = std::numeric_limits<float>::infinity();
    if (nodes_.empty()) return false;
    int stack[128];
    int sp = 0;
    stack[sp++] = 0;
    while (sp) {
      const Node& n = nodes_[stack[--sp]];
      float bt;
      if (!box_hit(n, o, d, tnear, tfar, &bt) || bt > best.t) continue;
      if (n.count > 0) {
        for (int k = 0; k < n.count; ++k) {
          int prim = order_[n.left_or_first + k];
          float t, u, v;
          if (intersect_tri(tris_[prim], o, d, tnear, tfar, &t, &u, &v)) {
            if (t < best.t || (t == best.t && prim < best.prim)) {
              best.t = t;
              best.u = u;
              best.v = v;
              best.prim = prim;
            }
          }
        }
      } else {
        // Visit the nearer child first.
        float t0 = 0.f, t1 = 0.f;
        bool h0 = box_hit(nodes_[n.left_or_first], o, d, tnear, tfar, &t0);
        bool h1 = box_hit(nodes_[n.left_or_first + 1], o, d, tnear, tfar, &t1);
        if (h0 && h1) {
          if (t0 <= t1) {
            stack[sp++] = n.left_or_first + 1;
            stack[sp++] = n.left_or_first;
          } else {
            stack[sp++] = n.left_or_first;
            stack[sp++] = n.left_or_first + 1;
          }
        } else if (h0) {
          stack[sp++] = n.left_or_first;
        } else if (h1) {
          stack[sp++] = n.left_or_first + 1;
        }
      }
    }
    if (best.prim < 0) return false;
    *out = best;
    return true;
  }

  bool brute_force_closest(const float o[3], const float d[3], float tnear, float tfar, Hit* out) const {
    Hit best;
    best.t = std::numeric_limits<float>::infinity();
    for (int prim = 0; prim < (int)tris_.size(); ++prim) {
      float t, u, v;
      if (intersect_tri(tris_[prim], o, d, tnear, tfar, &t, &u, &v)) {
        if (t < best.t || (t == best.t && prim < best.prim)) {
          best.t = t;
          best.u = u;
          best.v = v;
          best.prim = prim;
        }
      }
    }
    if (best.prim < 0) return false;
    *out = best;
    return true;
  }

  void bounds(float lo[3], float hi[3]) const {
    for (int k = 0; k < 3; ++k) {
      lo[k] = nodes_.empty() ? 0.f : root_lo_[k];
      hi[k] = nodes_.empty() ? 0.f : root_hi_[k];
    }
  }
  int num_tris() const { return (int)tris_.size(); }
  size_t num_nodes() const { return nodes_.size(); }

 private:
  std::vector<Tri> tris_;
  std::vector<int32_t> order_;
  std::vector<Node> nodes_;
  float root_lo_[3] = {0, 0, 0}, root_hi_[3] = {0, 0, 0};

  // Inclusive slab test against a padded box; zero direction components are
  // handled without forming 0 * inf.
  static bool box_hit(const Node& n, const float o[3], const float d[3], float tnear, float tfar, float* tenter) {
    float t0 = tnear, t1 = tfar;
    for (int k = 0; k < 3; ++k) {
      if (d[k] == 0.f) {
        if (o[k] < n.lo[k] || o[k] > n.hi[k]) return false;
        continue;
      }
      float inv = 1.f / d[k];
      float a = (n.lo[k] - o[k]) * inv;
      float b = (n.hi[k] - o[k]) * inv;
      if (a > b) std::swap(a, b);
      // Widen by a few ulps of relative error so rounding never culls a hit.
      a = a - std::fabs(a) * 1e-6f;
      b = b + std::fabs(b) * 1e-6f;
      if (a > t0) t0 = a;
      if (b < t1) t1 = b;
      if (t0 > t1) return false;
    }
    *tenter = t0;
    return true;
  }

  void set_bounds(Node& n, int begin, int end, const std::vector<float>& lo, const std::vector<float>& hi) {
    float a[3] = {INFINITY, INFINITY, INFINITY}, b[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = begin; i < end; ++i) {
      int p = order_[i];
      for (int k = 0; k < 3; ++k) {
        a[k] = std::min(a[k], lo[3 * p + k]);
        b[k] = std::max(b[k], hi[3 * p + k]);
      }
    }
    for (int k = 0; k < 3; ++k) {
      float ext = b[k] - a[k];
      float mag = std::max(std::fabs(a[k]), std::fabs(b[k]));
      float pad = ext * 1e-5f + mag * 1e-6f + 1e-30f;
      n.lo[k] = a[k] - pad;
      n.hi[k] = b[k] + pad;
    }
  }

  void build_rec(int node_idx, int begin, int end, const std::vector<float>& lo, const std::vector<float>& hi,
                 const std::vector<float>& ce, int depth) {
    set_bounds(nodes_[node_idx], begin, end, lo, hi);
    if (node_idx == 0)
      for (int k = 0; k < 3; ++k) {
        root_lo_[k] = nodes_[0].lo[k];
        root_hi_[k] = nodes_[0].hi[k];
      }
    int count = end - begin;
    if (count <= 4 || depth >= 100) {
      nodes_[node_idx].left_or_first = begin;
      nodes_[node_idx].count = count;
      return;
    }
    // Binned SAH over centroid bounds.
    float cl[3] = {INFINITY, INFINITY, INFINITY}, ch[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int i = begin; i < end; ++i) {
      int p = order_[i];
      for (int k = 0; k < 3; ++k) {
        cl[k] = std::min(cl[k], ce[3 * p + k]);
        ch[k] = std::max(ch[k], ce[3 * p + k]);
      }
    }
    const int B = 16;
    int best_axis = -1, best_split = -1;
    float best_cost = INFINITY;
    for (int axis = 0; axis < 3; ++axis) {
      float ext = ch[axis] - cl[axis];
      if (!(ext > 0.f)) continue;
      int cnt[B] = {0};
      float blo[B][3], bhi[B][3];
      for (int b = 0; b < B; ++b)
        for (int k = 0; k < 3; ++k) {
          blo[b][k] = INFINITY;
          bhi[b][k] = -INFINITY;
        }
      for (int i = begin; i < end; ++i) {
        int p = order_[i];
        int b = std::min(B - 1, (int)((ce[3 * p + axis] - cl[axis]) / ext * B));
        cnt[b]++;
        for (int k = 0; k < 3; ++k) {
          blo[b][k] = std::min(blo[b][k], lo[3 * p + k]);
          bhi[b][k] = std::max(bhi[b][k], hi[3 * p + k]);
        }
      }
      float rarea[B];
      int rcnt[B];
      float al[3] = {INFINITY, INFINITY, INFINITY}, ah[3] = {-INFINITY, -INFINITY, -INFINITY};
      int ac = 0;
      for (int b = B - 1; b > 0; --b) {
        ac += cnt[b];
        for (int k = 0; k < 3; ++k) {
          al[k] = std::min(al[k], blo[b][k]);
          ah[k] = std::max(ah[k], bhi[b][k]);
        }
        rcnt[b] = ac;
        rarea[b] = ac ? area(al, ah) : 0.f;
      }
      for (int k = 0; k < 3; ++k) {
        al[k] = INFINITY;
        ah[k] = -INFINITY;
      }
      ac = 0;
      for (int b = 0; b < B - 1; ++b) {
        ac += cnt[b];
        for (int k = 0; k < 3; ++k) {
          al[k] = std::min(al[k], blo[b][k]);
          ah[k] = std::max(ah[k], bhi[b][k]);
        }
        if (ac == 0 || rcnt[b + 1] == 0) continue;
        float cost = area(al, ah) * ac + rarea[b + 1] * rcnt[b + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_split = b;
        }
      }
    }
    int mid;
    if (best_axis < 0) {
      mid = begin + count / 2;  // all centroids coincide: split the list in half
    } else {
      float ext = ch[best_axis] - cl[best_axis];
      auto it = std::partition(order_.begin() + begin, order_.begin() + end, [&](int p) {
        int b = std::min(B - 1, (int)((ce[3 * p + best_axis] - cl[best_axis]) / ext * B));
        return b <= best_split;
      });
      mid = (int)(it - order_.begin());
      if (mid == begin || mid == end) mid = begin + count / 2;
    }
    int left = (int)nodes_.size();
    nodes_.push_back(Node{});
    nodes_.push_back(Node{});
    nodes_[node_idx].left_or_first = left;
    nodes_[node_idx].count = 0;
    build_rec(left, begin, mid, lo, hi, ce, depth + 1);
    build_rec(left + 1, mid, end, lo, hi, ce, depth + 1);
  }

  static float area(const float a[3], const float b[3]) {
    float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    return dx * dy + dy * dz + dz * dx;
  }
};

}  // namespace oracle_bvh
