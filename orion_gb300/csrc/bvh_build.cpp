// Binned-SAH BVH build on the host, flattened for the GPU.
//
// Replaces the acceleration structure the reference builds inside Embree
// (EmbreeKernel::build, src/core/kernel.cpp:63-110): one static triangle set
// in primID order. Output layout:
//   * 32-byte nodes (BvhNode); the children of an inner node are an
//     adjacent pair, so one 64-byte fetch gives both child boxes;
//   * optionally the first `top_bfs_nodes` slots hold the top levels in
//     breadth-first order (so a kernel can stage them in shared memory),
//     the rest of each subtree follows depth-first for locality;
//   * Woop unit-triangle records (3 x float4 = 48 bytes) in leaf order, and
//     the leaf-order -> primID map.
// Subtrees below the top levels are built on worker threads.
#include "bvh_build.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <deque>
#include <future>
#include <limits>
#include <mutex>
#include <thread>

namespace orion_gb300 {

void woop_record(const float* p, float out[12]) {
  double v0[3] = {p[0], p[1], p[2]};
  double a[3] = {(double)p[3] - p[0], (double)p[4] - p[1], (double)p[5] - p[2]};  // e1
  double b[3] = {(double)p[6] - p[0], (double)p[7] - p[1], (double)p[8] - p[2]};  // e2
  double c[3] = {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};  // n
  auto cross = [](const double* x, const double* y, double* r) {
    r[0] = x[1] * y[2] - x[2] * y[1];
    r[1] = x[2] * y[0] - x[0] * y[2];
    r[2] = x[0] * y[1] - x[1] * y[0];
  };
  double bc[3], ca[3], ab[3];
  cross(b, c, bc);
  cross(c, a, ca);
  cross(a, b, ab);
  double det = a[0] * bc[0] + a[1] * bc[1] + a[2] * bc[2];
  if (!(std::fabs(det) > 0.0) || !std::isfinite(det)) {
    std::memset(out, 0, 12 * sizeof(float));
    return;
  }
  double r0[3], r1[3], r2[3];
  for (int k = 0; k < 3; ++k) {
    r0[k] = bc[k] / det;  // row giving u (along e1)
    r1[k] = ca[k] / det;  // row giving v (along e2)
    r2[k] = ab[k] / det;  // row giving the offset along n
  }
  // Origin-relative form: the fourth components hold v0, and the kernel
  // works with C = o - v0, so t = -(r2.C) / (r2.d), u = r0.C + t r0.d,
  // v = r1.C + t r1.d. Subtracting v0 first keeps t accurate for ray
  // origins close to the triangle's plane (every secondary ray).
  out[0] = (float)r2[0];
  out[1] = (float)r2[1];
  out[2] = (float)r2[2];
  out[3] = (float)v0[0];
  out[4] = (float)r0[0];
  out[5] = (float)r0[1];
  out[6] = (float)r0[2];
  out[7] = (float)v0[1];
  out[8] = (float)r1[0];
  out[9] = (float)r1[1];
  out[10] = (float)r1[2];
  out[11] = (float)v0[2];
}

namespace {

struct TmpNode {
  float lo[3], hi[3];
  int32_t begin = 0, count = 0;  // leaf range in the reference array
  int32_t first = 0, total = 0;  // the subtree's triangles: refs[first, first + total)
  TmpNode* child[2] = {nullptr, nullptr};
  int depth = 0;
};

// One triangle's box and id, 32 bytes. The build partitions these records
// themselves (not indices into per-triangle arrays), so every scan of a
// range reads memory in order.
struct PrimRef {
  float lo[3];
  int32_t id;
  float hi[3];
  float pad;
  float centroid(int k) const { return 0.5f * (lo[k] + hi[k]); }
};

struct Builder {
  const BvhBuildOptions& opt;
  PrimRef* refs;
  std::mutex arena_mu;
  std::vector<std::unique_ptr<std::deque<TmpNode>>> arenas;
  std::atomic<int> max_depth{0};
  std::atomic<int> leaves{0};
  int spawn_depth;
  int threads;
  std::atomic<int> running{0};  // subtrees building on threads of their own

  Builder(const BvhBuildOptions& o, PrimRef* r, int nthreads) : opt(o), refs(r), threads(nthreads) {
    spawn_depth = 0;
    while ((1 << spawn_depth) < 4 * threads) ++spawn_depth;
  }

  std::deque<TmpNode>* new_arena() {
    std::lock_guard<std::mutex> g(arena_mu);
    arenas.emplace_back(new std::deque<TmpNode>());
    return arenas.back().get();
  }

  static float half_area(const float* a, const float* b) {
    float dx = b[0] - a[0], dy = b[1] - a[1], dz = b[2] - a[2];
    return dx * dy + dy * dz + dz * dx;
  }

  // Ranges above this many primitives are scanned by several threads (the
  // top levels of the tree, which would otherwise run on one thread).
  static constexpr int kParallelScan = 1 << 16;

  // Runs f(b, e, part) over `parts` contiguous pieces of [begin, end) in parallel.
  template <class F>
  static void parallel_parts(int begin, int end, int parts, F f) {
    std::vector<std::thread> th;
    const int64_t n = end - begin;
    for (int t = 0; t < parts; ++t) {
      const int b = begin + (int)(n * t / parts), e = begin + (int)(n * (t + 1) / parts);
      th.emplace_back(f, b, e, t);
    }
    for (auto& x : th) x.join();
  }

  int scan_parts(int count) const {
    if (count < kParallelScan) return 1;
    return std::max(1, std::min(threads, count / (kParallelScan / 4)));
  }

  // Box of the primitives (centroids: the box of their centres) over [begin, end).
  void bounds_range(bool centroids, int begin, int end, float* bl, float* bh) const {
    for (int k = 0; k < 3; ++k) {
      bl[k] = std::numeric_limits<float>::infinity();
      bh[k] = -std::numeric_limits<float>::infinity();
    }
    for (int i = begin; i < end; ++i) {
      const PrimRef& r = refs[i];
      for (int k = 0; k < 3; ++k) {
        const float a = centroids ? r.centroid(k) : r.lo[k], b = centroids ? a : r.hi[k];
        bl[k] = std::min(bl[k], a);
        bh[k] = std::max(bh[k], b);
      }
    }
  }

  // bounds_range, in parallel for large ranges.
  void box_of(bool centroids, int begin, int end, float* bl, float* bh) const {
    const int parts = scan_parts(end - begin);
    if (parts == 1) return bounds_range(centroids, begin, end, bl, bh);
    std::vector<float> r(6 * (size_t)parts);
    parallel_parts(begin, end, parts,
                   [&](int s, int e, int t) { bounds_range(centroids, s, e, &r[6 * t], &r[6 * t + 3]); });
    for (int k = 0; k < 3; ++k) {
      bl[k] = std::numeric_limits<float>::infinity();
      bh[k] = -std::numeric_limits<float>::infinity();
    }
    for (int t = 0; t < parts; ++t)
      for (int k = 0; k < 3; ++k) {
        bl[k] = std::min(bl[k], r[6 * t + k]);
        bh[k] = std::max(bh[k], r[6 * t + 3 + k]);
      }
  }

  void bounds(int begin, int end, float* bl, float* bh) const { box_of(false, begin, end, bl, bh); }

  TmpNode* build(int begin, int end, int depth, std::deque<TmpNode>* arena) {
    arena->emplace_back();
    TmpNode* n = &arena->back();
    n->depth = depth;
    bounds(begin, end, n->lo, n->hi);
    int count = end - begin;
    n->first = begin;
    n->total = count;
    int cur = max_depth.load();
    while (depth > cur && !max_depth.compare_exchange_weak(cur, depth)) {
    }
    if (count <= 1) return make_leaf(n, begin, count);
    // Remaining depth a balanced split would need from here.
    int need = 0;
    while (((int64_t)opt.max_leaf << need) < count) ++need;
    bool forced_median = depth + need + 1 >= opt.max_depth;
    int mid = -1;
    if (!forced_median) {
      float cost_leaf = (float)count;
      float split_cost;
      mid = sah_split(begin, end, n, &split_cost);
      if (mid < 0 || (count <= opt.max_leaf && cost_leaf <= split_cost)) {
        if (count <= opt.max_leaf) return make_leaf(n, begin, count);
        mid = -1;
      }
    }
    if (mid < 0) mid = median_split(begin, end);
    // A subtree goes to a new thread while fewer than 2 x threads are busy, so
    // uneven SAH splits still keep every core working.
    bool spawn = false;
    if (count > 8192) {
      int live = running.load();
      while (live < 2 * threads && !(spawn = running.compare_exchange_weak(live, live + 1))) {
      }
    }
    if (spawn) {
      auto fut = std::async(std::launch::async, [=] {
        std::deque<TmpNode>* a2 = new_arena();
        TmpNode* r = build(begin, mid, depth + 1, a2);
        running.fetch_sub(1);
        return r;
      });
      n->child[1] = build(mid, end, depth + 1, arena);
      n->child[0] = fut.get();
    } else {
      n->child[0] = build(begin, mid, depth + 1, arena);
      n->child[1] = build(mid, end, depth + 1, arena);
    }
    return n;
  }

  TmpNode* make_leaf(TmpNode* n, int begin, int count) {
    n->begin = begin;
    n->count = count;
    leaves.fetch_add(1);
    return n;
  }

  int median_split(int begin, int end) {
    float cl[3], ch[3];
    centroid_bounds(begin, end, cl, ch);
    int axis = 0;
    for (int k = 1; k < 3; ++k)
      if (ch[k] - cl[k] > ch[axis] - cl[axis]) axis = k;
    int mid = begin + (end - begin) / 2;
    std::nth_element(refs + begin, refs + mid, refs + end,
                     [&](const PrimRef& a, const PrimRef& b) { return a.centroid(axis) < b.centroid(axis); });
    return mid;
  }

  void centroid_bounds(int begin, int end, float* cl, float* ch) const { box_of(true, begin, end, cl, ch); }

  struct Bins {
    int cnt[3][64];
    float blo[3][64][3], bhi[3][64][3];
    void clear(int B) {
      for (int axis = 0; axis < 3; ++axis)
        for (int b = 0; b < B; ++b) {
          cnt[axis][b] = 0;
          for (int k = 0; k < 3; ++k) {
            blo[axis][b][k] = std::numeric_limits<float>::infinity();
            bhi[axis][b][k] = -std::numeric_limits<float>::infinity();
          }
        }
    }
  };

  void bin_range(int begin, int end, int B, const float* cl, const float* scale, Bins& bins) const {
    bins.clear(B);
    for (int i = begin; i < end; ++i) {
      const PrimRef& r = refs[i];
      for (int axis = 0; axis < 3; ++axis) {
        if (scale[axis] == 0.f) continue;
        int b = std::min(B - 1, (int)((r.centroid(axis) - cl[axis]) * scale[axis]));
        bins.cnt[axis][b]++;
        for (int k = 0; k < 3; ++k) {
          bins.blo[axis][b][k] = std::min(bins.blo[axis][b][k], r.lo[k]);
          bins.bhi[axis][b][k] = std::max(bins.bhi[axis][b][k], r.hi[k]);
        }
      }
    }
  }

  // Returns the partition point of the best binned SAH split, or -1.
  int sah_split(int begin, int end, const TmpNode* n, float* best_cost_out) {
    // Small ranges get as many bins as primitives (at least 4): the per-bin
    // clear and sweep would otherwise dominate near the leaves.
    const int B = std::max(2, std::min(std::min(opt.bins, 64), std::max(4, end - begin)));
    float cl[3], ch[3];
    centroid_bounds(begin, end, cl, ch);
    float parent_area = half_area(n->lo, n->hi);
    int best_axis = -1, best_bin = -1;
    float best_cost = std::numeric_limits<float>::infinity();
    float scale[3];
    for (int axis = 0; axis < 3; ++axis) {
      float ext = ch[axis] - cl[axis];
      scale[axis] = ext > 0.f ? B / ext : 0.f;
    }
    Bins all;
    const int parts = scan_parts(end - begin);
    if (parts == 1) {
      bin_range(begin, end, B, cl, scale, all);
    } else {  // per-thread bins, merged (counts add, boxes union: independent of timing)
      std::vector<Bins> part(parts);
      parallel_parts(begin, end, parts, [&](int s, int e, int t) { bin_range(s, e, B, cl, scale, part[t]); });
      all.clear(B);
      for (const Bins& pb : part)
        for (int axis = 0; axis < 3; ++axis)
          for (int b = 0; b < B; ++b) {
            all.cnt[axis][b] += pb.cnt[axis][b];
            for (int k = 0; k < 3; ++k) {
              all.blo[axis][b][k] = std::min(all.blo[axis][b][k], pb.blo[axis][b][k]);
              all.bhi[axis][b][k] = std::max(all.bhi[axis][b][k], pb.bhi[axis][b][k]);
            }
          }
    }
    auto& cnt = all.cnt;
    auto& blo = all.blo;
    auto& bhi = all.bhi;
    for (int axis = 0; axis < 3; ++axis) {
      if (scale[axis] == 0.f) continue;
      float rarea[64];
      int rcnt[64];
      float al[3], ah[3];
      for (int k = 0; k < 3; ++k) {
        al[k] = std::numeric_limits<float>::infinity();
        ah[k] = -std::numeric_limits<float>::infinity();
      }
      int ac = 0;
      for (int b = B - 1; b > 0; --b) {
        ac += cnt[axis][b];
        for (int k = 0; k < 3; ++k) {
          al[k] = std::min(al[k], blo[axis][b][k]);
          ah[k] = std::max(ah[k], bhi[axis][b][k]);
        }
        rcnt[b] = ac;
        rarea[b] = ac ? half_area(al, ah) : 0.f;
      }
      for (int k = 0; k < 3; ++k) {
        al[k] = std::numeric_limits<float>::infinity();
        ah[k] = -std::numeric_limits<float>::infinity();
      }
      ac = 0;
      for (int b = 0; b < B - 1; ++b) {
        ac += cnt[axis][b];
        for (int k = 0; k < 3; ++k) {
          al[k] = std::min(al[k], blo[axis][b][k]);
          ah[k] = std::max(ah[k], bhi[axis][b][k]);
        }
        if (ac == 0 || rcnt[b + 1] == 0) continue;
        float cost = half_area(al, ah) * ac + rarea[b + 1] * rcnt[b + 1];
        if (cost < best_cost) {
          best_cost = cost;
          best_axis = axis;
          best_bin = b;
        }
      }
    }
    if (best_axis < 0) return -1;
    *best_cost_out = parent_area > 0.f ? 1.f + best_cost / parent_area : 1.f;
    float s = scale[best_axis], c0 = cl[best_axis];
    PrimRef* it = std::partition(refs + begin, refs + end, [&](const PrimRef& r) {
      int b = std::min(B - 1, (int)((r.centroid(best_axis) - c0) * s));
      return b <= best_bin;
    });
    int mid = (int)(it - refs);
    if (mid == begin || mid == end) return -1;
    return mid;
  }
};

void write_node(BvhNode* dst, const TmpNode* n) {
  for (int k = 0; k < 3; ++k) {
    float ext = n->hi[k] - n->lo[k];
    float mag = std::max(std::fabs(n->lo[k]), std::fabs(n->hi[k]));
    float pad = ext * 1e-6f + mag * 2e-7f;
    dst->lo[k] = n->lo[k] - pad;
    dst->hi[k] = n->hi[k] + pad;
  }
  dst->a = n->count > 0 ? n->begin : 0;
  dst->b = n->count;
}

struct Flattener {
  std::vector<BvhNode>& out;
  explicit Flattener(std::vector<BvhNode>& o) : out(o) {}
  int alloc_pair() {
    int i = (int)out.size();
    out.resize(out.size() + 2);
    return i;
  }
  void dfs(const TmpNode* n, int idx) {
    write_node(&out[idx], n);
    if (n->count > 0) return;
    int c = alloc_pair();
    out[idx].a = c;
    out[idx].b = 0;
    dfs(n->child[0], c);
    dfs(n->child[1], c + 1);
  }
  void run(const TmpNode* root, int top_bfs) {
    out.resize(1);
    if (top_bfs <= 1) {
      dfs(root, 0);
      return;
    }
    // Breadth-first for the first `top_bfs` slots, then depth-first below.
    std::vector<std::pair<const TmpNode*, int>> level{{root, 0}}, frontier;
    write_node(&out[0], root);
    while (!level.empty()) {
      std::vector<std::pair<const TmpNode*, int>> next;
      for (auto& e : level) {
        const TmpNode* n = e.first;
        if (n->count > 0) continue;
        if ((int)out.size() + 2 <= top_bfs) {
          int c = alloc_pair();
          out[e.second].a = c;
          out[e.second].b = 0;
          write_node(&out[c], n->child[0]);
          write_node(&out[c + 1], n->child[1]);
          next.push_back({n->child[0], c});
          next.push_back({n->child[1], c + 1});
        } else {
          frontier.push_back(e);
        }
      }
      level.swap(next);
      if ((int)out.size() + 2 > top_bfs) {
        for (auto& e : level)
          if (e.first->count == 0) frontier.push_back(e);
        break;
      }
    }
    for (auto& e : frontier) dfs(e.first, e.second);
  }
};

// Collapses the binary tree into 8-wide nodes. Each wide node takes the
// children of a binary node and keeps opening its internal child of largest
// surface area until it has 8 children or only leaves; children are placed
// in slots by the direction of their centre from the node's centre (the
// slot order a ray visits depends on its octant); boxes are padded like the
// binary nodes' and quantised outwards.
struct WideCollapser {
  const int32_t* order;            // binary leaf order -> primID
  std::vector<WideNode>& out;
  std::vector<int32_t>& tris;      // wide leaf order -> primID

  static void padded(const TmpNode* n, double lo[3], double hi[3]) {
    BvhNode b;
    write_node(&b, n);
    for (int k = 0; k < 3; ++k) {
      lo[k] = b.lo[k];
      hi[k] = b.hi[k];
    }
  }

  static double area(const TmpNode* n) {
    float dx = n->hi[0] - n->lo[0], dy = n->hi[1] - n->lo[1], dz = n->hi[2] - n->lo[2];
    return (double)dx * dy + (double)dy * dz + (double)dz * dx;
  }

  // A child becomes a leaf slot when its subtree holds at most kWideLeaf triangles.
  static constexpr int kWideLeaf = 3;
  static bool is_leaf(const TmpNode* n) { return n->total <= kWideLeaf; }

  void gather(const TmpNode* n, std::vector<const TmpNode*>& ch) const {
    ch.clear();
    if (is_leaf(n)) {  // a small root: one leaf child
      ch.push_back(n);
      return;
    }
    ch.push_back(n->child[0]);
    ch.push_back(n->child[1]);
    while (ch.size() < 8) {
      int best = -1;
      double best_a = -1.0;
      for (int i = 0; i < (int)ch.size(); ++i)
        if (!is_leaf(ch[i]) && area(ch[i]) > best_a) {
          best_a = area(ch[i]);
          best = i;
        }
      if (best < 0) break;
      const TmpNode* c = ch[best];
      ch[best] = c->child[0];
      ch.push_back(c->child[1]);
    }
    // Slots left over: split leaf-sized subtrees too, for tighter leaf boxes.
    while (ch.size() < 8) {
      int best = -1;
      double best_a = -1.0;
      for (int i = 0; i < (int)ch.size(); ++i)
        if (ch[i]->count == 0 && ch[i]->child[0] && area(ch[i]) > best_a) {
          best_a = area(ch[i]);
          best = i;
        }
      if (best < 0) break;
      const TmpNode* c = ch[best];
      ch[best] = c->child[0];
      ch.push_back(c->child[1]);
    }
  }

  // Slot of each child: greedy matching of child directions to the eight
  // octant directions of the slots.
  static void assign_slots(const std::vector<const TmpNode*>& ch, const double nlo[3], const double nhi[3],
                           int slot_of[8]) {
    const int m = (int)ch.size();
    double score[8][8];
    for (int c = 0; c < m; ++c) {
      double off[3];
      for (int k = 0; k < 3; ++k)
        off[k] = 0.5 * ((double)ch[c]->lo[k] + ch[c]->hi[k]) - 0.5 * (nlo[k] + nhi[k]);
      for (int s = 0; s < 8; ++s) {
        double v = 0.0;
        for (int k = 0; k < 3; ++k) v += ((s >> k) & 1) ? off[k] : -off[k];
        score[c][s] = v;
      }
    }
    bool used_c[8] = {}, used_s[8] = {};
    for (int it = 0; it < m; ++it) {
      int bc = -1, bs = -1;
      double bv = -std::numeric_limits<double>::infinity();
      for (int c = 0; c < m; ++c) {
        if (used_c[c]) continue;
        for (int s = 0; s < 8; ++s)
          if (!used_s[s] && score[c][s] > bv) {
            bv = score[c][s];
            bc = c;
            bs = s;
          }
      }
      used_c[bc] = used_s[bs] = true;
      slot_of[bc] = bs;
    }
  }

  // Builds the wide node of binary node `n` into `w`: its internal children
  // get placeholder slots appended to `nodes` (from w.child_base) and are
  // returned in `kids` in slot order; its leaf triangles are appended to `tris`.
  void fill_node(const TmpNode* n, WideNode& w, std::vector<WideNode>& nodes, std::vector<int32_t>& tris,
                 const TmpNode* kids[8], int* nkids) const {
    std::vector<const TmpNode*> ch;
    ch.reserve(8);
    gather(n, ch);
    const int m = (int)ch.size();
    double clo[8][3], chi[8][3], nlo[3], nhi[3];
    for (int k = 0; k < 3; ++k) {
      nlo[k] = std::numeric_limits<double>::infinity();
      nhi[k] = -std::numeric_limits<double>::infinity();
    }
    for (int c = 0; c < m; ++c) {
      padded(ch[c], clo[c], chi[c]);
      for (int k = 0; k < 3; ++k) {
        nlo[k] = std::min(nlo[k], clo[c][k]);
        nhi[k] = std::max(nhi[k], chi[c][k]);
      }
    }
    int slot_of[8];
    assign_slots(ch, nlo, nhi, slot_of);
    const TmpNode* in_slot[8] = {};
    int child_of_slot[8];
    for (int c = 0; c < m; ++c) {
      in_slot[slot_of[c]] = ch[c];
      child_of_slot[slot_of[c]] = c;
    }
    std::memset(&w, 0, sizeof(w));
    // Empty slots get inverted boxes (lo = 255 > hi = 0 on every axis), which
    // no ray hits whatever its direction.
    std::memset(w.qlo, 0xff, sizeof(w.qlo));
    // Quantisation grid per axis: the smallest power-of-two cell with 255 cells
    // covering the node, at most 2^112 (the traversal scales cells by 2^15).
    double cell[3];
    for (int k = 0; k < 3; ++k) {
      w.p[k] = (float)nlo[k];
      if ((double)w.p[k] > nlo[k]) w.p[k] = std::nextafter(w.p[k], -std::numeric_limits<float>::infinity());
      const double ext = nhi[k] - (double)w.p[k];
      int e = -126;
      if (ext > 0.0) {
        int ex;
        const double m = std::frexp(ext / 255.0, &ex);  // ext / 255 = m * 2^ex, m in [0.5, 1)
        e = std::max(-126, std::min(112, m == 0.5 ? ex - 1 : ex));
      }
      while (e < 112 && std::ldexp(255.0, e) < ext) ++e;  // guards the rounding of ext / 255
      w.e[k] = (uint8_t)(e + 127);
      cell[k] = std::ldexp(1.0, e);
    }
    // Internal children first (their node slots), then leaf triangles.
    int n_internal = 0;
    for (int s = 0; s < 8; ++s)
      if (in_slot[s] && !is_leaf(in_slot[s])) ++n_internal;
    const int child_base = (int)nodes.size();
    nodes.resize(nodes.size() + n_internal);
    w.child_base = child_base;
    w.tri_base = (int)tris.size();
    for (int s = 0; s < 8; ++s) {
      const TmpNode* c = in_slot[s];
      if (!c) continue;
      const int ci = child_of_slot[s];
      for (int k = 0; k < 3; ++k) {
        double ql = std::floor((clo[ci][k] - w.p[k]) / cell[k]);
        double qh = std::ceil((chi[ci][k] - w.p[k]) / cell[k]);
        ql = std::max(0.0, std::min(255.0, ql));
        qh = std::max(0.0, std::min(255.0, qh));
        while (ql > 0.0 && (double)w.p[k] + ql * cell[k] > clo[ci][k]) ql -= 1.0;
        while (qh < 255.0 && (double)w.p[k] + qh * cell[k] < chi[ci][k]) qh += 1.0;
        w.qlo[k][s] = (uint8_t)ql;
        w.qhi[k][s] = (uint8_t)qh;
      }
      if (!is_leaf(c)) {
        w.imask |= (uint8_t)(1u << s);
        w.meta[s] = 0x80;
      } else {
        const int off = (int)tris.size() - w.tri_base;
        w.meta[s] = (uint8_t)((c->total << 5) | off);
        for (int i = 0; i < c->total; ++i) tris.push_back(order[c->first + i]);
      }
    }
    *nkids = 0;
    for (int s = 0; s < 8; ++s)
      if (in_slot[s] && !is_leaf(in_slot[s])) kids[(*nkids)++] = in_slot[s];
  }

  // The wide subtree of `n` into nodes[idx] and below, depth first.
  void fill(int idx, const TmpNode* n, std::vector<WideNode>& nodes, std::vector<int32_t>& tris) const {
    WideNode w;
    const TmpNode* kids[8];
    int nk;
    fill_node(n, w, nodes, tris, kids, &nk);
    nodes[idx] = w;
    for (int r = 0; r < nk; ++r) fill(w.child_base + r, kids[r], nodes, tris);
  }

  // The top levels breadth first on this thread until there are enough
  // subtrees for every core, then the subtrees in parallel, each into arrays
  // of its own, appended in order with their child and triangle bases shifted.
  void run(const TmpNode* root, int threads) {
    out.assign(1, WideNode{});
    std::vector<std::pair<int, const TmpNode*>> frontier{{0, root}}, next;
    for (int level = 0; level < 6 && !frontier.empty() && (int)frontier.size() < 4 * threads; ++level) {
      next.clear();
      for (auto& f : frontier) {
        WideNode w;
        const TmpNode* kids[8];
        int nk;
        fill_node(f.second, w, out, tris, kids, &nk);
        out[f.first] = w;
        for (int r = 0; r < nk; ++r) next.push_back({w.child_base + r, kids[r]});
      }
      frontier.swap(next);
    }
    struct Task {
      int idx;
      const TmpNode* n;
      WideNode root;
      std::vector<WideNode> nodes;
      std::vector<int32_t> tris;
    };
    std::vector<Task> tasks(frontier.size());
    std::atomic<int> next_task{0};
    auto worker = [&](int, int, int) {
      for (int t; (t = next_task.fetch_add(1)) < (int)tasks.size();) {
        Task& tk = tasks[t];
        tk.idx = frontier[t].first;
        tk.n = frontier[t].second;
        const TmpNode* kids[8];
        int nk;
        fill_node(tk.n, tk.root, tk.nodes, tk.tris, kids, &nk);
        for (int r = 0; r < nk; ++r) fill(tk.root.child_base + r, kids[r], tk.nodes, tk.tris);
      }
    };
    if (!tasks.empty()) Builder::parallel_parts(0, threads, std::max(1, std::min(threads, (int)tasks.size())), worker);
    for (Task& tk : tasks) {
      const int node_off = (int)out.size(), tri_off = (int)tris.size();
      for (WideNode& w : tk.nodes) {
        w.child_base += node_off;
        w.tri_base += tri_off;
      }
      tk.root.child_base += node_off;
      tk.root.tri_base += tri_off;
      out[tk.idx] = tk.root;
      out.insert(out.end(), tk.nodes.begin(), tk.nodes.end());
      tris.insert(tris.end(), tk.tris.begin(), tk.tris.end());
    }
  }
};

}  // namespace

void build_bvh(const float* positions, int64_t num_tris, const BvhBuildOptions& opt, BvhBuild* out) {
  const int T = (int)num_tris;
  out->nodes.clear();
  out->woop.assign(12 * (size_t)T, 0.f);
  out->tri_prim.resize(T);
  out->depth = 0;
  out->leaves = 0;
  out->wide.clear();
  if (T == 0 && opt.wide) {
    WideNode empty;
    std::memset(&empty, 0, sizeof(empty));  // no slot in use, inverted boxes: nothing hits
    std::memset(empty.qlo, 0xff, sizeof(empty.qlo));
    for (int k = 0; k < 3; ++k) empty.e[k] = 127;
    out->wide.push_back(empty);
    return;
  }
  if (T == 0) {
    BvhNode empty;
    std::memset(&empty, 0, sizeof(empty));
    for (int k = 0; k < 3; ++k) {
      empty.lo[k] = 1.f;
      empty.hi[k] = -1.f;  // inverted box: nothing hits
    }
    out->nodes.push_back(empty);
    return;
  }
  int threads = opt.threads > 0 ? opt.threads : (int)std::max(1u, std::thread::hardware_concurrency());
  std::vector<PrimRef> refs(T);
  Builder::parallel_parts(0, T, std::max(1, std::min(threads, T / 4096)), [&](int s, int e, int) {
    for (int i = s; i < e; ++i) {
      const float* p = positions + 9 * (size_t)i;
      PrimRef& r = refs[i];
      for (int k = 0; k < 3; ++k) {
        r.lo[k] = std::min(std::min(p[k], p[3 + k]), p[6 + k]);
        r.hi[k] = std::max(std::max(p[k], p[3 + k]), p[6 + k]);
      }
      r.id = i;
      r.pad = 0.f;
    }
  });
  Builder b(opt, refs.data(), threads);
  std::deque<TmpNode>* arena = b.new_arena();
  TmpNode* root = b.build(0, T, 0, arena);
  out->depth = b.max_depth.load();
  out->leaves = b.leaves.load();
  std::vector<int32_t> order(T);  // binary leaf order -> primID
  for (int i = 0; i < T; ++i) order[i] = refs[i].id;
  // Woop records of triangles in `ids` order, in parallel.
  auto records = [&](const std::vector<int32_t>& ids) {
    Builder::parallel_parts(0, T, std::max(1, std::min(threads, T / 4096)), [&](int s, int e, int) {
      for (int i = s; i < e; ++i) {
        out->tri_prim[i] = ids[i];
        woop_record(positions + 9 * (size_t)ids[i], &out->woop[12 * (size_t)i]);
      }
    });
  };
  if (opt.wide) {
    std::vector<int32_t> tris;
    tris.reserve(T);
    WideCollapser wc{order.data(), out->wide, tris};
    wc.run(root, threads);
    records(tris);
    return;
  }
  Flattener fl(out->nodes);
  fl.run(root, opt.top_bfs_nodes);
  records(order);
  // SAH cost of the result (traversal + intersection, relative to the root).
  double root_area = Builder::half_area(out->nodes[0].lo, out->nodes[0].hi);
  double cost = 0.0;
  for (const BvhNode& n : out->nodes) {
    double a = Builder::half_area(n.lo, n.hi) / (root_area > 0 ? root_area : 1.0);
    cost += n.b > 0 ? a * n.b : a;
  }
  out->sah_cost = cost;
}

}  // namespace orion_gb300
