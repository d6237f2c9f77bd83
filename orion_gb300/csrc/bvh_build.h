// Host SAH BVH build for the GPU traversal kernels.
#pragma once
#include <stdint.h>

#include <vector>

#include "device_types.h"

namespace orion_gb300 {

struct BvhBuildOptions {
  int max_leaf = 4;        // triangles per leaf at most
  int max_depth = kMaxBvhDepth;  // depth bound; deeper subtrees fall back to median splits
  int bins = 32;           // SAH bins per axis
  int top_bfs_nodes = 0;   // the first N node slots hold the top levels in breadth-first order
  int threads = 0;         // build threads, 0 = hardware concurrency
  bool wide = false;       // collapse into the 8-wide quantised BVH (needs max_leaf <= 3)
};

struct BvhBuild {
  std::vector<BvhNode> nodes;    // binary: node 0 is the root; children of an inner node are (a, a+1)
  std::vector<WideNode> wide;    // wide: node 0 is the root (binary `nodes` then left empty)
  std::vector<float> woop;       // 12 floats per triangle (3 x float4), leaf order
  std::vector<int32_t> tri_prim; // leaf order -> primID
  int depth = 0;                 // levels below the root (of the binary tree; bounds the wide tree's)
  int leaves = 0;
  double sah_cost = 0.0;
};

// positions: T x 9 floats in primID order.
void build_bvh(const float* positions, int64_t num_tris, const BvhBuildOptions& opt, BvhBuild* out);

// Woop unit-triangle transform of one triangle (3 x float4 rows). A
// degenerate triangle gets an all-zero record, which never reports a hit.
void woop_record(const float* p9, float out[12]);

}  // namespace orion_gb300
