// Test infrastructure: lets the reference's own renderer compile and run here.
//
// Compiled together with the reference sources (see oracle/ref/Makefile);
// never part of the shipped library. It supplies three things the reference
// gets from places that do not exist on Linux:
//   1. `EmbreeKernel` (src/core/kernel.h:26-45). The reference's methods in
//      src/core/kernel.cpp:44-179 call the closed Embree 2 binary; kernel.cpp
//      is not compiled and these definitions trace with the project CPU BVH
//      (oracle/cpu_bvh.h) instead. The post-hit reconstruction restates
//      kernel.cpp:127-169 (p, uv, ns from barycentrics, ng from the edge cross
//      product, the (u, v, ns) shading frame, `front`, `t`).
//   2. The resource directory (src/util/envvariable.cpp:37-45). The reference
//      prefixes it with the executable path, which on Linux is the full
//      interpreter path; here it is resolved against the directory of the
//      scene file instead (`oracle_set_scene_dir`).
//   3. The progress bar (src/util/renderinfo.cpp:6-50), silenced.
#include <core/geometry.h>
#include <core/intersection.h>
#include <core/kernel.h>
#include <core/primitive.h>
#include <core/triangle.h>
#include <util/envvariable.h>
#include <util/renderinfo.h>

#include <unordered_map>

#include "../cpu_bvh.h"

namespace orion {

// Registry of the last built kernel, so the harness can map hits to primIDs
// and read back the primitives after the parser has erased its own list.
struct ShimKernelState {
  oracle_bvh::BVH bvh;
  std::vector<std::shared_ptr<Primitive>> prims;
  std::unordered_map<const Primitive*, int> index;
};
ShimKernelState* g_last_kernel = nullptr;

static ShimKernelState* state_of(RTCScene s) { return reinterpret_cast<ShimKernelState*>(s); }

EmbreeKernel::EmbreeKernel(const std::vector<std::shared_ptr<Primitive>>& prims) : primitives(prims) {
  rtcDevice = nullptr;
  rtcScene = nullptr;
  geomID = 0;
  build();
  for (const std::shared_ptr<Primitive>& prim : primitives) bound = Union(bound, prim->worldBound());
}

EmbreeKernel::~EmbreeKernel() { clear(); }

void EmbreeKernel::clear() {
  ShimKernelState* st = state_of(rtcScene);
  if (st == g_last_kernel) g_last_kernel = nullptr;
  delete st;
  rtcScene = nullptr;
  primitives.clear();
}

void EmbreeKernel::build() {
  int n = (int)primitives.size();
  std::vector<float> pos(9 * (size_t)n);
  ShimKernelState* st = new ShimKernelState();
  st->prims = primitives;
  for (int i = 0; i < n; ++i) {
    const Triangle& tri = *primitives[i]->triangle;
    for (int k = 0; k < 3; ++k) {
      const Point3f& p = tri.mesh->p[tri.triNumber * 3 + k];
      pos[9 * (size_t)i + 3 * k + 0] = p.x;
      pos[9 * (size_t)i + 3 * k + 1] = p.y;
      pos[9 * (size_t)i + 3 * k + 2] = p.z;
    }
    st->index[primitives[i].get()] = i;
  }
  st->bvh.build(pos.data(), n);
  rtcScene = reinterpret_cast<RTCScene>(st);
  g_last_kernel = st;
}

bool EmbreeKernel::intersect(const Ray& ray, Intersection* isec) const {
  const ShimKernelState* st = state_of(rtcScene);
  float o[3] = {ray.o.x, ray.o.y, ray.o.z};
  float d[3] = {ray.d.x, ray.d.y, ray.d.z};
  oracle_bvh::Hit h;
  if (!st->bvh.closest(o, d, ray.t, ray.tMax, &h)) return false;
  const Primitive& prim = *primitives[h.prim];
  const Triangle& tri = *prim.triangle;
  const int b = tri.triNumber * 3;
  Float cu = h.u, cv = h.v;
  const Point3f& p0 = tri.mesh->p[b];
  const Point3f& p1 = tri.mesh->p[b + 1];
  const Point3f& p2 = tri.mesh->p[b + 2];
  Point3f p = (1 - cu - cv) * p0 + cu * p1 + cv * p2;
  const Point2f& t0 = tri.mesh->uv[b];
  const Point2f& t1 = tri.mesh->uv[b + 1];
  const Point2f& t2 = tri.mesh->uv[b + 2];
  Point2f uv = (1 - cu - cv) * t0 + cu * t1 + cv * t2;
  const Normal3f& n0 = tri.mesh->n[b];
  const Normal3f& n1 = tri.mesh->n[b + 1];
  const Normal3f& n2 = tri.mesh->n[b + 2];
  Normal3f ns = n0 * (1 - cu - cv) + n1 * cu + n2 * cv;
  Normal3f ng = Normal3f(normalize(cross(p1 - p0, p2 - p0)));
  bool front = dot(ray.o - p0, ns) > 0;
  *isec = Intersection(p, ng, ns, uv, h.t, front);
  Vector3f su = normalize(p1 - p0);
  Vector3f sv = normalize(cross(ns, su));
  su = normalize(cross(sv, ns));
  isec->u = su;
  isec->v = sv;
  isec->primitive = &prim;
  return true;
}

Bounds3f EmbreeKernel::worldBound() const { return bound; }

// --- resource directory ---------------------------------------------------
static std::string g_scene_dir;
static std::string g_res_path;

std::string getExecutiveDir() { return g_scene_dir; }
std::string getFullPath(const std::string& name) { return g_scene_dir + name; }
void setResPath(const std::string& path) {
  if (!path.empty() && path[0] == '/')
    g_res_path = path;
  else
    g_res_path = g_scene_dir + path;
}
std::string getResPath() { return g_res_path; }

// --- progress bar ---------------------------------------------------------
void ProcessReporter::outputProgress() {}

}  // namespace orion

extern "C" void oracle_set_scene_dir(const char* dir) {
  orion::g_scene_dir = dir ? dir : "";
  if (!orion::g_scene_dir.empty() && orion::g_scene_dir.back() != '/') orion::g_scene_dir += '/';
}
