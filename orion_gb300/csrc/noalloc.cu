// Ray queries that allocate no device memory: orion_gpu_trace_noalloc.
//
// The same traversal kernel as orion_gpu_trace (k_trace_rays through
// launch_trace), but its ray and hit buffers live in one file-scope static
// device array instead of per-call cudaMalloc/cudaFree. It exists for callers
// that must not allocate: a ray query (picking, a probe) issued from a second
// context while a long render runs on the same device. cudaFree synchronises
// the whole device, so orion_gpu_trace would wait for that render to finish;
// and under the serving loop's memory budget every device byte is already
// accounted for. This entry point waits only for its own stream.
//
// Limits and rules:
//   * at most ORION_NOALLOC_MAX_RAYS rays per call (3 MiB of scratch in all);
//     larger calls are rejected with ORION_ERR_INVALID before any GPU work;
//   * nothing in the scratch needs to start at zero: the kernel writes t, u, v
//     and prim for every ray of the call, and only those are copied back;
//   * the scratch is one array per device per process. Calls on one context
//     are serialised by that context's lock, but calls that overlap on one
//     device from different contexts race on the scratch;
//   * the first call on each device looks up the array's address
//     (cudaGetSymbolAddress, with that device current). That set-up should
//     come before any stream capture on the device.

#include <cuda_runtime.h>

#include <mutex>
#include <string>

#include "../../include/orion_gpu.h"
#include "kernels.h"

namespace orion_gb300 {

namespace {

constexpr int64_t kMaxRays = ORION_NOALLOC_MAX_RAYS;
constexpr size_t kRayBytes = 8 * sizeof(float);          // o.xyz, d.xyz, tmin, tmax
constexpr size_t kHitBytes = 3 * sizeof(float) + sizeof(int);  // t, u, v, prim
constexpr size_t kScratchBytes = (size_t)kMaxRays * (kRayBytes + kHitBytes);
constexpr int kMaxDevices = 64;

// rays [kMaxRays x 8 floats] | t | u | v | prim   (each section 256-byte aligned)
static __device__ __align__(256) unsigned char g_trace_scratch[kScratchBytes];

struct ScratchAddress {
  std::mutex mu;
  unsigned char* ptr[kMaxDevices] = {};
};

ScratchAddress& scratch_address() {
  static ScratchAddress a;
  return a;
}

}  // namespace

// Address of this device's scratch, looked up once per device with that
// device current. Returns a cudaError_t.
int noalloc_trace_scratch(int device, unsigned char** out, std::string* err) {
  if (device < 0 || device >= kMaxDevices) {
    *err = "device ordinal " + std::to_string(device) + " beyond the scratch table";
    return cudaErrorInvalidDevice;
  }
  ScratchAddress& a = scratch_address();
  std::lock_guard<std::mutex> g(a.mu);
  if (!a.ptr[device]) {
    int cur = -1;
    cudaError_t e = cudaGetDevice(&cur);
    const bool switched = e == cudaSuccess && cur != device;
    if (switched) e = cudaSetDevice(device);
    void* p = nullptr;
    if (e == cudaSuccess) e = cudaGetSymbolAddress(&p, g_trace_scratch);
    if (switched) cudaSetDevice(cur);  // the calling thread keeps its current device
    if (e != cudaSuccess) {
      *err = std::string("cudaGetSymbolAddress(trace scratch): ") + cudaGetErrorString(e);
      return e;
    }
    a.ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = a.ptr[device];
  return cudaSuccess;
}

void noalloc_trace_layout(unsigned char* base, float** rays, float** t, float** u, float** v, int** prim) {
  *rays = reinterpret_cast<float*>(base);
  unsigned char* hits = base + (size_t)kMaxRays * kRayBytes;
  *t = reinterpret_cast<float*>(hits);
  *u = reinterpret_cast<float*>(hits + (size_t)kMaxRays * 4);
  *v = reinterpret_cast<float*>(hits + (size_t)kMaxRays * 8);
  *prim = reinterpret_cast<int*>(hits + (size_t)kMaxRays * 12);
}

}  // namespace orion_gb300
