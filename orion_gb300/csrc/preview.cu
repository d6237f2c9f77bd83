// Progressive preview: a request's FP64 film averaged and quantised to the
// 8-bit pixels saveAsBmp writes (src/core/texture.cpp:77-136) on the device,
// so a preview moves 4 bytes a pixel to the host instead of the 52 of the
// film (sums, sums of squares, counts).
#include <cuda_runtime.h>

#include <algorithm>

#include "kernels.h"

namespace orion_gb300 {

namespace {

// clamp(c, 0, 1) * 255 truncated; NaN becomes 0 (as the host BMP writer).
__device__ __forceinline__ uint8_t to_byte(float f) {
  if (!(f > 0.f)) f = 0.f;
  if (f > 1.f) f = 1.f;
  return (uint8_t)__float2int_rz(__fmul_rn(f, 255.f));
}

__global__ void k_film_preview(const double* __restrict__ sum, const uint32_t* __restrict__ count, int width,
                               int height, int bottom_up, uchar4* __restrict__ out) {
  const int64_t n = (int64_t)width * height;
  for (int64_t p = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; p < n; p += (int64_t)gridDim.x * blockDim.x) {
    const int j = (int)(p / width), i = (int)(p % width);
    const uint32_t c = count[p];
    uchar4 px = make_uchar4(0, 0, 0, 255);
    if (c > 0) {
      // RenderTarget::getAveraged (src/texture/rendertarget.cpp:28-37): sum / count
      const double* s = sum + 3 * p;
      px.x = to_byte((float)(s[2] / c));
      px.y = to_byte((float)(s[1] / c));
      px.z = to_byte((float)(s[0] / c));
    }
    const int row = bottom_up ? height - 1 - j : j;
    out[(int64_t)row * width + i] = px;
  }
}

}  // namespace

void launch_film_preview(const double* sum, const uint32_t* count, int width, int height, int bottom_up,
                         uint8_t* bgra, cudaStream_t stream) {
  const int64_t n = (int64_t)width * height;
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  k_film_preview<<<grid > 0 ? grid : 1, 256, 0, stream>>>(sum, count, width, height, bottom_up,
                                                          reinterpret_cast<uchar4*>(bgra));
}

}  // namespace orion_gb300
