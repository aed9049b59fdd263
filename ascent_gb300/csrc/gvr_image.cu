// gvr_image.cu — the canvas-to-PNG pixel conversion on the device.
//
// PNGEncoder::Encode(const float *) (png_utils/ascent_png_encoder.cpp:77-118)
// turns the float canvas into the 8-bit rows lodepng compresses: rows are
// flipped (the canvas has y up, PNG rows run top down) and every channel
// becomes (unsigned char)(value * 255.f), a truncating conversion. Here one
// thread converts one pixel: a 16-byte load and a 4-byte store, so the pass
// streams W*H*20 bytes; the deflate of the PNG itself stays on the host.
// Values are clamped to [0, 255] before the truncation (the reference's cast
// of an out-of-range float is undefined; the canvas holds values in [0, 1]).
#include <cstdint>

#include "gvr_internal.h"

namespace gvr {
namespace {

__global__ void __launch_bounds__(256)
rgba8_kernel(const float4 *__restrict__ rgba, int width, int height, uchar4 *__restrict__ out)
{
  const int64_t n = (int64_t)width * height;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int y = (int)(i / width), x = (int)(i - (int64_t)y * width);
    const float4 v = rgba[i];
    auto q = [](float c) {
      return (unsigned char)__float2uint_rz(fminf(fmaxf(c * 255.f, 0.f), 255.f));
    };
    out[(int64_t)(height - 1 - y) * width + x] = make_uchar4(q(v.x), q(v.y), q(v.z), q(v.w));
  }
}

}  // namespace
}  // namespace gvr

using namespace gvr;

extern "C" int gvr_canvas_to_rgba8(const float *rgba, int width, int height, uint8_t *out,
                                   int location, void *stream)
{
  if (!rgba || !out) return set_error(GVR_ERR_INVALID_ARGUMENT, "image buffers are NULL");
  if (width < 1 || height < 1 || (int64_t)width * height > (1ll << 28))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image size must be >= 1 and <= 2^28 pixels");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad location");
  const int64_t pixels = (int64_t)width * height;
  cudaStream_t st = (cudaStream_t)stream;
  const float4 *d_in = reinterpret_cast<const float4 *>(rgba);
  uchar4 *d_out = reinterpret_cast<uchar4 *>(out);
  void *scratch = nullptr;
  cudaError_t e = cudaSuccess;
  if (location == GVR_MEM_HOST) {
    e = scratch_alloc(&scratch, (size_t)pixels * (sizeof(float4) + sizeof(uchar4)), st);
    if (e != cudaSuccess) return cuda_error(e, "allocate image scratch");
    d_in = static_cast<const float4 *>(scratch);
    d_out = reinterpret_cast<uchar4 *>(static_cast<float4 *>(scratch) + pixels);
    e = cudaMemcpyAsync(const_cast<float4 *>(d_in), rgba, sizeof(float4) * pixels,
                        cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) {
    const int grid = (int)std::min<int64_t>((pixels + 255) / 256, 152 * 8);
    rgba8_kernel<<<grid, 256, 0, st>>>(d_in, width, height, d_out);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && location == GVR_MEM_HOST) {
    e = cudaMemcpyAsync(out, d_out, sizeof(uchar4) * pixels, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (scratch) cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cuda_error(e, "canvas to rgba8");
  return GVR_OK;
}
