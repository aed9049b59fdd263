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
//
// Also here: the Z-buffer compositing of opaque canvases (surface plots
// rendered per domain or per plot) that Renderer::Composite does in
// Z_BUFFER_SURFACE mode before the volume pass draws over the result
// (Renderer.cpp:111-142, Compositor.cpp:86-125, ImageCompositor.hpp:49-76,
// Image.hpp:80-113, Renderer::ImageToCanvas :271-289). One thread per pixel
// walks the images in order: each image's colour goes through the 8-bit
// vtkh::Image (truncation), its depth through |depth|; image i > 0 replaces
// the kept pixel where its depth is <= 1 and not behind the kept depth; the
// kept 8-bit colour comes back as value / 255 with its depth.
#include <cmath>
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

// Colour bar body: every pixel of the bar's pixel rectangle takes the
// colour-table entry of its position along the bar's long axis (opaque);
// the rectangle's outermost pixels take the foreground colour.
__global__ void __launch_bounds__(256)
color_bar_kernel(float4 *__restrict__ rgba, int width, int x0, int y0, int bw, int bh,
                 const float4 *__restrict__ lut, int n, int vertical, float4 fg)
{
  const int64_t count = (int64_t)bw * bh;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < count;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int lx = (int)(i % bw), ly = (int)(i / bw);
    float4 c;
    if (lx == 0 || ly == 0 || lx == bw - 1 || ly == bh - 1) {
      c = fg;
    } else {
      const float t = vertical ? ((float)ly + 0.5f) / (float)bh : ((float)lx + 0.5f) / (float)bw;
      const float4 e = lut[min((int)(t * (float)n), n - 1)];
      c = make_float4(e.x, e.y, e.z, 1.f);
    }
    rgba[(int64_t)(y0 + ly) * width + (x0 + lx)] = c;
  }
}

constexpr int kMaxZImages = 64;

struct ZImages {
  const float4 *rgba[kMaxZImages];
  const float *depth[kMaxZImages];
};

__device__ __forceinline__ uchar4 to_u8(float4 v)
{
  auto q = [](float c) {
    return (unsigned char)__float2uint_rz(fminf(fmaxf(c * 255.f, 0.f), 255.f));
  };
  return make_uchar4(q(v.x), q(v.y), q(v.z), q(v.w));
}

__global__ void __launch_bounds__(256)
zbuffer_kernel(const ZImages images, int n_images, int64_t n, float4 *__restrict__ out_rgba,
               float *__restrict__ out_depth)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    // Image::Init of the first image: 8-bit colour, |depth|; each later
    // image that passes ZBufferComposite's test replaces both, so the
    // result is the last winner's colour: the depths are tested first (all
    // loads independent) and only the winner's colour is read
    float d = fabsf(images.depth[0][i]);
    int win = 0;
#pragma unroll 8
    for (int k = 1; k < n_images; ++k) {
      const float dk = fabsf(images.depth[k][i]);
      if (dk > 1.f || d < dk) continue;   // ZBufferComposite's test
      d = dk;
      win = k;
    }
    const uchar4 c = to_u8(images.rgba[win][i]);
    const float s = 1.f / 255.f;          // ImageToCanvas
    out_rgba[i] = make_float4((float)c.x * s, (float)c.y * s, (float)c.z * s, (float)c.w * s);
    out_depth[i] = d;
  }
}

}  // namespace
}  // namespace gvr

using namespace gvr;

extern "C" int gvr_zbuffer_composite(int n_images, const float *const *rgba,
                                     const float *const *depth, int width, int height,
                                     float *out_rgba, float *out_depth, int location, void *stream)
{
  if (n_images < 1 || n_images > kMaxZImages)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "n_images must be 1 .. 64");
  if (!rgba || !depth || !out_rgba || !out_depth)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image buffers are NULL");
  for (int k = 0; k < n_images; ++k)
    if (!rgba[k] || !depth[k]) return set_error(GVR_ERR_INVALID_ARGUMENT, "image buffers are NULL");
  if (width < 1 || height < 1 || (int64_t)width * height > (1ll << 28))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image size must be >= 1 and <= 2^28 pixels");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad location");
  const int64_t pixels = (int64_t)width * height;
  // one canvas per block: colour (16-byte aligned) then depth; blocks padded
  // to 256 bytes so that every colour array stays float4-aligned
  const size_t per = ((size_t)pixels * (sizeof(float4) + sizeof(float)) + 255) & ~(size_t)255;
  cudaStream_t st = (cudaStream_t)stream;
  ZImages im{};
  float4 *d_out = reinterpret_cast<float4 *>(out_rgba);
  float *d_dep = out_depth;
  void *scratch = nullptr;
  cudaError_t e = cudaSuccess;
  if (location == GVR_MEM_HOST) {
    // inputs and output staged in one scratch block: n + 1 canvases
    e = scratch_alloc(&scratch, per * (size_t)(n_images + 1), st);
    if (e != cudaSuccess) return cuda_error(e, "allocate image scratch");
    char *b = static_cast<char *>(scratch);
    for (int k = 0; k < n_images && e == cudaSuccess; ++k) {
      float4 *c = reinterpret_cast<float4 *>(b + per * k);
      float *z = reinterpret_cast<float *>(c + pixels);
      e = cudaMemcpyAsync(c, rgba[k], sizeof(float4) * pixels, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(z, depth[k], sizeof(float) * pixels, cudaMemcpyHostToDevice, st);
      im.rgba[k] = c;
      im.depth[k] = z;
    }
    d_out = reinterpret_cast<float4 *>(b + per * n_images);
    d_dep = reinterpret_cast<float *>(d_out + pixels);
  } else {
    for (int k = 0; k < n_images; ++k) {
      im.rgba[k] = reinterpret_cast<const float4 *>(rgba[k]);
      im.depth[k] = depth[k];
    }
  }
  if (e == cudaSuccess) {
    const int grid = (int)std::min<int64_t>((pixels + 255) / 256, 152 * 8);
    zbuffer_kernel<<<grid, 256, 0, st>>>(im, n_images, pixels, d_out, d_dep);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && location == GVR_MEM_HOST) {
    e = cudaMemcpyAsync(out_rgba, d_out, sizeof(float4) * pixels, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(out_depth, d_dep, sizeof(float) * pixels, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  }
  if (scratch) cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cuda_error(e, "z-buffer composite");
  return GVR_OK;
}

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

extern "C" int gvr_canvas_color_bar(float *rgba, int width, int height, const float *lut_rgba,
                                    int lut_size, const float box[4], const float fg[4],
                                    int location, void *stream)
{
  if (!rgba || !lut_rgba || !box || !fg) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (width < 1 || height < 1 || (int64_t)width * height > (1ll << 28))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image size must be >= 1 and <= 2^28 pixels");
  if (lut_size < 2 || lut_size > kMaxLut) return set_error(GVR_ERR_INVALID_ARGUMENT, "lut_size must be in [2, 4096]");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad location");
  for (int k = 0; k < 4; ++k)
    if (!std::isfinite(box[k])) return set_error(GVR_ERR_INVALID_ARGUMENT, "colour bar box must be finite");
  if (!(box[1] > box[0]) || !(box[3] > box[2]))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "colour bar box needs xmin < xmax and ymin < ymax");
  // screen coordinates [-1, 1] -> the pixel rectangle, clipped to the image
  // (in double, where these products of a float and an image size are exact)
  auto px = [](float v, int n) { return (int)std::floor(((double)v + 1.0) * 0.5 * (double)n + 0.5); };
  const int x0 = std::max(0, px(box[0], width)), x1 = std::min(width, px(box[1], width));
  const int y0 = std::max(0, px(box[2], height)), y1 = std::min(height, px(box[3], height));
  if (x1 - x0 < 1 || y1 - y0 < 1) return GVR_OK;   // nothing of the bar is in the image
  const int bw = x1 - x0, bh = y1 - y0;
  // orientation from the requested box, as the reference's bars: taller than wide -> vertical
  const int vertical = ((double)box[3] - box[2]) * height >= ((double)box[1] - box[0]) * width;
  const int64_t pixels = (int64_t)width * height;
  cudaStream_t st = (cudaStream_t)stream;
  float4 *d_img = reinterpret_cast<float4 *>(rgba);
  float4 *d_lut = nullptr;
  void *scratch = nullptr;
  const size_t lut_bytes = sizeof(float4) * lut_size;
  cudaError_t e = scratch_alloc(&scratch, lut_bytes + (location == GVR_MEM_HOST ? sizeof(float4) * pixels : 0), st);
  if (e != cudaSuccess) return cuda_error(e, "allocate colour bar scratch");
  d_lut = static_cast<float4 *>(scratch);
  e = cudaMemcpyAsync(d_lut, lut_rgba, lut_bytes, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && location == GVR_MEM_HOST) {
    d_img = d_lut + lut_size;
    e = cudaMemcpyAsync(d_img, rgba, sizeof(float4) * pixels, cudaMemcpyHostToDevice, st);
  }
  if (e == cudaSuccess) {
    const int grid = (int)std::min<int64_t>(((int64_t)bw * bh + 255) / 256, 152 * 8);
    color_bar_kernel<<<grid, 256, 0, st>>>(d_img, width, x0, y0, bw, bh, d_lut, lut_size, vertical,
                                           make_float4(fg[0], fg[1], fg[2], fg[3]));
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess && location == GVR_MEM_HOST)
    e = cudaMemcpyAsync(rgba, d_img, sizeof(float4) * pixels, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);   // the LUT was copied from host memory
  cudaFreeAsync(scratch, st);
  if (e != cudaSuccess) return cuda_error(e, "colour bar");
  return GVR_OK;
}
