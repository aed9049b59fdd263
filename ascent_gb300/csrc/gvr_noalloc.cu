// gvr_noalloc.cu — a volume render that allocates no device memory.
//
// In-situ visualization runs inside a simulation's process, and many such
// simulations hand out all of the GPU's memory through their own pool
// allocator and do not let a library call cudaMalloc/cudaFree: a library
// allocation can fail against the pool's budget, and cudaMalloc/cudaFree
// synchronise the device, stalling the simulation's own streams. For those
// callers gvr_render_uniform_noalloc renders one uniform domain straight
// from the caller's device field into the caller's device image.
//
// The kernel is the single-domain march of gvr_march.cu reading the field in
// its plain node layout (x fastest) instead of the scene's bricks. Its only
// scratch — the device copy of the transfer function and the sample counter
// — lives in g_scratch below, a file-scope array of fixed size that every
// GPU loading the library holds until the process exits. Every call shares
// it and it keeps the last call's contents: the LUT is rewritten and the
// counter cleared on every call, and calls that overlap on the GPU (on
// different streams or threads) race on it.
#include <cfloat>
#include <mutex>

#include "gvr_internal.h"

namespace gvr {
namespace {

constexpr int kNoAllocMaxLut = 4096;                              // LUT entries
constexpr size_t kScratchLutBytes = sizeof(float4) * kNoAllocMaxLut;  // 64 KiB
constexpr size_t kScratchBytes = kScratchLutBytes + 256;          // + counters

// The scratch. In host code `g_scratch` is only a host-side stand-in for the
// symbol; its device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_mu;
unsigned char *g_addr[kMaxDevices] = {};

// Device address of g_scratch on the current device, looked up once per
// device (the first call on a device does this set-up).
int scratch_address(int device, unsigned char **out)
{
  if (device < 0 || device >= kMaxDevices)
    return set_error(GVR_ERR_UNSUPPORTED, "device index beyond 63");
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_scratch);
    if (e != cudaSuccess) return cuda_error(e, "cudaGetSymbolAddress(scratch)");
    g_addr[device] = static_cast<unsigned char *>(p);
  }
  *out = g_addr[device];
  return GVR_OK;
}

struct Grid {
  const float *field;
  int dims[3];
  float origin[3];
  float inv_spacing[3];
  float lo[3];
  float hi[3];
};

__device__ __forceinline__ float lerp1(float a, float b, float w) { return fmaf(w, b - a, a); }

__global__ void __launch_bounds__(256, 4)
noalloc_march(const Grid g, const ViewDev view, const MarchParams mp,
              const float4 *__restrict__ g_lut, unsigned long long *__restrict__ samples,
              float4 *__restrict__ rgba, float *__restrict__ depth)
{
  extern __shared__ float4 lut[];
  for (int i = threadIdx.x; i < mp.lut_size; i += blockDim.x) lut[i] = g_lut[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int py = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
  int count = 0;
  if (px < mp.width && py < mp.height) {
    const float fx = view.dx_scale * ((float)px - 0.5f * (float)mp.width - view.xoff);
    const float fy = view.dy_scale * ((float)py - 0.5f * (float)mp.height - view.yoff);
    float o[3], d[3], dn = 0.f;
    for (int a = 0; a < 3; ++a) {
      d[a] = view.look[a] + view.ru[a] * fx + view.rv[a] * fy;
      dn = fmaf(d[a], d[a], dn);
    }
    const float inv = rsqrtf(dn);
    float t0 = 0.f, t1 = FLT_MAX;
    bool hit = true;
    for (int a = 0; a < 3; ++a) {
      o[a] = view.origin[a];
      d[a] *= inv;
      if (d[a] != 0.f) {
        const float r = 1.f / d[a];
        float ta = (g.lo[a] - o[a]) * r, tb = (g.hi[a] - o[a]) * r;
        if (ta > tb) { const float t = ta; ta = tb; tb = t; }
        t0 = fmaxf(t0, ta);
        t1 = fminf(t1, tb);
      } else if (o[a] < g.lo[a] || o[a] > g.hi[a]) {
        hit = false;
      }
    }
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (hit && t1 > t0) {
      float A[3], B[3];
      for (int a = 0; a < 3; ++a) {
        A[a] = (o[a] - g.origin[a]) * g.inv_spacing[a];
        B[a] = d[a] * g.inv_spacing[a];
      }
      const int64_t sy = g.dims[0], sz = (int64_t)g.dims[0] * g.dims[1];
      const float thr = mp.early_term < 1.f ? mp.early_term : 2.f;
      const float nm1 = (float)(mp.lut_size - 1);
      // a sample in the cell of the sample before keeps that cell's corners
      // (the scene march does the same; the values, and so the image, are
      // unchanged)
      int64_t last = -1;
      float lc[8];
      for (int k = 0;; ++k) {
        const float t = fmaf((float)k, mp.sample_dist, t0);
        if (!(t < t1)) break;
        ++count;
        int c[3];
        float w[3];
        for (int a = 0; a < 3; ++a) {
          const float gg = fmaf(t, B[a], A[a]);
          c[a] = max(0, min((int)gg, g.dims[a] - 2));
          w[a] = gg - (float)c[a];
        }
        const int64_t off = c[2] * sz + (int64_t)c[1] * sy + c[0];
        if (off != last) {
          const float *p = g.field + off;
          lc[0] = __ldg(p);
          lc[1] = __ldg(p + 1);
          lc[2] = __ldg(p + sy);
          lc[3] = __ldg(p + sy + 1);
          lc[4] = __ldg(p + sz);
          lc[5] = __ldg(p + sz + 1);
          lc[6] = __ldg(p + sz + sy);
          lc[7] = __ldg(p + sz + sy + 1);
          last = off;
        }
        const float c00 = lerp1(lc[0], lc[1], w[0]);
        const float c10 = lerp1(lc[2], lc[3], w[0]);
        const float c01 = lerp1(lc[4], lc[5], w[0]);
        const float c11 = lerp1(lc[6], lc[7], w[0]);
        const float v = lerp1(lerp1(c00, c10, w[1]), lerp1(c01, c11, w[1]), w[2]);
        const float s = __saturatef((v - mp.scalar_min) * mp.inv_range);
        float4 col;
        if (mp.lut_filter == GVR_LUT_LINEAR) {
          const float x = s * nm1;
          const int i0 = min((int)x, mp.lut_size - 2);
          const float ww = x - (float)i0;
          const float4 a0 = lut[i0], a1 = lut[i0 + 1];
          col = make_float4(lerp1(a0.x, a1.x, ww), lerp1(a0.y, a1.y, ww), lerp1(a0.z, a1.z, ww),
                            lerp1(a0.w, a1.w, ww));
        } else {
          col = lut[min((int)(s * nm1), mp.lut_size - 1)];
        }
        const float wa = (1.f - acc.w) * col.w;
        acc.x = fmaf(wa, col.x, acc.x);
        acc.y = fmaf(wa, col.y, acc.y);
        acc.z = fmaf(wa, col.z, acc.z);
        acc.w += wa;
        if (acc.w >= thr) break;
      }
    }
    float4 out = make_float4(0.f, 0.f, 0.f, 0.f);
    float dep = mp.clear_depth;
    if (acc.w >= mp.alpha_cull) {
      out = acc;
      // image depth of the partial's exit distance, ray rebuilt as the
      // reference's partials_to_canvas does (delta_y along ru)
      const float ex = view.dx_scale * (float)(2 * px - mp.width) * 0.5f;
      const float ey = view.dy_scale * (float)(2 * py - mp.height) * 0.5f;
      float q[3], qn = 0.f;
      for (int a = 0; a < 3; ++a) {
        q[a] = view.look[a] + view.ru[a] * ex + view.ru[a] * ey;
        qn = fmaf(q[a], q[a], qn);
      }
      const float qi = rsqrtf(qn);
      float pos[3];
      for (int a = 0; a < 3; ++a) pos[a] = fmaf(t1, q[a] * qi, view.origin[a]);
      const float *M = view.projview;
      const float z = M[8] * pos[0] + M[9] * pos[1] + M[10] * pos[2] + M[11];
      const float wv = M[12] * pos[0] + M[13] * pos[1] + M[14] * pos[2] + M[15];
      dep = 0.5f * (z / wv) + 0.49f;
    }
    if (mp.quantize_uint8) {
      out.x = (float)(unsigned char)fminf(out.x * 255.f, 255.f) * (1.f / 255.f);
      out.y = (float)(unsigned char)fminf(out.y * 255.f, 255.f) * (1.f / 255.f);
      out.z = (float)(unsigned char)fminf(out.z * 255.f, 255.f) * (1.f / 255.f);
      out.w = (float)(unsigned char)fminf(out.w * 255.f, 255.f) * (1.f / 255.f);
      dep = fabsf(dep);
    }
    if (mp.render_bg) {
      const float om = 1.f - out.w;
      out.x = fmaf(mp.bg[0], om, out.x);
      out.y = fmaf(mp.bg[1], om, out.y);
      out.z = fmaf(mp.bg[2], om, out.z);
      out.w = fmaf(mp.bg[3], om, out.w);
    }
    const int64_t pix = (int64_t)py * mp.width + px;
    rgba[pix] = out;
    depth[pix] = dep;
  }
  if (samples) {
    unsigned long long cc = (unsigned long long)count;
    for (int o = 16; o > 0; o >>= 1) cc += __shfl_xor_sync(0xffffffffu, cc, o);
    if (lane == 0 && cc) atomicAdd(samples, cc);
  }
}

bool finite3(const float *p) { return isfinite(p[0]) && isfinite(p[1]) && isfinite(p[2]); }

}  // namespace
}  // namespace gvr

using namespace gvr;

extern "C" int gvr_render_uniform_noalloc(const float *field, const int dims[3],
                                          const double origin[3], const double spacing[3],
                                          const gvr_camera *camera, const gvr_render_params *p,
                                          float *rgba, float *depth, void *stream,
                                          uint64_t *samples_out)
{
  if (!field || !dims || !origin || !spacing || !camera || !p || !rgba || !depth)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (p->lut_size > kNoAllocMaxLut)
    return set_error(GVR_ERR_INVALID_ARGUMENT,
                     "lut_size " + std::to_string(p->lut_size) +
                         " exceeds the 4096 entries the no-allocation scratch holds");
  if (!p->lut_rgba || p->lut_size < 2)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "lut_size must be in [2, 4096]");
  if (p->lut_filter != GVR_LUT_NEAREST && p->lut_filter != GVR_LUT_LINEAR)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad lut_filter");
  if (p->width < 1 || p->height < 1 || (int64_t)p->width * p->height > (1ll << 28))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image size must be >= 1 and <= 2^28 pixels");
  if (!(p->sample_dist > 0) || !isfinite(p->sample_dist))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "sample_dist must be > 0");
  if (!isfinite(p->scalar_min) || !isfinite(p->scalar_max))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "scalar range must be finite");
  if (!finite3(camera->position) || !finite3(camera->look_at) || !finite3(camera->up) ||
      !(camera->fov_y > 0 && camera->fov_y < 180))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad camera");
  {
    const float d[3] = {camera->look_at[0] - camera->position[0],
                        camera->look_at[1] - camera->position[1],
                        camera->look_at[2] - camera->position[2]};
    const float r[3] = {d[1] * camera->up[2] - d[2] * camera->up[1],
                        d[2] * camera->up[0] - d[0] * camera->up[2],
                        d[0] * camera->up[1] - d[1] * camera->up[0]};
    if (d[0] == 0.f && d[1] == 0.f && d[2] == 0.f)
      return set_error(GVR_ERR_INVALID_ARGUMENT, "camera position equals look_at");
    if (r[0] == 0.f && r[1] == 0.f && r[2] == 0.f)
      return set_error(GVR_ERR_INVALID_ARGUMENT, "camera up is parallel to the view direction");
  }
  Grid g;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] < 2) return set_error(GVR_ERR_INVALID_ARGUMENT, "every dimension needs >= 2 nodes");
    const float o = (float)origin[a], sp = (float)spacing[a];
    if (!(sp > 0) || !isfinite(o))
      return set_error(GVR_ERR_INVALID_ARGUMENT, "uniform spacing must be > 0 and origin finite");
    g.dims[a] = dims[a];
    g.origin[a] = o;
    g.inv_spacing[a] = 1.0f / sp;
    g.lo[a] = o;
    g.hi[a] = (float)((double)o + (double)(dims[a] - 1) * (double)sp);
  }
  g.field = field;
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDevice");
  unsigned char *scratch = nullptr;
  int rc = scratch_address(dev, &scratch);
  if (rc != GVR_OK) return rc;
  float4 *d_lut = reinterpret_cast<float4 *>(scratch);
  unsigned long long *d_count = reinterpret_cast<unsigned long long *>(scratch + kScratchLutBytes);
  cudaStream_t st = (cudaStream_t)stream;

  MarchParams mp{};
  mp.width = p->width;
  mp.height = p->height;
  mp.n_domains = 1;
  mp.lut_size = p->lut_size;
  mp.lut_filter = p->lut_filter;
  mp.quantize_uint8 = p->quantize_uint8 ? 1 : 0;
  mp.render_bg = p->render_bg ? 1 : 0;
  mp.sample_dist = p->sample_dist;
  mp.scalar_min = p->scalar_min;
  mp.inv_range = p->scalar_max > p->scalar_min ? 1.0f / (p->scalar_max - p->scalar_min) : 0.f;
  mp.alpha_cull = p->alpha_cull;
  mp.early_term = p->early_term >= 1.f ? 2.f : p->early_term;
  mp.clear_depth = p->clear_depth;
  for (int c = 0; c < 4; ++c) mp.bg[c] = p->bg_color[c];
  ViewDev view;
  make_view(*camera, p->width, p->height, &view);

  e = cudaMemcpyAsync(d_lut, p->lut_rgba, sizeof(float4) * p->lut_size, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && samples_out) e = cudaMemsetAsync(d_count, 0, sizeof(*d_count), st);
  if (e != cudaSuccess) return cuda_error(e, "scratch set-up");
  const size_t smem = sizeof(float4) * p->lut_size;
  if (smem > 48 * 1024) {
    e = cudaFuncSetAttribute(noalloc_march, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             (int)kScratchLutBytes);
    if (e != cudaSuccess) return cuda_error(e, "shared-memory attribute");
  }
  dim3 grid((p->width + 15) / 16, (p->height + 15) / 16);
  noalloc_march<<<grid, 256, smem, st>>>(
      g, view, mp, d_lut, samples_out ? d_count : nullptr, (float4 *)rgba, depth);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "no-allocation march launch");
  if (samples_out) {
    unsigned long long n = 0;
    e = cudaMemcpyAsync(&n, d_count, sizeof(n), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "read sample counter");
    *samples_out = n;
  }
  return GVR_OK;
}
