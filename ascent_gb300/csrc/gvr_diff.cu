// gvr_diff.cu — differentiable volume render: forward with transmittance
// checkpoints and its hand-written adjoint.
//
// The render is the single-uniform-domain march of gvr_march.cu (same ray
// model, stepping rule and front-to-back blend) with the two changes a
// gradient needs: the transfer function is looked up with linear
// interpolation (so colour and opacity are differentiable in the scalar),
// and no partial is culled. Inputs are the caller's device buffers: the node
// field in its plain layout (x fastest) and the LUT (n RGBA floats), both
// differentiable.
//
// Forward (training): one thread per ray; it stores the transmittance at the
// start of every kDiffK-sample segment and caches every sample's scalar v_k
// in a workspace ([sample][ray], so that a warp writes contiguous rays).
// Backward: per ray, segments from last to first. A segment's transmittances
// T_k are rebuilt forward from its checkpoint through the cached scalars and
// the LUT — no field loads, and the blend is never inverted — into a
// thread-local array; then its samples are walked back to front with the
// suffix composite (R', A') of the samples behind them:
//   dL/dc_k = T_k a_k g_rgb,
//   dL/da_k = T_k (g_rgb . (c_k - R'_k) + g_A (1 - A'_k)),
//   R'_{k-1} = a_k c_k + (1 - a_k) R'_k,  A'_{k-1} = a_k + (1 - a_k) A'_k.
// LUT gradients are summed in registers while consecutive samples of a ray
// stay in one LUT interval, then added with two float4 atomics to the CTA's
// private copy in global memory; a last kernel sums the copies. Field
// gradients are
// summed per ray while consecutive samples stay in one cell, then combined
// with the neighbouring lane's sums when both leave the same cell at the
// same step, and added with two float4 atomics per cell into a corner-quad
// buffer that is folded into the node gradient at the end.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>

#include "gvr_internal.h"

namespace gvr {
namespace {

constexpr int kDiffK = 64;          // samples per transmittance checkpoint
constexpr int kSub = 8;             // backward: scalars loaded together
constexpr int kMaxDiffViews = 64;
constexpr int kDiffLut = 4096;

struct DiffViews {
  ViewDev v[kMaxDiffViews];
};

struct DiffGrid {
  int dims[3];
  float origin[3];
  float inv_spacing[3];
  float lo[3];
  float hi[3];
};

struct DiffParams {
  int width;
  int height;
  int n_views;
  int lut_size;
  int n_seg;       // checkpoint segments per ray
  int lut_copies;  // backward: LUT-gradient copies in global memory (CTA c uses c % copies)
  int64_t n_rays;  // views x height x width
  int64_t v_offset;  // start of the per-sample scalar cache in the workspace
  float sample_dist;
  float scalar_min;
  float inv_range;
};

__device__ __forceinline__ float lerp2(float a, float b, float w) { return fmaf(w, b - a, a); }

// Ray of pixel (px, py) of view v: origin, unit direction, [t0, t1) inside the
// grid; false when the ray misses it.
__device__ __forceinline__ bool diff_ray(const ViewDev &view, const DiffGrid &g, const DiffParams &p,
                                         int px, int py, float o[3], float d[3], float &t0,
                                         float &t1)
{
  const float fx = view.dx_scale * ((float)px - 0.5f * (float)p.width - view.xoff);
  const float fy = view.dy_scale * ((float)py - 0.5f * (float)p.height - view.yoff);
  float dn = 0.f;
  for (int a = 0; a < 3; ++a) {
    d[a] = view.look[a] + view.ru[a] * fx + view.rv[a] * fy;
    dn = fmaf(d[a], d[a], dn);
  }
  const float inv = rsqrtf(dn);
  t0 = 0.f;
  t1 = FLT_MAX;
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
      return false;
    }
  }
  return t1 > t0;
}

// Cell (linear index of its corner 000) and trilinear weights of sample t.
__device__ __forceinline__ int64_t diff_cell(const DiffGrid &g, const float A[3], const float B[3],
                                             float t, float w[3])
{
  int c[3];
  for (int a = 0; a < 3; ++a) {
    const float gg = fmaf(t, B[a], A[a]);
    c[a] = max(0, min((int)gg, g.dims[a] - 2));
    w[a] = gg - (float)c[a];
  }
  return ((int64_t)c[2] * g.dims[1] + c[1]) * g.dims[0] + c[0];
}

// The 8 corners of the cell at base: (x, y, z) bits of the index are
// (1, 2, 4).
__device__ __forceinline__ void diff_corners(const float *__restrict__ f, const DiffGrid &g,
                                             int64_t base, float c[8])
{
  const int64_t sy = g.dims[0], sz = (int64_t)g.dims[0] * g.dims[1];
  const float *p = f + base;
  c[0] = __ldg(p);
  c[1] = __ldg(p + 1);
  c[2] = __ldg(p + sy);
  c[3] = __ldg(p + sy + 1);
  c[4] = __ldg(p + sz);
  c[5] = __ldg(p + sz + 1);
  c[6] = __ldg(p + sz + sy);
  c[7] = __ldg(p + sz + sy + 1);
}

__device__ __forceinline__ float diff_interp(const float c[8], const float w[3])
{
  const float c00 = lerp2(c[0], c[1], w[0]);
  const float c10 = lerp2(c[2], c[3], w[0]);
  const float c01 = lerp2(c[4], c[5], w[0]);
  const float c11 = lerp2(c[6], c[7], w[0]);
  return lerp2(lerp2(c00, c10, w[1]), lerp2(c01, c11, w[1]), w[2]);
}

// Opacity of the linear LUT lookup at scalar v (the w of diff_lut), from the
// LUT's opacity column.
__device__ __forceinline__ float lut_alpha(const float *lut_a, const DiffParams &p, float v)
{
  const float x = __saturatef((v - p.scalar_min) * p.inv_range) * (float)(p.lut_size - 1);
  const int i0 = min((int)x, p.lut_size - 2);
  return lerp2(lut_a[i0], lut_a[i0 + 1], x - (float)i0);
}

// Linear LUT lookup at scalar v; also returns the entry index i0 and weight.
__device__ __forceinline__ float4 diff_lut(const float4 *lut, const DiffParams &p, float v,
                                           float &s_raw, int &i0, float &wl)
{
  s_raw = (v - p.scalar_min) * p.inv_range;
  const float s = __saturatef(s_raw);
  const float x = s * (float)(p.lut_size - 1);
  i0 = min((int)x, p.lut_size - 2);
  wl = x - (float)i0;
  const float4 a = lut[i0], b = lut[i0 + 1];
  return make_float4(lerp2(a.x, b.x, wl), lerp2(a.y, b.y, wl), lerp2(a.z, b.z, wl),
                     lerp2(a.w, b.w, wl));
}

__global__ void __launch_bounds__(256)
diff_forward(const float *__restrict__ field, const DiffGrid g, const DiffViews views,
             const DiffParams p, const float4 *__restrict__ g_lut, float4 *__restrict__ rgba,
             float *__restrict__ ws)
{
  extern __shared__ float4 lut[];
  for (int i = threadIdx.x; i < p.lut_size; i += blockDim.x) lut[i] = g_lut[i];
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int py = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
  const int v = blockIdx.z;
  if (px >= p.width || py >= p.height) return;
  const int64_t ray = ((int64_t)v * p.height + py) * p.width + px;
  float o[3], d[3], t0, t1;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  if (diff_ray(views.v[v], g, p, px, py, o, d, t0, t1)) {
    float A[3], B[3];
    for (int a = 0; a < 3; ++a) {
      A[a] = (o[a] - g.origin[a]) * g.inv_spacing[a];
      B[a] = d[a] * g.inv_spacing[a];
    }
    // corners of the last cell loaded, reused while samples stay in it
    int64_t last = -1;
    float cc[8];
    for (int k = 0;; ++k) {
      const float t = fmaf((float)k, p.sample_dist, t0);
      if (!(t < t1)) break;
      if (ws) {
        // transmittance checkpoint at each segment start, scalar of every sample
        if ((k % kDiffK) == 0) ws[ray * p.n_seg + k / kDiffK] = 1.f - acc.w;
      }
      float w[3];
      const int64_t base = diff_cell(g, A, B, t, w);
      if (base != last) {
        diff_corners(field, g, base, cc);
        last = base;
      }
      const float val = diff_interp(cc, w);
      if (ws) ws[p.v_offset + (int64_t)k * p.n_rays + ray] = val;
      float s_raw, wl;
      int i0;
      const float4 c = diff_lut(lut, p, val, s_raw, i0, wl);
      const float wa = (1.f - acc.w) * c.w;
      acc.x = fmaf(wa, c.x, acc.x);
      acc.y = fmaf(wa, c.y, acc.y);
      acc.z = fmaf(wa, c.z, acc.z);
      acc.w += wa;
    }
  }
  rgba[ray] = acc;
}

// Add g8 (the gradients of one cell's eight corners) to the field gradient.
// Warp-aggregated in pairs: lanes 2i and 2i + 1 (neighbouring pixels in x)
// that flush the same cell at the same step add their sums first, so one
// atomic covers both. Measured against pooling whole peer sets
// (__match_any_sync, then shuffles) and against 2x2 / 4x2 pixel groups,
// pairs were fastest: wider groups cost more shuffles than they save
// atomics. The sums go to the corner-quad buffer gq (one float4 per cell
// base: corners (x, y), (x+1, y), (x, y+1), (x+1, y+1) of one z layer), so a
// flush is two 16-byte vector atomics, each in one sector; fold_quads adds
// the quads into the node gradient afterwards. Called by all lanes.
__device__ __forceinline__ void flush_cell(float4 *__restrict__ gq, const DiffGrid &g,
                                           int64_t base, const float g8[8], bool active)
{
  const int lane = threadIdx.x & 31;
  const int64_t ob = __shfl_xor_sync(0xffffffffu, active ? base : -1 - (int64_t)lane, 1);
  const bool pair = active && ob == base;
  float s[8];
#pragma unroll
  for (int m = 0; m < 8; ++m) {
    const float x = __shfl_xor_sync(0xffffffffu, g8[m], 1);
    s[m] = g8[m] + (pair ? x : 0.f);
  }
  if (!active || (pair && (lane & 1))) return;
  const int64_t sz = (int64_t)g.dims[0] * g.dims[1];
  atomicAdd(gq + base, make_float4(s[0], s[1], s[2], s[3]));
  atomicAdd(gq + base + sz, make_float4(s[4], s[5], s[6], s[7]));
}

// grad[i] += quads whose corners include node i: its own quad's (x, y)
// entry, the (x+1, y) entry of the quad to its left, and so on.
__global__ void fold_quads(const float4 *__restrict__ gq, const DiffGrid g,
                           float *__restrict__ grad)
{
  const int64_t nx = g.dims[0], ny = g.dims[1], n = nx * ny * g.dims[2];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t x = i % nx, y = (i / nx) % ny;
    float acc = gq[i].x;
    if (x > 0) acc += gq[i - 1].y;
    if (y > 0) acc += gq[i - nx].z;
    if (x > 0 && y > 0) acc += gq[i - nx - 1].w;
    if (acc != 0.f) grad[i] += acc;
  }
}

// Add the register sums of LUT interval li (entries li and li + 1) to this
// CTA's LUT-gradient copy as two float4 atomics, and clear them.
__device__ __forceinline__ void flush_lut4(float *copy, int li, float (&lg)[8])
{
  if (li < 0) return;
  float4 *q = reinterpret_cast<float4 *>(copy + 4 * li);
  atomicAdd(q, make_float4(lg[0], lg[1], lg[2], lg[3]));
  atomicAdd(q + 1, make_float4(lg[4], lg[5], lg[6], lg[7]));
#pragma unroll
  for (int m = 0; m < 8; ++m) lg[m] = 0.f;
}

__global__ void __launch_bounds__(256)
diff_backward(const float *__restrict__ field, const DiffGrid g, const DiffViews views,
              const DiffParams p, const float4 *__restrict__ g_lut,
              const float4 *__restrict__ grad_rgba, const float *__restrict__ ws,
              float4 *__restrict__ gq, float *__restrict__ glut_cta)
{
  extern __shared__ float4 smem[];
  float4 *lut = smem;
  // LUT gradient: this CTA's private copy in global memory (L2-resident),
  // two float4 atomics per flushed interval. Measured against 16 padded
  // private copies in shared memory per CTA (8 scalar shared atomics per
  // flush, bank conflicts, 64 KB of shared memory taken from L1): 4.72 vs
  // 5.86 ms for the whole training step.
  float *lut_a = reinterpret_cast<float *>(smem + p.lut_size);  // opacity column
  const int64_t cta = ((int64_t)blockIdx.z * gridDim.y + blockIdx.y) * gridDim.x + blockIdx.x;
  float *slg = glut_cta + (cta % p.lut_copies) * 4 * p.lut_size;
  for (int i = threadIdx.x; i < p.lut_size; i += blockDim.x) {
    lut[i] = g_lut[i];
    lut_a[i] = g_lut[i].w;
  }
  __syncthreads();
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = blockIdx.x * 16 + (warp & 1) * 8 + (lane & 7);
  const int py = blockIdx.y * 16 + (warp >> 1) * 4 + (lane >> 3);
  const int v = blockIdx.z;
  const bool inside = px < p.width && py < p.height;
  float o[3], d[3], t0 = 0.f, t1 = 0.f;
  const bool hit = inside && diff_ray(views.v[v], g, p, min(px, p.width - 1), min(py, p.height - 1),
                                      o, d, t0, t1);
  int n = 0;
  float4 gr = make_float4(0.f, 0.f, 0.f, 0.f);
  float A[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f};
  int64_t ray = 0;
  if (hit) {
    ray = ((int64_t)v * p.height + py) * p.width + px;
    gr = grad_rgba[ray];
    for (int a = 0; a < 3; ++a) {
      A[a] = (o[a] - g.origin[a]) * g.inv_spacing[a];
      B[a] = d[a] * g.inv_spacing[a];
    }
    while (fmaf((float)n, p.sample_dist, t0) < t1) ++n;
  }
  // the warp walks segments in lock step so that lanes can pool their
  // field gradients; lanes with fewer segments idle
  int nseg = hit ? (n + kDiffK - 1) / kDiffK : 0;
  int max_seg = nseg;
  for (int off = 16; off > 0; off >>= 1) max_seg = max(max_seg, __shfl_xor_sync(0xffffffffu, max_seg, off));
  float Rr = 0.f, Rg = 0.f, Rb = 0.f, Ra = 0.f;  // suffix composite behind the sample
  int64_t cur = -1;
  float g8[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int li = -1;  // LUT interval of the register sums lg
  float lg[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  const int64_t vcache = p.v_offset + ray;
  float T[kDiffK];
  for (int sidx = max_seg - 1; sidx >= 0; --sidx) {
    const int k0 = sidx * kDiffK, k1 = sidx < nseg ? min(k0 + kDiffK, n) : k0;
    // transmittance of every sample of the segment, forward from its
    // checkpoint through the cached scalars (no field loads); the scalars
    // are loaded kSub at a time so that their latencies overlap
    if (k1 > k0) {
      float Tr = ws[ray * p.n_seg + sidx];
      for (int kq = k0; kq < k1; kq += kSub) {
        float vv[kSub];
#pragma unroll
        for (int j = 0; j < kSub; ++j) vv[j] = kq + j < k1 ? ws[vcache + (int64_t)(kq + j) * p.n_rays] : 0.f;
#pragma unroll
        for (int j = 0; j < kSub; ++j) {
          T[kq - k0 + j] = Tr;
          if (kq + j < k1) Tr *= 1.f - lut_alpha(lut_a, p, vv[j]);
        }
      }
    }
    // walk it back to front, from the warp's last sample in the segment
    // (uniform trip count across the warp); the scalar and transmittance of
    // the next sample are loaded one step ahead
    {
      const int jn = (int)__reduce_max_sync(0xffffffffu, (unsigned)(k1 - k0));
      float v_next = k1 > k0 + jn - 1 ? ws[vcache + (int64_t)(k0 + jn - 1) * p.n_rays] : 0.f;
      float t_next = T[max(jn - 1, 0)];
      for (int j = jn - 1; j >= 0; --j) {
        const int k = k0 + j;
        const bool on = k < k1;
        const float v_cur = v_next, Tk = t_next;
        if (j > 0) {
          v_next = k - 1 < k1 ? ws[vcache + (int64_t)(k - 1) * p.n_rays] : 0.f;
          t_next = T[j - 1];
        }
        int64_t base = -1;
        float w[3] = {0.f, 0.f, 0.f}, dv = 0.f;
        if (on) {
          const float t = fmaf((float)k, p.sample_dist, t0);
          base = diff_cell(g, A, B, t, w);
          float s_raw, wl;
          int i0;
          const float4 c = diff_lut(lut, p, v_cur, s_raw, i0, wl);
          const float ta = Tk * c.w;
          const float dcr = ta * gr.x, dcg = ta * gr.y, dcb = ta * gr.z;
          const float da = Tk * (gr.x * (c.x - Rr) + gr.y * (c.y - Rg) + gr.z * (c.z - Rb) +
                                 gr.w * (1.f - Ra));
          Rr = fmaf(c.w, c.x, (1.f - c.w) * Rr);
          Rg = fmaf(c.w, c.y, (1.f - c.w) * Rg);
          Rb = fmaf(c.w, c.z, (1.f - c.w) * Rb);
          Ra = c.w + (1.f - c.w) * Ra;
          // transfer-function entries i0 and i0 + 1: summed in registers
          // while consecutive samples stay in one LUT interval
          if (i0 != li) {
            flush_lut4(slg, li, lg);
            li = i0;
          }
          const float w0 = 1.f - wl;
          lg[0] = fmaf(w0, dcr, lg[0]);
          lg[1] = fmaf(w0, dcg, lg[1]);
          lg[2] = fmaf(w0, dcb, lg[2]);
          lg[3] = fmaf(w0, da, lg[3]);
          lg[4] = fmaf(wl, dcr, lg[4]);
          lg[5] = fmaf(wl, dcg, lg[5]);
          lg[6] = fmaf(wl, dcb, lg[6]);
          lg[7] = fmaf(wl, da, lg[7]);
          // scalar: d(rgba)/dx = lut[i0 + 1] - lut[i0], x = s (n - 1)
          if (s_raw > 0.f && s_raw < 1.f) {
            const float4 a0 = lut[i0], a1 = lut[i0 + 1];
            const float dx = dcr * (a1.x - a0.x) + dcg * (a1.y - a0.y) + dcb * (a1.z - a0.z) +
                             da * (a1.w - a0.w);
            dv = dx * (float)(p.lut_size - 1) * p.inv_range;
          }
        }
        // pool the field gradient per cell; flush when a lane changes cell
        const bool change = on && base != cur && cur >= 0;
        flush_cell(gq, g, cur, g8, change);
        if (change) {
#pragma unroll
          for (int m = 0; m < 8; ++m) g8[m] = 0.f;
        }
        if (on) {
          cur = base;
          const float x0 = 1.f - w[0], y0 = 1.f - w[1], z0 = 1.f - w[2];
          g8[0] = fmaf(dv, x0 * y0 * z0, g8[0]);
          g8[1] = fmaf(dv, w[0] * y0 * z0, g8[1]);
          g8[2] = fmaf(dv, x0 * w[1] * z0, g8[2]);
          g8[3] = fmaf(dv, w[0] * w[1] * z0, g8[3]);
          g8[4] = fmaf(dv, x0 * y0 * w[2], g8[4]);
          g8[5] = fmaf(dv, w[0] * y0 * w[2], g8[5]);
          g8[6] = fmaf(dv, x0 * w[1] * w[2], g8[6]);
          g8[7] = fmaf(dv, w[0] * w[1] * w[2], g8[7]);
        }
      }
    }
  }
  flush_cell(gq, g, cur, g8, cur >= 0);
  flush_lut4(slg, li, lg);
}

// glut[i] += the CTAs' private LUT-gradient copies, 32 CTAs per thread
__global__ void sum_lut_copies(const float *__restrict__ glut_cta, int64_t n_cta, int n,
                               float *__restrict__ glut)
{
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int64_t c0 = (int64_t)blockIdx.y * 32, c1 = min(c0 + 32, n_cta);
  float acc = 0.f;
  for (int64_t c = c0; c < c1; ++c) acc += glut_cta[c * n + i];
  if (acc != 0.f) atomicAdd(glut + i, acc);
}

int diff_setup(const float *field, const int dims[3], const double origin[3],
               const double spacing[3], const gvr_camera *cameras, int n_views,
               const gvr_render_params *params, DiffGrid &g, DiffViews &views, DiffParams &p)
{
  if (!field || !dims || !origin || !spacing || !cameras || !params)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n_views < 1 || n_views > kMaxDiffViews)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "the differentiable render takes 1..64 views");
  if (params->width < 1 || params->height < 1 || params->lut_size < 2 || params->lut_size > kDiffLut)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad image size or lut_size (2..4096)");
  if (!(params->sample_dist > 0)) return set_error(GVR_ERR_INVALID_ARGUMENT, "sample_dist must be > 0");
  double diag = 0;
  for (int a = 0; a < 3; ++a) {
    if (dims[a] < 2 || !(spacing[a] > 0))
      return set_error(GVR_ERR_INVALID_ARGUMENT, "dims >= 2 and spacing > 0 required");
    const float o = (float)origin[a], sp = (float)spacing[a];
    g.dims[a] = dims[a];
    g.origin[a] = o;
    g.inv_spacing[a] = 1.f / sp;
    g.lo[a] = o;
    g.hi[a] = (float)((double)o + (double)(dims[a] - 1) * sp);
    diag += (double)(dims[a] - 1) * sp * (double)(dims[a] - 1) * sp;
  }
  for (int v = 0; v < n_views; ++v) make_view(cameras[v], params->width, params->height, &views.v[v]);
  p.width = params->width;
  p.height = params->height;
  p.n_views = n_views;
  p.lut_size = params->lut_size;
  p.sample_dist = params->sample_dist;
  p.scalar_min = params->scalar_min;
  p.inv_range = params->scalar_max > params->scalar_min
                    ? 1.f / (params->scalar_max - params->scalar_min) : 0.f;
  const double max_samples = std::sqrt(diag) / params->sample_dist + 2.0;
  p.n_seg = (int)((max_samples + kDiffK - 1) / kDiffK);
  p.lut_copies = 1;
  p.n_rays = (int64_t)n_views * params->width * params->height;
  p.v_offset = p.n_rays * p.n_seg;
  return GVR_OK;
}

}  // namespace
}  // namespace gvr

using namespace gvr;

extern "C" {

int gvr_diff_workspace(const int dims[3], const double spacing[3], float sample_dist,
                       int *floats_per_ray)
{
  if (!dims || !spacing || !floats_per_ray || !(sample_dist > 0))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad arguments");
  double diag = 0;
  for (int a = 0; a < 3; ++a) diag += (double)(dims[a] - 1) * spacing[a] * (double)(dims[a] - 1) * spacing[a];
  const double max_samples = std::sqrt(diag) / sample_dist + 2.0;
  const int n_seg = (int)((max_samples + kDiffK - 1) / kDiffK);
  *floats_per_ray = n_seg * (1 + kDiffK);
  return GVR_OK;
}

int gvr_diff_render_forward(const float *field, const int dims[3], const double origin[3],
                            const double spacing[3], const gvr_camera *cameras, int n_views,
                            const gvr_render_params *params, const float *lut, float *rgba,
                            float *workspace, void *stream)
{
  DiffGrid g;
  DiffViews views;
  DiffParams p;
  int rc = diff_setup(field, dims, origin, spacing, cameras, n_views, params, g, views, p);
  if (rc != GVR_OK) return rc;
  if (!lut || !rgba) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL lut or rgba");
  const size_t smem = sizeof(float4) * p.lut_size;
  cudaError_t e = cudaFuncSetAttribute(diff_forward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(float4) * kDiffLut));
  if (e != cudaSuccess) return cuda_error(e, "shared-memory attribute");
  dim3 grid((p.width + 15) / 16, (p.height + 15) / 16, n_views);
  diff_forward<<<grid, 256, smem, (cudaStream_t)stream>>>(field, g, views, p, (const float4 *)lut,
                                                          (float4 *)rgba, workspace);
  count_launch();
  e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_error(e, "differentiable forward launch");
  return GVR_OK;
}

int gvr_diff_render_backward(const float *field, const int dims[3], const double origin[3],
                             const double spacing[3], const gvr_camera *cameras, int n_views,
                             const gvr_render_params *params, const float *lut,
                             const float *grad_rgba, const float *workspace, float *grad_field,
                             float *grad_lut, void *stream)
{
  DiffGrid g;
  DiffViews views;
  DiffParams p;
  int rc = diff_setup(field, dims, origin, spacing, cameras, n_views, params, g, views, p);
  if (rc != GVR_OK) return rc;
  if (!lut || !grad_rgba || !workspace || !grad_field || !grad_lut)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL buffer");
  const size_t smem = (sizeof(float4) + sizeof(float)) * p.lut_size;
  cudaError_t e = cudaFuncSetAttribute(diff_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)smem);
  if (e != cudaSuccess) return cuda_error(e, "shared-memory attribute");
  // corner-quad buffer of the field gradient, from the library's pool
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t nodes = (int64_t)g.dims[0] * g.dims[1] * g.dims[2];
  float4 *gq = nullptr;
  dim3 grid((p.width + 15) / 16, (p.height + 15) / 16, n_views);
  const int64_t n_cta = (int64_t)grid.x * grid.y * grid.z;
  // one copy per CTA, at most 512 MB of copies (CTAs then share them)
  p.lut_copies = (int)std::max<int64_t>(
      1, std::min<int64_t>(n_cta, ((int64_t)512 << 20) / (16 * (int64_t)p.lut_size)));
  float *glc = nullptr;
  e = scratch_alloc((void **)&gq, sizeof(float4) * nodes, st);
  if (e != cudaSuccess) return cuda_error(e, "allocate gradient quads");
  e = scratch_alloc((void **)&glc, sizeof(float) * 4 * p.lut_size * p.lut_copies, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(glc, 0, sizeof(float) * 4 * p.lut_size * p.lut_copies, st);
  if (e == cudaSuccess) e = cudaMemsetAsync(gq, 0, sizeof(float4) * nodes, st);
  if (e == cudaSuccess) {
    diff_backward<<<grid, 256, smem, st>>>(field, g, views, p, (const float4 *)lut,
                                           (const float4 *)grad_rgba, workspace, gq, glc);
    count_launch();
    sum_lut_copies<<<dim3((4 * p.lut_size + 255) / 256, (unsigned)((p.lut_copies + 31) / 32)), 256, 0,
                     st>>>(glc, p.lut_copies, 4 * p.lut_size, grad_lut);
    count_launch();
    fold_quads<<<(unsigned)std::min<int64_t>((nodes + 255) / 256, 152 * 16), 256, 0, st>>>(gq, g,
                                                                                         grad_field);
    count_launch();
    e = cudaGetLastError();
  }
  cudaFreeAsync(gq, st);
  if (glc) cudaFreeAsync(glc, st);
  if (e != cudaSuccess) return cuda_error(e, "differentiable backward launch");
  return GVR_OK;
}

}  // extern "C"
