// gvr_hex.cu — hexahedral domains: ingest, on-device LBVH build, point
// location.
//
// Replaces, for the volume plot's unstructured-hex input, the Blueprint
// unstructured adapter (ascent_vtkh_data_adapter.cpp:1618-1780) and the
// VTK-m ConnectivityProxy setup (VolumeRenderer.cpp:182-220). The acceleration
// structure follows Devil Ray's LinearBVHBuilder
// (src/libs/dray/linear_bvh_builder.cpp): cell boxes, 30-bit Morton codes of
// box centres normalised by the scene box (:60-97, morton_codes.hpp:18-45),
// a sort of the codes (:120-140; here a stable device radix sort, so equal
// codes keep cell order), Karras's radix-tree construction (:148-251) and a
// bottom-up box refit with per-node arrival counters (:253-317). Morton
// arithmetic uses explicitly rounded FP32 operations so that codes, order
// and topology are bit-identical to a CPU rebuild.
#include <algorithm>
#include <cfloat>
#include <chrono>
#include <cmath>
#include <cstring>

#include "gvr_hex_device.cuh"

namespace gvr {
namespace {

__device__ __forceinline__ float load_f(const void *src, int dtype, int64_t i)
{
  return dtype == GVR_DTYPE_FLOAT64 ? (float)((const double *)src)[i] : ((const float *)src)[i];
}

__global__ void pack_nodes_kernel(const void *x, const void *y, const void *z, int cdtype,
                                  const void *field, int fdtype, int64_t n,
                                  float4 *__restrict__ nodes, int *__restrict__ bad)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float4 v = make_float4(load_f(x, cdtype, i), load_f(y, cdtype, i), load_f(z, cdtype, i),
                                 field ? load_f(field, fdtype, i) : 0.f);
    if (!(isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w))) *bad = 1;
    nodes[i] = v;
  }
}

__global__ void pack_conn_kernel(const void *conn, int idtype, int64_t n_cells, int64_t n_nodes,
                                 int4 *__restrict__ out, int *__restrict__ bad)
{
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    int v[8];
    for (int k = 0; k < 8; ++k) {
      const int64_t id = idtype == 1 ? ((const int64_t *)conn)[8 * c + k]
                                     : (int64_t)((const int32_t *)conn)[8 * c + k];
      if (id < 0 || id >= n_nodes) {
        *bad = 2;
        v[k] = 0;
      } else {
        v[k] = (int)id;
      }
    }
    out[2 * c] = make_int4(v[0], v[1], v[2], v[3]);
    out[2 * c + 1] = make_int4(v[4], v[5], v[6], v[7]);
  }
}

// Cell boxes and per-CTA scene box (6 floats per CTA).
__global__ void __launch_bounds__(256)
cell_box_kernel(const float4 *__restrict__ nodes, const int4 *__restrict__ conn, int64_t n,
                float4 *__restrict__ lo, float4 *__restrict__ hi, float *__restrict__ part)
{
  float bl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int4 a = conn[2 * c], b = conn[2 * c + 1];
    const int ids[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    float l[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, h[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int k = 0; k < 8; ++k) {
      const float4 v = nodes[ids[k]];
      l[0] = fminf(l[0], v.x); h[0] = fmaxf(h[0], v.x);
      l[1] = fminf(l[1], v.y); h[1] = fmaxf(h[1], v.y);
      l[2] = fminf(l[2], v.z); h[2] = fmaxf(h[2], v.z);
    }
    lo[c] = make_float4(l[0], l[1], l[2], 0.f);
    hi[c] = make_float4(h[0], h[1], h[2], 0.f);
    for (int a2 = 0; a2 < 3; ++a2) {
      bl[a2] = fminf(bl[a2], l[a2]);
      bh[a2] = fmaxf(bh[a2], h[a2]);
    }
  }
  __shared__ float s[8][6];
  for (int a2 = 0; a2 < 3; ++a2)
    for (int o = 16; o > 0; o >>= 1) {
      bl[a2] = fminf(bl[a2], __shfl_xor_sync(0xffffffffu, bl[a2], o));
      bh[a2] = fmaxf(bh[a2], __shfl_xor_sync(0xffffffffu, bh[a2], o));
    }
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0)
    for (int a2 = 0; a2 < 3; ++a2) { s[w][a2] = bl[a2]; s[w][3 + a2] = bh[a2]; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i)
      for (int a2 = 0; a2 < 3; ++a2) {
        bl[a2] = fminf(bl[a2], s[i][a2]);
        bh[a2] = fmaxf(bh[a2], s[i][3 + a2]);
      }
    for (int a2 = 0; a2 < 3; ++a2) {
      part[6 * blockIdx.x + a2] = bl[a2];
      part[6 * blockIdx.x + 3 + a2] = bh[a2];
    }
  }
}

// 10 bits -> every third bit of 30 (the usual Morton bit spreading).
__device__ __forceinline__ uint32_t spread3(uint32_t x)
{
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

__device__ __forceinline__ uint32_t quant10(float u)
{
  return (uint32_t)fminf(fmaxf(__fmul_rn(u, 1024.0f), 0.0f), 1023.0f);
}

__global__ void morton_kernel(const float4 *__restrict__ lo, const float4 *__restrict__ hi,
                              int64_t n, float mx, float my, float mz, float ix, float iy,
                              float iz, uint32_t *__restrict__ codes, uint32_t *__restrict__ ids)
{
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n;
       c += (int64_t)gridDim.x * blockDim.x) {
    const float4 l = lo[c], h = hi[c];
    const float cx = __fmul_rn(0.5f, __fadd_rn(l.x, h.x));
    const float cy = __fmul_rn(0.5f, __fadd_rn(l.y, h.y));
    const float cz = __fmul_rn(0.5f, __fadd_rn(l.z, h.z));
    const uint32_t qx = quant10(__fmul_rn(__fsub_rn(cx, mx), ix));
    const uint32_t qy = quant10(__fmul_rn(__fsub_rn(cy, my), iy));
    const uint32_t qz = quant10(__fmul_rn(__fsub_rn(cz, mz), iz));
    codes[c] = (spread3(qz) << 2) | (spread3(qy) << 1) | spread3(qx);
    ids[c] = (uint32_t)c;
  }
}

// Common-prefix length of sorted keys a and b; equal keys compare their
// positions (+32), out-of-range b gives -1 (Karras 2012, section 4).
__device__ __forceinline__ int prefix(const uint32_t *codes, int n_leaves, int a, int b)
{
  if (b < 0 || b >= n_leaves) return -1;
  const uint32_t x = codes[a] ^ codes[b];
  if (x) return __clz(x);
  return 32 + __clz((uint32_t)a ^ (uint32_t)b);
}

// One thread per inner node i in [0, n_leaves - 2]: children and parents.
__global__ void karras_kernel(const uint32_t *__restrict__ codes, int n_leaves,
                              int *__restrict__ left, int *__restrict__ right,
                              int *__restrict__ parent)
{
  const int n_inner = n_leaves - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inner; i += gridDim.x * blockDim.x) {
    const int d = prefix(codes, n_leaves, i, i + 1) - prefix(codes, n_leaves, i, i - 1) < 0 ? -1 : 1;
    const int dmin = prefix(codes, n_leaves, i, i - d);
    int lmax = 2;
    while (prefix(codes, n_leaves, i, i + lmax * d) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
      if (prefix(codes, n_leaves, i, i + (l + t) * d) > dmin) l += t;
    const int j = i + l * d;
    const int dnode = prefix(codes, n_leaves, i, j);
    int s = 0;
    for (int k = 1;; ++k) {
      const int t = (l + (1 << k) - 1) >> k;  // ceil(l / 2^k)
      if (prefix(codes, n_leaves, i, i + (s + t) * d) > dnode) s += t;
      if (t <= 1) break;
    }
    const int split = i + s * d + min(d, 0);
    const int lo = min(i, j), hi = max(i, j);
    const int lc = lo == split ? n_inner + split : split;
    const int rc = hi == split + 1 ? n_inner + split + 1 : split + 1;
    left[i] = lc;
    right[i] = rc;
    parent[lc] = i;
    parent[rc] = i;
    if (i == 0) parent[0] = -1;
  }
}

// Bottom-up refit: the second thread to reach a node computes its box.
__global__ void refit_kernel(const float4 *__restrict__ leaf_lo, const float4 *__restrict__ leaf_hi,
                             const uint32_t *__restrict__ ids, int n_leaves,
                             const int *__restrict__ left, const int *__restrict__ right,
                             const int *__restrict__ parent, int *__restrict__ counters,
                             float4 *box)
{
  const int n_inner = n_leaves - 1;
  for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < n_leaves; k += gridDim.x * blockDim.x) {
    int node = parent[n_inner + k];
    while (node >= 0) {
      __threadfence();
      if (atomicAdd(&counters[node], 1) == 0) break;
      __threadfence();
      float4 l[2], h[2];
      const int ch[2] = {left[node], right[node]};
      for (int q = 0; q < 2; ++q) {
        if (ch[q] >= n_inner) {
          const uint32_t cell = ids[ch[q] - n_inner];
          l[q] = leaf_lo[cell];
          h[q] = leaf_hi[cell];
        } else {
          l[q] = __ldcg(box + 2 * ch[q]);
          h[q] = __ldcg(box + 2 * ch[q] + 1);
        }
      }
      box[2 * node] = make_float4(fminf(l[0].x, l[1].x), fminf(l[0].y, l[1].y),
                                  fminf(l[0].z, l[1].z), 0.f);
      box[2 * node + 1] = make_float4(fmaxf(h[0].x, h[1].x), fmaxf(h[0].y, h[1].y),
                                      fmaxf(h[0].z, h[1].z), 0.f);
      node = parent[node];
    }
  }
}

__global__ void emit_kernel(const float4 *__restrict__ leaf_lo, const float4 *__restrict__ leaf_hi,
                            const uint32_t *__restrict__ ids, int n_leaves,
                            const int *__restrict__ left, const int *__restrict__ right,
                            const float4 *__restrict__ box, float4 *__restrict__ bvh)
{
  const int n_inner = n_leaves - 1;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n_inner; i += gridDim.x * blockDim.x) {
    float4 l[2], h[2];
    int enc[2];
    const int ch[2] = {left[i], right[i]};
    for (int q = 0; q < 2; ++q) {
      if (ch[q] >= n_inner) {
        const int k = ch[q] - n_inner;
        const uint32_t cell = ids[k];
        l[q] = leaf_lo[cell];
        h[q] = leaf_hi[cell];
        enc[q] = -(k + 1);
      } else {
        l[q] = box[2 * ch[q]];
        h[q] = box[2 * ch[q] + 1];
        enc[q] = ch[q];
      }
    }
    bvh[4 * (int64_t)i + 0] = make_float4(l[0].x, l[0].y, l[0].z, h[0].x);
    bvh[4 * (int64_t)i + 1] = make_float4(h[0].y, h[0].z, l[1].x, l[1].y);
    bvh[4 * (int64_t)i + 2] = make_float4(l[1].z, h[1].x, h[1].y, h[1].z);
    bvh[4 * (int64_t)i + 3] = make_float4(__int_as_float(enc[0]), __int_as_float(enc[1]), 0.f, 0.f);
  }
}

__global__ void locate_kernel(const DomainDev dm, const float *__restrict__ pts, int n,
                              int *__restrict__ cells, float *__restrict__ rst_out)
{
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]};
    float rst[3];
    HexGeom v;
    const int c = hex_locate(dm, p, rst, v);
    cells[i] = c;
    rst_out[3 * i] = rst[0];
    rst_out[3 * i + 1] = rst[1];
    rst_out[3 * i + 2] = rst[2];
  }
}

__global__ void set_node_field_kernel(const void *field, int dtype, int64_t stride, int64_t n,
                                      float4 *__restrict__ nodes, int *__restrict__ bad)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = load_f(field, dtype, i * stride);
    if (!isfinite(v)) *bad = 1;
    nodes[i].w = v;
  }
}

__global__ void node_range_kernel(const float4 *__restrict__ nodes, int64_t n, float2 *part)
{
  float lo = FLT_MAX, hi = -FLT_MAX;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = nodes[i].w;
    lo = fminf(lo, v);
    hi = fmaxf(hi, v);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  __shared__ float2 s[8];
  if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = make_float2(lo, hi);
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      lo = fminf(lo, s[i].x);
      hi = fmaxf(hi, s[i].y);
    }
    part[blockIdx.x] = make_float2(lo, hi);
  }
}

// Monomial coefficients of every cell's trilinear map (position and vertex
// field) from its corner nodes: 32 floats per cell, c0.xyz .. c7.xyz then
// w0 .. w7 (see hex_load).
__global__ void coef_kernel(const float4 *__restrict__ nodes, const int4 *__restrict__ conn,
                            int64_t n_cells, float4 *__restrict__ coef)
{
  for (int64_t c = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; c < n_cells;
       c += (int64_t)gridDim.x * blockDim.x) {
    const int4 a = conn[2 * c], b = conn[2 * c + 1];
    const int ids[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
    float4 v[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) v[i] = nodes[ids[i]];
    auto comb = [&](float s0, float s1, float s2, float s3, float s4, float s5, float s6, float s7,
                    float (float4::*m)) {
      return s0 * v[0].*m + s1 * v[1].*m + s2 * v[2].*m + s3 * v[3].*m + s4 * v[4].*m +
             s5 * v[5].*m + s6 * v[6].*m + s7 * v[7].*m;
    };
    float4 *o = coef + 8 * c;
    // c0 = v0, c1 = v1 - v0, c2 = v3 - v0, c3 = v4 - v0, c4 = v2 - v1 - v3 + v0,
    // c5 = v5 - v1 - v4 + v0, c6 = v7 - v3 - v4 + v0,
    // c7 = v6 - v2 - v5 - v7 + v1 + v3 + v4 - v0
    const float w[8][8] = {{1, 0, 0, 0, 0, 0, 0, 0},   {-1, 1, 0, 0, 0, 0, 0, 0},
                           {-1, 0, 0, 1, 0, 0, 0, 0},  {-1, 0, 0, 0, 1, 0, 0, 0},
                           {1, -1, 1, -1, 0, 0, 0, 0}, {1, -1, 0, 0, -1, 1, 0, 0},
                           {1, 0, 0, -1, -1, 0, 0, 1}, {-1, 1, -1, 1, 1, -1, 1, -1}};
    float f[32];
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      f[3 * k] = comb(w[k][0], w[k][1], w[k][2], w[k][3], w[k][4], w[k][5], w[k][6], w[k][7], &float4::x);
      f[3 * k + 1] = comb(w[k][0], w[k][1], w[k][2], w[k][3], w[k][4], w[k][5], w[k][6], w[k][7], &float4::y);
      f[3 * k + 2] = comb(w[k][0], w[k][1], w[k][2], w[k][3], w[k][4], w[k][5], w[k][6], w[k][7], &float4::z);
      f[24 + k] = comb(w[k][0], w[k][1], w[k][2], w[k][3], w[k][4], w[k][5], w[k][6], w[k][7], &float4::w);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) o[k] = make_float4(f[4 * k], f[4 * k + 1], f[4 * k + 2], f[4 * k + 3]);
  }
}

// Faces of a VTK hexahedron as local node ids, numbered like
// hex_exit_face: r = 0, r = 1, s = 0, s = 1, t = 0, t = 1.
__constant__ int kHexFace[6][4] = {{0, 3, 7, 4}, {1, 2, 6, 5}, {0, 1, 5, 4},
                                   {3, 2, 6, 7}, {0, 1, 2, 3}, {4, 5, 6, 7}};

// The three smallest node ids of face f (= 6 * cell + local face), ascending.
// In a conforming mesh two faces share at most an edge, so the triple names
// the face.
__device__ __forceinline__ void face_triple(const int4 *__restrict__ conn, uint32_t f,
                                            uint32_t t[3])
{
  const int64_t cell = f / 6;
  const int k = f % 6;
  const int4 a = conn[2 * cell], b = conn[2 * cell + 1];
  const int ids[8] = {a.x, a.y, a.z, a.w, b.x, b.y, b.z, b.w};
  uint32_t n0 = (uint32_t)ids[kHexFace[k][0]], n1 = (uint32_t)ids[kHexFace[k][1]];
  uint32_t n2 = (uint32_t)ids[kHexFace[k][2]], n3 = (uint32_t)ids[kHexFace[k][3]];
  uint32_t x;
#define CSWAP(p, q) if (p > q) { x = p; p = q; q = x; }
  CSWAP(n0, n1); CSWAP(n2, n3); CSWAP(n0, n2); CSWAP(n1, n3); CSWAP(n1, n2);
#undef CSWAP
  t[0] = n0;
  t[1] = n1;
  t[2] = n2;
}

// First sort key: the largest id of the triple; value: the face.
__global__ void face_key_kernel(const int4 *__restrict__ conn, int64_t nf, uint32_t *__restrict__ key,
                                uint32_t *__restrict__ face)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t t[3];
    face_triple(conn, (uint32_t)i, t);
    key[i] = t[2];
    face[i] = (uint32_t)i;
  }
}

// Second sort key, in the first sort's order: the two smallest ids.
__global__ void face_key2_kernel(const int4 *__restrict__ conn, const uint32_t *__restrict__ face,
                                 int64_t nf, uint64_t *__restrict__ key)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t t[3];
    face_triple(conn, face[i], t);
    key[i] = ((uint64_t)t[0] << 32) | t[1];
  }
}

// Faces sorted by triple: equal neighbours in the order are the two sides of
// one face.
__global__ void face_pair_kernel(const int4 *__restrict__ conn, const uint32_t *__restrict__ face,
                                 int64_t nf, int *__restrict__ nbr)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < nf;
       i += (int64_t)gridDim.x * blockDim.x) {
    uint32_t t[3], u[3];
    face_triple(conn, face[i], t);
    int other = -1;
    if (i + 1 < nf) {
      face_triple(conn, face[i + 1], u);
      if (u[0] == t[0] && u[1] == t[1] && u[2] == t[2]) other = (int)(face[i + 1] / 6);
    }
    if (other < 0 && i > 0) {
      face_triple(conn, face[i - 1], u);
      if (u[0] == t[0] && u[1] == t[1] && u[2] == t[2]) other = (int)(face[i - 1] / 6);
    }
    nbr[face[i]] = other;
  }
}

int grid_for(int64_t n, int threads = 256)
{
  int64_t b = (n + threads - 1) / threads;
  return (int)std::max<int64_t>(1, std::min<int64_t>(b, 152 * 16));
}

template <typename T>
cudaError_t dev_alloc(T **p, size_t count)
{
  return cudaMalloc((void **)p, sizeof(T) * std::max<size_t>(count, 1));
}

// Stage `bytes` of a host array on the device (or return the device pointer).
cudaError_t stage(const void *src, size_t bytes, int on_device, void **owned, const void **out)
{
  *owned = nullptr;
  if (on_device) {
    *out = src;
    return cudaSuccess;
  }
  cudaError_t e = cudaMalloc(owned, bytes);
  if (e == cudaSuccess) e = cudaMemcpy(*owned, src, bytes, cudaMemcpyHostToDevice);
  *out = *owned;
  return e;
}

}  // namespace

void free_hex(Domain &d)
{
  cudaFree(d.d_nodes);
  cudaFree(d.d_conn);
  cudaFree(d.d_bvh);
  cudaFree(d.d_codes);
  cudaFree(d.d_ids);
  cudaFree(d.d_left);
  cudaFree(d.d_right);
  cudaFree(d.d_parent);
  cudaFree(d.d_inner_box);
  cudaFree(d.d_nbr);
  d.d_nbr = nullptr;
  cudaFree(d.d_coef);
  d.d_coef = nullptr;
  d.d_nodes = nullptr;
  d.d_conn = nullptr;
  d.d_bvh = nullptr;
  d.d_codes = d.d_ids = nullptr;
  d.d_left = d.d_right = d.d_parent = nullptr;
  d.d_inner_box = nullptr;
}

// Range of the vertex field held in nodes[].w.
static int node_range(Domain &d)
{
  const int gb = grid_for(d.n_nodes);
  float2 *part = nullptr;
  cudaError_t e = dev_alloc(&part, gb);
  std::vector<float2> h(gb);
  if (e == cudaSuccess) {
    node_range_kernel<<<gb, 256>>>(d.d_nodes, d.n_nodes, part);
    count_launch();
    e = cudaMemcpy(h.data(), part, sizeof(float2) * gb, cudaMemcpyDeviceToHost);
  }
  cudaFree(part);
  if (e != cudaSuccess) return cuda_error(e, "hex field range");
  double lo = INFINITY, hi = -INFINITY;
  for (const float2 &r : h) {
    lo = std::min(lo, (double)r.x);
    hi = std::max(hi, (double)r.y);
  }
  d.range[0] = lo;
  d.range[1] = hi;
  return GVR_OK;
}

int hex_update_field(Domain &d, const void *field, int dtype, int64_t stride, int location)
{
  if (d.dev.assoc == GVR_ASSOC_ELEMENT) {
    cudaError_t e = launch_cells_field(field, dtype, stride, location == GVR_MEM_DEVICE, d.n_cells,
                                       d.d_cells, d.range, d.stg, 0);
    if (e != cudaSuccess) return cuda_error(e, "hex cell field");
    if (!(std::isfinite(d.range[0]) && std::isfinite(d.range[1])))
      return set_error(GVR_ERR_INVALID_ARGUMENT, "field contains non-finite values");
    return GVR_OK;
  }
  const size_t esz = dtype == GVR_DTYPE_FLOAT64 ? 8 : 4;
  const size_t bytes = (size_t)((d.n_nodes - 1) * stride + 1) * esz;
  const void *src = field;
  cudaError_t e = cudaSuccess;
  if (location != GVR_MEM_DEVICE) {
    if (bytes > d.stg.bytes) {
      cudaFree(d.stg.buf);
      d.stg.buf = nullptr;
      d.stg.bytes = 0;
      e = cudaMalloc(&d.stg.buf, bytes);
      if (e != cudaSuccess) return cuda_error(e, "hex field staging");
      d.stg.bytes = bytes;
    }
    e = cudaMemcpy(d.stg.buf, field, bytes, cudaMemcpyHostToDevice);
    src = d.stg.buf;
  }
  int *flag = nullptr;
  if (e == cudaSuccess) e = dev_alloc(&flag, 1);
  if (e == cudaSuccess) e = cudaMemset(flag, 0, sizeof(int));
  int bad = 0;
  if (e == cudaSuccess) {
    set_node_field_kernel<<<grid_for(d.n_nodes), 256>>>(src, dtype, stride, d.n_nodes, d.d_nodes, flag);
    count_launch();
    e = cudaMemcpy(&bad, flag, sizeof(int), cudaMemcpyDeviceToHost);
  }
  cudaFree(flag);
  if (e != cudaSuccess) return cuda_error(e, "hex field update");
  if (bad) return set_error(GVR_ERR_INVALID_ARGUMENT, "field contains non-finite values");
  coef_kernel<<<grid_for(d.n_cells), 256>>>(d.d_nodes, d.d_conn, d.n_cells, d.d_coef);
  count_launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_error(e, "hex coefficients");
  return node_range(d);
}

// Build everything a hex domain needs on the device; fills d.dev and bounds.
// Face-neighbour table: 6 cell ids per cell (-1 on the boundary), from two
// stable radix sorts of the faces by their node-id triples.
static int build_neighbours(Domain &d)
{
  const auto t0 = std::chrono::steady_clock::now();
  const int64_t nf = 6 * d.n_cells;
  uint32_t *key = nullptr, *key_tmp = nullptr, *face = nullptr, *face_tmp = nullptr, *scr = nullptr;
  uint64_t *key2 = nullptr, *key2_tmp = nullptr;
  int rc = GVR_OK;
  cudaError_t e = cudaSuccess;
  int bits = 1;
  while (bits < 32 && ((int64_t)1 << bits) < d.n_nodes) ++bits;
#define NB_TRY(expr, what)                                   \
  do {                                                       \
    e = (expr);                                              \
    if (e != cudaSuccess) { rc = cuda_error(e, what); goto done; } \
  } while (0)
  NB_TRY(dev_alloc(&d.d_nbr, nf), "alloc neighbours");
  NB_TRY(dev_alloc(&key, nf), "alloc face keys");
  NB_TRY(dev_alloc(&key_tmp, nf), "alloc face keys");
  NB_TRY(dev_alloc(&face, nf), "alloc faces");
  NB_TRY(dev_alloc(&face_tmp, nf), "alloc faces");
  NB_TRY(dev_alloc(&scr, sort_scratch_words(nf)), "alloc sort");
  face_key_kernel<<<grid_for(nf), 256>>>(d.d_conn, nf, key, face);
  count_launch();
  NB_TRY(radix_sort_pairs<uint32_t>(key, face, key_tmp, face_tmp, nf, bits, scr, 0), "sort faces");
  cudaFree(key);
  cudaFree(key_tmp);
  key = key_tmp = nullptr;
  NB_TRY(dev_alloc(&key2, nf), "alloc face keys");
  NB_TRY(dev_alloc(&key2_tmp, nf), "alloc face keys");
  face_key2_kernel<<<grid_for(nf), 256>>>(d.d_conn, face, nf, key2);
  count_launch();
  NB_TRY(radix_sort_pairs<uint64_t>(key2, face, key2_tmp, face_tmp, nf, 32 + bits, scr, 0),
         "sort faces");
  face_pair_kernel<<<grid_for(nf), 256>>>(d.d_conn, face, nf, d.d_nbr);
  count_launch();
  NB_TRY(cudaGetLastError(), "neighbour launch");
  NB_TRY(cudaDeviceSynchronize(), "neighbours");
done:
#undef NB_TRY
  cudaFree(key);
  cudaFree(key_tmp);
  cudaFree(key2);
  cudaFree(key2_tmp);
  cudaFree(face);
  cudaFree(face_tmp);
  cudaFree(scr);
  d.nbr_build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  return rc;
}

static int build_hex(Domain &d, const void *x, const void *y, const void *z, int cdtype,
                     const void *conn, int idtype, const void *field, int fdtype, int assoc,
                     int location)
{
  const int64_t nn = d.n_nodes, nc = d.n_cells;
  const size_t cbytes = (cdtype == GVR_DTYPE_FLOAT64 ? 8 : 4);
  const size_t fbytes = (fdtype == GVR_DTYPE_FLOAT64 ? 8 : 4);
  const size_t ibytes = idtype == 1 ? 8 : 4;
  const int on_dev = location == GVR_MEM_DEVICE;
  void *own[5] = {nullptr, nullptr, nullptr, nullptr, nullptr};
  const void *dx, *dy, *dz, *dconn, *dfield = nullptr;
  int *d_flag = nullptr;
  float4 *leaf_lo = nullptr, *leaf_hi = nullptr;
  float *part = nullptr;
  uint32_t *keys_tmp = nullptr, *vals_tmp = nullptr, *sort_scr = nullptr;
  int *counters = nullptr;
  int rc = GVR_OK;
  cudaError_t e = cudaSuccess;
  const auto t0 = std::chrono::steady_clock::now();
#define HEX_TRY(expr, what)                                  \
  do {                                                       \
    e = (expr);                                              \
    if (e != cudaSuccess) { rc = cuda_error(e, what); goto done; } \
  } while (0)
  {
    HEX_TRY(stage(x, cbytes * nn, on_dev, &own[0], &dx), "stage x");
    HEX_TRY(stage(y, cbytes * nn, on_dev, &own[1], &dy), "stage y");
    HEX_TRY(stage(z, cbytes * nn, on_dev, &own[2], &dz), "stage z");
    HEX_TRY(stage(conn, ibytes * 8 * nc, on_dev, &own[3], &dconn), "stage connectivity");
    const int64_t nf = assoc == GVR_ASSOC_VERTEX ? nn : nc;
    HEX_TRY(stage(field, fbytes * nf, on_dev, &own[4], &dfield), "stage field");
    HEX_TRY(dev_alloc(&d.d_nodes, nn), "alloc nodes");
    HEX_TRY(dev_alloc(&d.d_conn, 2 * nc), "alloc conn");
    HEX_TRY(dev_alloc(&d_flag, 2), "alloc flag");
    HEX_TRY(cudaMemset(d_flag, 0, sizeof(int) * 2), "clear flag");
    pack_nodes_kernel<<<grid_for(nn), 256>>>(dx, dy, dz, cdtype,
                                             assoc == GVR_ASSOC_VERTEX ? dfield : nullptr, fdtype,
                                             nn, d.d_nodes, d_flag);
    count_launch();
    pack_conn_kernel<<<grid_for(nc), 256>>>(dconn, idtype, nc, nn, d.d_conn, d_flag + 1);
    count_launch();
    if (assoc == GVR_ASSOC_ELEMENT) {
      HEX_TRY(dev_alloc(&d.d_cells, nc), "alloc cell field");
      HEX_TRY(launch_cells_field(dfield, fdtype, 1, 1, nc, d.d_cells, d.range, d.stg, 0),
              "cell field");
    }
    int flags[2];
    HEX_TRY(cudaMemcpy(flags, d_flag, sizeof(flags), cudaMemcpyDeviceToHost), "read flags");
    if (flags[0]) { rc = set_error(GVR_ERR_INVALID_ARGUMENT, "hex coordinates or field are not finite"); goto done; }
    if (flags[1]) { rc = set_error(GVR_ERR_INVALID_ARGUMENT, "hex connectivity refers to a missing node"); goto done; }
    HEX_TRY(dev_alloc(&d.d_coef, 8 * nc), "alloc coefficients");
    coef_kernel<<<grid_for(nc), 256>>>(d.d_nodes, d.d_conn, nc, d.d_coef);
    count_launch();

    // cell boxes + scene box
    const int gb = grid_for(nc);
    HEX_TRY(dev_alloc(&leaf_lo, nc), "alloc boxes");
    HEX_TRY(dev_alloc(&leaf_hi, nc), "alloc boxes");
    HEX_TRY(dev_alloc(&part, 6 * (size_t)gb), "alloc box partials");
    cell_box_kernel<<<gb, 256>>>(d.d_nodes, d.d_conn, nc, leaf_lo, leaf_hi, part);
    count_launch();
    std::vector<float> hp(6 * (size_t)gb);
    HEX_TRY(cudaMemcpy(hp.data(), part, sizeof(float) * hp.size(), cudaMemcpyDeviceToHost), "read box");
    float bl[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, bh[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (int b = 0; b < gb; ++b)
      for (int a = 0; a < 3; ++a) {
        bl[a] = std::min(bl[a], hp[6 * b + a]);
        bh[a] = std::max(bh[a], hp[6 * b + 3 + a]);
      }
    float inv[3];
    for (int a = 0; a < 3; ++a) {
      const float ext = bh[a] - bl[a];
      inv[a] = ext == 0.f ? 0.f : 1.f / ext;
      d.dev.lo[a] = bl[a];
      d.dev.hi[a] = bh[a];
      d.bounds[2 * a] = bl[a];
      d.bounds[2 * a + 1] = bh[a];
    }
    // Morton codes, stable sort
    HEX_TRY(dev_alloc(&d.d_codes, nc), "alloc codes");
    HEX_TRY(dev_alloc(&d.d_ids, nc), "alloc ids");
    morton_kernel<<<gb, 256>>>(leaf_lo, leaf_hi, nc, bl[0], bl[1], bl[2], inv[0], inv[1], inv[2],
                               d.d_codes, d.d_ids);
    count_launch();
    HEX_TRY(dev_alloc(&keys_tmp, nc), "alloc sort");
    HEX_TRY(dev_alloc(&vals_tmp, nc), "alloc sort");
    HEX_TRY(dev_alloc(&sort_scr, sort_scratch_words(nc)), "alloc sort");
    HEX_TRY(radix_sort_pairs<uint32_t>(d.d_codes, d.d_ids, keys_tmp, vals_tmp, nc, 30, sort_scr, 0),
            "sort Morton codes");
    // topology + refit + flat layout
    if (nc > 1) {
      const int64_t ni = nc - 1;
      HEX_TRY(dev_alloc(&d.d_left, ni), "alloc tree");
      HEX_TRY(dev_alloc(&d.d_right, ni), "alloc tree");
      HEX_TRY(dev_alloc(&d.d_parent, 2 * nc - 1), "alloc tree");
      HEX_TRY(dev_alloc(&d.d_inner_box, 2 * ni), "alloc tree");
      HEX_TRY(dev_alloc(&counters, ni), "alloc counters");
      HEX_TRY(dev_alloc(&d.d_bvh, 4 * ni), "alloc bvh");
      HEX_TRY(cudaMemset(counters, 0, sizeof(int) * ni), "clear counters");
      karras_kernel<<<grid_for(ni), 256>>>(d.d_codes, (int)nc, d.d_left, d.d_right, d.d_parent);
      count_launch();
      refit_kernel<<<grid_for(nc), 256>>>(leaf_lo, leaf_hi, d.d_ids, (int)nc, d.d_left, d.d_right,
                                          d.d_parent, counters, d.d_inner_box);
      count_launch();
      emit_kernel<<<grid_for(ni), 256>>>(leaf_lo, leaf_hi, d.d_ids, (int)nc, d.d_left, d.d_right,
                                         d.d_inner_box, d.d_bvh);
      count_launch();
    }
    HEX_TRY(cudaGetLastError(), "BVH build launch");
    HEX_TRY(cudaDeviceSynchronize(), "BVH build");
    if (assoc == GVR_ASSOC_VERTEX) {
      rc = node_range(d);
      if (rc != GVR_OK) goto done;
    }
  }
done:
#undef HEX_TRY
  for (void *p : own) cudaFree(p);
  cudaFree(d_flag);
  cudaFree(leaf_lo);
  cudaFree(leaf_hi);
  cudaFree(part);
  cudaFree(keys_tmp);
  cudaFree(vals_tmp);
  cudaFree(sort_scr);
  cudaFree(counters);
  d.bvh_build_ms = std::chrono::duration<float, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (rc == GVR_OK) rc = build_neighbours(d);
  d.dev.hex_nbr = d.d_nbr;
  d.dev.hex_coef = d.d_coef;
  d.dev.hex_nodes = d.d_nodes;
  d.dev.hex_conn = d.d_conn;
  d.dev.hex_bvh = d.d_bvh;
  d.dev.hex_ids = (const int *)d.d_ids;
  d.dev.cells = d.d_cells;
  d.dev.n_cells = (int)nc;
  return rc;
}

}  // namespace gvr

using namespace gvr;

extern "C" {

int gvr_scene_add_hex(gvr_scene *s, int64_t n_nodes, const void *x, const void *y, const void *z,
                      int coord_dtype, int64_t n_cells, const void *conn, int conn_int64,
                      const void *field, int dtype, int association, int location, int *domain_id)
{
  if (!s || !x || !y || !z || !conn || !field)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (n_nodes < 8 || n_cells < 1)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "a hex domain needs >= 8 nodes and >= 1 cell");
  if (n_nodes >= ((int64_t)1 << 31) || n_cells >= ((int64_t)1 << 29))
    return set_error(GVR_ERR_UNSUPPORTED, "hex domains hold < 2^31 nodes and < 2^29 cells");
  if ((coord_dtype != GVR_DTYPE_FLOAT32 && coord_dtype != GVR_DTYPE_FLOAT64) ||
      (dtype != GVR_DTYPE_FLOAT32 && dtype != GVR_DTYPE_FLOAT64))
    return set_error(GVR_ERR_UNSUPPORTED, "coordinates and field must be float32 or float64");
  if (association != GVR_ASSOC_VERTEX && association != GVR_ASSOC_ELEMENT)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad field association");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad location");
  if ((int)s->domains.size() >= kMaxDomains)
    return set_error(GVR_ERR_UNSUPPORTED, "a scene holds at most 64 domains");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  Domain d;
  std::memset(&d.dev, 0, sizeof(d.dev));
  d.dev.kind = GVR_DOMAIN_HEX;
  d.dev.assoc = association;
  d.n_nodes = n_nodes;
  d.n_cells = n_cells;
  d.n_values = association == GVR_ASSOC_VERTEX ? (size_t)n_nodes : (size_t)n_cells;
  int rc = build_hex(d, x, y, z, coord_dtype, conn, conn_int64 ? 1 : 0, field, dtype, association,
                     location);
  if (rc != GVR_OK) {
    free_hex(d);
    cudaFree(d.d_cells);
    cudaFree(d.stg.buf);
    cudaFree(d.stg.block_range);
    return rc;
  }
  s->domains.push_back(d);
  s->table_dirty = true;
  s->classify_valid = false;
  s->has_hex = true;
  if (domain_id) *domain_id = (int)s->domains.size() - 1;
  return GVR_OK;
}

int gvr_scene_hex_bvh(const gvr_scene *s, int domain_id, uint32_t *codes, uint32_t *ids,
                      int32_t *left, int32_t *right, int32_t *parent, float *inner_boxes,
                      float *build_ms)
{
  if (!s || domain_id < 0 || domain_id >= (int)s->domains.size())
    return set_error(GVR_ERR_NOT_FOUND, "no such domain");
  const Domain &d = s->domains[domain_id];
  if (d.dev.kind != GVR_DOMAIN_HEX) return set_error(GVR_ERR_INVALID_ARGUMENT, "not a hex domain");
  cudaError_t e = cudaSetDevice(s->device);
  const int64_t nc = d.n_cells, ni = nc - 1;
  if (e == cudaSuccess && codes) e = cudaMemcpy(codes, d.d_codes, 4 * nc, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && ids) e = cudaMemcpy(ids, d.d_ids, 4 * nc, cudaMemcpyDeviceToHost);
  if (ni > 0) {
    if (e == cudaSuccess && left) e = cudaMemcpy(left, d.d_left, 4 * ni, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && right) e = cudaMemcpy(right, d.d_right, 4 * ni, cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && parent)
      e = cudaMemcpy(parent, d.d_parent, 4 * (2 * nc - 1), cudaMemcpyDeviceToHost);
    if (e == cudaSuccess && inner_boxes) {
      std::vector<float4> b(2 * ni);
      e = cudaMemcpy(b.data(), d.d_inner_box, sizeof(float4) * 2 * ni, cudaMemcpyDeviceToHost);
      for (int64_t i = 0; i < ni && e == cudaSuccess; ++i) {
        const float v[6] = {b[2 * i].x, b[2 * i].y, b[2 * i].z, b[2 * i + 1].x, b[2 * i + 1].y,
                            b[2 * i + 1].z};
        std::memcpy(inner_boxes + 6 * i, v, sizeof(v));
      }
    }
  }
  if (e != cudaSuccess) return cuda_error(e, "copy BVH");
  if (build_ms) *build_ms = d.bvh_build_ms;
  return GVR_OK;
}

int gvr_scene_hex_neighbors(const gvr_scene *s, int domain_id, int32_t *nbr, float *build_ms)
{
  if (!s || domain_id < 0 || domain_id >= (int)s->domains.size())
    return set_error(GVR_ERR_NOT_FOUND, "no such domain");
  const Domain &d = s->domains[domain_id];
  if (d.dev.kind != GVR_DOMAIN_HEX) return set_error(GVR_ERR_INVALID_ARGUMENT, "not a hex domain");
  cudaError_t e = cudaSetDevice(s->device);
  if (e == cudaSuccess && nbr) e = cudaMemcpy(nbr, d.d_nbr, sizeof(int) * 6 * d.n_cells, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "copy neighbours");
  if (build_ms) *build_ms = d.nbr_build_ms;
  return GVR_OK;
}

int gvr_scene_hex_locate(gvr_scene *s, int domain_id, const float *points, int n, int *cells,
                         float *rst)
{
  if (!s || domain_id < 0 || domain_id >= (int)s->domains.size())
    return set_error(GVR_ERR_NOT_FOUND, "no such domain");
  if (n < 0 || (n > 0 && (!points || !cells || !rst)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad point arrays");
  const Domain &d = s->domains[domain_id];
  if (d.dev.kind != GVR_DOMAIN_HEX) return set_error(GVR_ERR_INVALID_ARGUMENT, "not a hex domain");
  if (n == 0) return GVR_OK;
  cudaError_t e = cudaSetDevice(s->device);
  float *dp = nullptr, *dr = nullptr;
  int *dc = nullptr;
  if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(float) * 3 * n);
  if (e == cudaSuccess) e = cudaMalloc(&dr, sizeof(float) * 3 * n);
  if (e == cudaSuccess) e = cudaMalloc(&dc, sizeof(int) * n);
  if (e == cudaSuccess) e = cudaMemcpy(dp, points, sizeof(float) * 3 * n, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    locate_kernel<<<grid_for(n), 256>>>(d.dev, dp, n, dc, dr);
    count_launch();
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(cells, dc, sizeof(int) * n, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(rst, dr, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost);
  cudaFree(dp);
  cudaFree(dr);
  cudaFree(dc);
  if (e != cudaSuccess) return cuda_error(e, "hex locate");
  return GVR_OK;
}

}  // extern "C"
