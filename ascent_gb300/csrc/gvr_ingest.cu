// gvr_ingest.cu — field upload into the bricked device layout.
//
// Replaces the field half of the Blueprint -> VTK-m adapter
// (ascent_vtkh_data_adapter.cpp:1782-2040, AddField: float32/float64,
// strided, vertex/element) and the scalar-range pass of
// Renderer::PreExecute (Renderer.cpp:144-179). The output layout is the
// renderer's own: 8^3-cell bricks with a one-node apron plus a per-brick
// {min,max} macrocell grid used for empty-space skipping.
#include <cstdlib>
#include <cstring>
#include <cfloat>
#include <cstdint>
#include <cstdio>

#include "gvr_internal.h"

namespace gvr {
namespace {

__device__ __forceinline__ float load_value(const void *src, int dtype, int64_t i)
{
  return dtype == GVR_DTYPE_FLOAT64 ? (float)((const double *)src)[i]
                                    : ((const float *)src)[i];
}

// One CTA per brick: gather the brick's (2^bshift + 1)^3 nodes (clamped at
// the domain's last node), write them to the brick, and reduce their
// min/max.
__global__ void __launch_bounds__(256)
brick_kernel(const void *__restrict__ src, int dtype, int64_t stride, int nx,
             int ny, int nz, int nbx, int nby, int bshift, float *__restrict__ bricks,
             float2 *__restrict__ brick_range)
{
  const int64_t b = blockIdx.x;
  const int bx = (int)(b % nbx);
  const int by = (int)((b / nbx) % nby);
  const int bz = (int)(b / ((int64_t)nbx * nby));
  const int bc = brick_cells(bshift), bn = brick_nodes(bshift), bf = brick_floats(bshift);
  float vmin = FLT_MAX, vmax = -FLT_MAX;
  int bad = 0;
  float *dst = bricks + b * bf;
  for (int l = threadIdx.x; l < bf; l += blockDim.x) {
    float v = 0.f;
    if (l < bn * bn * bn) {
      const int lx = l % bn;
      const int ly = (l / bn) % bn;
      const int lz = l / (bn * bn);
      const int x = min(bx * bc + lx, nx - 1);
      const int y = min(by * bc + ly, ny - 1);
      const int z = min(bz * bc + lz, nz - 1);
      const int64_t idx = ((int64_t)z * ny + y) * nx + x;
      v = load_value(src, dtype, idx * stride);
      bad |= !isfinite(v);
      vmin = fminf(vmin, v);
      vmax = fmaxf(vmax, v);
    }
    dst[l] = v;
  }
  bad = __syncthreads_or(bad);
  // block min/max
  for (int o = 16; o > 0; o >>= 1) {
    vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  }
  __shared__ float smin[8], smax[8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smin[w] = vmin; smax[w] = vmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      vmin = fminf(vmin, smin[i]);
      vmax = fmaxf(vmax, smax[i]);
    }
    brick_range[b] = bad ? make_float2(NAN, NAN) : make_float2(vmin, vmax);
  }
}

// ---------------------------------------------------------------------
// Staged bricking of contiguous float32 fields. A CTA builds a run of up to
// 16 bricks along x: one thread issues a bulk copy (cp.async.bulk, completing
// on an mbarrier) of each of the run's 81 node rows (9 y x 9 z, ~129 floats
// each) into shared memory, then each warp writes two bricks from there with
// coalesced stores and reduces their min/max. The per-brick kernel above
// reads the same rows as 36-byte fragments. The number of bulk copies, not
// their bytes, bounds this kernel: runs of 8 bricks (81 copies of ~260
// bytes) published 8 x 257^3 in 0.63 ms, runs of 16 in 0.55 ms, runs of 32
// (85 KB of rows, 2 CTAs per SM) in 0.66 ms. A bulk copy must start on a
// 16-byte boundary and move a multiple of 16 bytes: each row's copy starts
// at the boundary at or below its first node and is rounded up; a row whose
// rounded range would leave the field's buffer is filled with plain loads.
// ---------------------------------------------------------------------
constexpr int kRunBricks = 16;
constexpr int kRunNodes = kRunBricks * kBrickCells + 1;   // 129
constexpr int kRowSlot = 136;                             // floats per staged row (544 B)
constexpr int kRows = kBrickNodes * kBrickNodes;          // 81
constexpr long long kStageSpin = 1ll << 22;               // bounded mbarrier wait

__device__ __forceinline__ unsigned smem_u32(const void *p)
{
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool mbar_try_wait(const uint64_t *bar, unsigned phase)
{
  unsigned ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(phase)
      : "memory");
  return ok != 0;
}

// Wait for phase 0 of the barrier, at most `polls` polls.
__device__ __forceinline__ bool mbar_wait_bounded(const uint64_t *bar, long long polls)
{
  for (long long i = 0; i < polls; ++i) {
    if (mbar_try_wait(bar, 0)) return true;
    if (i > 64) __nanosleep(64);
  }
  return false;
}

// One run of up to 16 bricks of one field (the body of both launches below).
__device__ __forceinline__ void brick_run(const float *__restrict__ src, int64_t n_src, int nx, int ny,
                                          int nz, int nbx, int nby, int run, int by, int bz,
                                          float *__restrict__ bricks, float2 *__restrict__ brick_range,
                                          int *__restrict__ timed_out, long long first_polls)
{
  __shared__ __align__(16) float rows[kRows * kRowSlot];
  // brick node l's place in `rows`, less the brick's first x: its row's slot
  // plus the row copy's lead plus its x within the brick (< 2^16)
  __shared__ unsigned short nodeoff[kBrickNodes * kBrickNodes * kBrickNodes];
  __shared__ __align__(8) uint64_t bar;
  static_assert(kRows * kRowSlot < 65536, "node offsets fit 16 bits");
  const int x0 = run * kRunBricks * kBrickCells;
  const int count = min(kRunNodes, nx - x0);
  const uintptr_t base = reinterpret_cast<uintptr_t>(src);
  const uintptr_t end = base + (uintptr_t)n_src * sizeof(float);
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();
  // 16-byte-aligned copy range of row r: start a, size sz (bytes)
  auto row_range = [&](int r, uintptr_t &a, unsigned &sz) {
    const int y = min(by * kBrickCells + r % kBrickNodes, ny - 1);
    const int z = min(bz * kBrickCells + r / kBrickNodes, nz - 1);
    const uintptr_t first = base + ((uintptr_t)(((int64_t)z * ny + y) * nx + x0)) * sizeof(float);
    a = first & ~(uintptr_t)15;
    sz = (unsigned)(((first - a) + (uintptr_t)count * sizeof(float) + 15) & ~(uintptr_t)15);
    return (int)((first - a) / sizeof(float));
  };
  // thread r plans row r: announces its bytes on the barrier and issues its
  // bulk copy (or marks the row for plain loads); thread 0 arrives once all
  // rows are announced, so the phase cannot complete early
  int my_plain = 0;
  if (threadIdx.x < kRows) {
    const int r = threadIdx.x;
    uintptr_t a;
    unsigned sz;
    row_range(r, a, sz);
    my_plain = (a < base || a + sz > end) ? 1 : 0;
    if (!my_plain) {
      asm volatile("mbarrier.expect_tx.relaxed.cta.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(&bar)),
                   "r"(sz)
                   : "memory");
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_u32(rows + r * kRowSlot)),
          "l"(a), "r"(sz), "r"(smem_u32(&bar))
          : "memory");
    }
  }
  const bool any_plain = __syncthreads_or(my_plain);
  if (threadIdx.x == 0)
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&bar)) : "memory");
  // while the copies are in flight: every brick node's offset in `rows`
  constexpr int kNodes = kBrickNodes * kBrickNodes * kBrickNodes;   // 729
  for (int l = threadIdx.x; l < kNodes; l += blockDim.x) {
    const int rr = l / kBrickNodes;
    uintptr_t a;
    unsigned sz;
    nodeoff[l] = (unsigned short)(rr * kRowSlot + row_range(rr, a, sz) + (l - kBrickNodes * rr));
  }
  __syncthreads();
  bool ok = mbar_wait_bounded(&bar, first_polls);
  // rows that could not be copied in bulk (only next to the end of the
  // field's buffer): plain loads
  if (any_plain) {
    for (int r = 0; r < kRows; ++r) {
      uintptr_t a;
      unsigned sz;
      const int lead = row_range(r, a, sz);
      if (!(a < base || a + sz > end)) continue;
      const int y = min(by * kBrickCells + r % kBrickNodes, ny - 1);
      const int z = min(bz * kBrickCells + r / kBrickNodes, nz - 1);
      const float *row = src + ((int64_t)z * ny + y) * nx + x0;
      for (int i = threadIdx.x; i < count; i += blockDim.x) rows[r * kRowSlot + lead + i] = row[i];
    }
  }
  if (!ok) {
    atomicOr(timed_out, 1);
    // The copies may still land in shared memory: wait for them once more,
    // for the full bound. If this wait gives up too, the block goes on and
    // exits while copies may still be landing in its shared memory; the
    // bricks it writes are marked non-finite either way, and the host reports
    // GVR_ERR_TIMEOUT. Only a copy that takes longer than both bounds
    // together (seconds) reaches that case.
    mbar_wait_bounded(&bar, kStageSpin);
  }
  __syncthreads();
  // warp w writes bricks run * 16 + w and run * 16 + 8 + w: lane i takes
  // nodes i, i + 32, ... (consecutive lanes read neighbouring nodes of a
  // row, so the shared-memory reads hardly conflict, and store 128
  // contiguous bytes per warp and step). A brick whose nodes all lie in the
  // field reads them at nodeoff + its first x; the last brick of a row that
  // ends inside a brick clamps x to the field's last node.
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x_last = nx - 1 - x0;   // last node of the field, relative to the run
  for (int half = 0; half < kRunBricks / 8; ++half) {
    const int bx = run * kRunBricks + half * 8 + w;
    if (bx >= nbx) return;
    const int64_t b = ((int64_t)bz * nby + by) * nbx + bx;
    float *dst = bricks + b * kBrickFloats;
    const int xb = bx * kBrickCells - x0;
    float vmin = FLT_MAX, vmax = -FLT_MAX;
    float nf = 0.f;   // 0 * node summed: NaN once a node is NaN or infinite
    if (xb + kBrickCells <= x_last) {
#pragma unroll
      for (int s = 0; s < kBrickFloats / 32; ++s) {
        const int l = lane + 32 * s;
        float t = 0.f;
        if (l < kNodes) {
          t = rows[nodeoff[l] + xb];
          nf = fmaf(t, 0.f, nf);
          vmin = fminf(vmin, t);
          vmax = fmaxf(vmax, t);
        }
        dst[l] = t;
      }
    } else {
      for (int l = lane; l < kBrickFloats; l += 32) {
        float t = 0.f;
        if (l < kNodes) {
          const int node = l % kBrickNodes;
          t = rows[nodeoff[l] - node + min(xb + node, x_last)];
          nf = fmaf(t, 0.f, nf);
          vmin = fminf(vmin, t);
          vmax = fmaxf(vmax, t);
        }
        dst[l] = t;
      }
    }
    int bad = !ok || !(nf == 0.f);
    bad = __any_sync(0xffffffffu, bad);
    for (int o = 16; o > 0; o >>= 1) {
      vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
      vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
    }
    if (lane == 0) brick_range[b] = bad ? make_float2(NAN, NAN) : make_float2(vmin, vmax);
  }
}

__global__ void __launch_bounds__(256, 5)   // 5 CTAs per SM: 44 KB of rows each
brick_staged_kernel(const float *__restrict__ src, int64_t n_src, int nx, int ny, int nz, int nbx,
                    int nby, float *__restrict__ bricks, float2 *__restrict__ brick_range,
                    int *__restrict__ timed_out, long long first_polls)
{
  brick_run(src, n_src, nx, ny, nz, nbx, nby, blockIdx.x, blockIdx.y, blockIdx.z, bricks, brick_range,
            timed_out, first_polls);
}

// Many fields in one launch (a device-resident publish): block b belongs to
// the job whose [first, first of the next) block range holds it and runs
// that field's run (b - first) % runs, row by, layer bz. One launch instead
// of one per domain lets the domains' tails overlap.
struct StagedJobs {
  const float *src[kMaxDomains];
  float *bricks[kMaxDomains];
  float2 *brick_range[kMaxDomains];
  int64_t n_src[kMaxDomains];
  int dims[kMaxDomains][3];
  int nbrick[kMaxDomains][3];
  int runs[kMaxDomains];
  int first[kMaxDomains + 1];   // first block of each job; first[n] = total
  int n;
};

__global__ void __launch_bounds__(256, 5)   // 5 CTAs per SM: 44 KB of rows each
brick_staged_multi_kernel(const __grid_constant__ StagedJobs jobs, int *__restrict__ timed_out,
                          long long first_polls)
{
  const int b = blockIdx.x;
  int j = 0;
  while (j + 1 < jobs.n && b >= jobs.first[j + 1]) ++j;
  const int local = b - jobs.first[j];
  const int run = local % jobs.runs[j];
  const int by = (local / jobs.runs[j]) % jobs.nbrick[j][1];
  const int bz = local / (jobs.runs[j] * jobs.nbrick[j][1]);
  brick_run(jobs.src[j], jobs.n_src[j], jobs.dims[j][0], jobs.dims[j][1], jobs.dims[j][2],
            jobs.nbrick[j][0], jobs.nbrick[j][1], run, by, bz, jobs.bricks[j], jobs.brick_range[j],
            timed_out, first_polls);
}

}  // namespace

namespace {

// Poll limit of the staged kernel's first wait for its bulk copies:
// kStageSpin, or GVR_STAGE_WAIT_POLLS from the environment (0 .. kStageSpin),
// read at every launch. Setting it to 0 makes every first wait give up at
// once, which exercises the timeout path (flag, non-finite ranges,
// GVR_ERR_TIMEOUT) while the second, full-length wait still lets the copies
// land before the block exits.
long long stage_first_polls()
{
  const char *v = getenv("GVR_STAGE_WAIT_POLLS");
  if (!v || !*v) return kStageSpin;
  char *end = nullptr;
  const long long n = strtoll(v, &end, 10);
  if (end == v || n < 0) return kStageSpin;
  return n < kStageSpin ? n : kStageSpin;
}

// Brick a field in device memory: the staged kernel for contiguous float32
// fields in 8^3-cell bricks, the per-brick gather otherwise.
cudaError_t launch_bricks(const void *dsrc, int dtype, int64_t stride, const int dims[3],
                          int bshift, float *d_bricks, const int nbrick[3], float2 *d_brick_range,
                          int *d_timed_out, cudaStream_t stream)
{
  const int64_t nb = (int64_t)nbrick[0] * nbrick[1] * nbrick[2];
  if (dtype == GVR_DTYPE_FLOAT32 && stride == 1 && bshift == kBrickShiftDefault) {
    const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
    dim3 grid((unsigned)((nbrick[0] + kRunBricks - 1) / kRunBricks), (unsigned)nbrick[1],
              (unsigned)nbrick[2]);
    brick_staged_kernel<<<grid, 256, 0, stream>>>((const float *)dsrc, n, dims[0], dims[1], dims[2],
                                                  nbrick[0], nbrick[1], d_bricks, d_brick_range,
                                                  d_timed_out, stage_first_polls());
  } else {
    brick_kernel<<<(unsigned)nb, 256, 0, stream>>>(dsrc, dtype, stride, dims[0], dims[1], dims[2],
                                                   nbrick[0], nbrick[1], bshift, d_bricks,
                                                   d_brick_range);
  }
  count_launch();
  return cudaGetLastError();
}

// Strided float32/float64 -> contiguous float32 with per-CTA min/max.
__global__ void __launch_bounds__(256)
convert_kernel(const void *__restrict__ src, int dtype, int64_t stride, int64_t n,
               float *__restrict__ dst, float2 *__restrict__ block_range)
{
  float vmin = FLT_MAX, vmax = -FLT_MAX;
  int bad = 0;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const float v = load_value(src, dtype, i * stride);
    bad |= !isfinite(v);
    dst[i] = v;
    vmin = fminf(vmin, v);
    vmax = fmaxf(vmax, v);
  }
  bad = __syncthreads_or(bad);
  for (int o = 16; o > 0; o >>= 1) {
    vmin = fminf(vmin, __shfl_xor_sync(0xffffffffu, vmin, o));
    vmax = fmaxf(vmax, __shfl_xor_sync(0xffffffffu, vmax, o));
  }
  __shared__ float smin[8], smax[8];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (lane == 0) { smin[w] = vmin; smax[w] = vmax; }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      vmin = fminf(vmin, smin[i]);
      vmax = fmaxf(vmax, smax[i]);
    }
    block_range[blockIdx.x] = bad ? make_float2(NAN, NAN) : make_float2(vmin, vmax);
  }
}

// A brick is empty when the transfer function's opacity is zero over every
// LUT entry its scalar range can reach.
__global__ void empty_kernel(const float2 *__restrict__ brick_range, int64_t n,
                             const float4 *__restrict__ lut, int lut_size,
                             int lut_filter, float smin, float inv_range,
                             uint8_t *__restrict__ empty, int *__restrict__ any_empty)
{
  for (int64_t b = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; b < n;
       b += (int64_t)gridDim.x * blockDim.x) {
    const float2 r = brick_range[b];
    const float s0 = __saturatef((r.x - smin) * inv_range);
    const float s1 = __saturatef((r.y - smin) * inv_range);
    const float x0 = s0 * (float)(lut_size - 1);
    const float x1 = s1 * (float)(lut_size - 1);
    int i0 = (int)x0;
    int i1 = lut_filter == GVR_LUT_LINEAR ? (int)ceilf(x1) : (int)x1;
    i0 = max(0, min(i0, lut_size - 1));
    i1 = max(0, min(i1, lut_size - 1));
    uint8_t e = 1;
    for (int i = i0; i <= i1; ++i)
      if (lut[i].w > 0.f) { e = 0; break; }
    empty[b] = e;
    if (e) *any_empty = 1;
  }
}

// Device-side source of a field upload: the caller's pointer when it is
// device memory, else the domain's staging buffer (grown once, reused by
// every later upload) filled from the host.
cudaError_t stage_source(const void *src, int dtype, int64_t stride,
                         int src_on_device, int64_t n, const void **dsrc,
                         Staging &stg, cudaStream_t stream)
{
  if (src_on_device) {
    *dsrc = src;
    return cudaSuccess;
  }
  const size_t esz = dtype == GVR_DTYPE_FLOAT64 ? 8 : 4;
  const size_t bytes = (size_t)((n - 1) * stride + 1) * esz;
  if (bytes > stg.bytes) {
    cudaFree(stg.buf);
    stg.buf = nullptr;
    stg.bytes = 0;
    cudaError_t e = cudaMalloc(&stg.buf, bytes);
    if (e != cudaSuccess) return e;
    stg.bytes = bytes;
  }
  *dsrc = stg.buf;
  return cudaMemcpyAsync(stg.buf, src, bytes, cudaMemcpyHostToDevice, stream);
}

}  // namespace

cudaError_t launch_brick_field(const void *src, int dtype, int64_t stride,
                               int src_on_device, const int dims[3], int bshift,
                               float *d_bricks, const int nbrick[3],
                               float2 *d_brick_range, double range_out[2],
                               Staging &stg, int *d_timed_out, bool *timed_out,
                               cudaStream_t stream)
{
  const int64_t n = (int64_t)dims[0] * dims[1] * dims[2];
  const void *dsrc = nullptr;
  cudaError_t e = stage_source(src, dtype, stride, src_on_device, n, &dsrc, stg, stream);
  if (e != cudaSuccess) return e;
  const int64_t nb = (int64_t)nbrick[0] * nbrick[1] * nbrick[2];
  e = cudaMemsetAsync(d_timed_out, 0, sizeof(int), stream);
  if (e != cudaSuccess) return e;
  e = launch_bricks(dsrc, dtype, stride, dims, bshift, d_bricks, nbrick, d_brick_range, d_timed_out,
                    stream);
  if (e != cudaSuccess) return e;
  std::vector<float2> h((size_t)nb);
  int flag = 0;
  e = cudaMemcpyAsync(h.data(), d_brick_range, sizeof(float2) * nb,
                      cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(&flag, d_timed_out, sizeof(int), cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  *timed_out = flag != 0;
  double lo = INFINITY, hi = -INFINITY;
  for (const float2 &r : h) {
    if (r.x != r.x || r.y != r.y) { lo = NAN; hi = NAN; break; }
    lo = r.x < lo ? r.x : lo;
    hi = r.y > hi ? r.y : hi;
  }
  range_out[0] = lo;
  range_out[1] = hi;
  return cudaSuccess;
}

namespace {

// Jobs of one range reduction launch: one block per domain.
constexpr int kRangeJobs = 64;
struct RangeJobs {
  const float2 *ranges[kRangeJobs];
  int64_t n_bricks[kRangeJobs];
  float2 *out[kRangeJobs];
};

// Block j: min and max over domain j's per-brick ranges into *out[j] (NaN
// when any brick holds a non-finite value).
__global__ void __launch_bounds__(1024) range_of_bricks_kernel(const RangeJobs jobs)
{
  __shared__ float lo_s[32], hi_s[32];
  __shared__ int bad_s;
  const float2 *__restrict__ r = jobs.ranges[blockIdx.x];
  const int64_t nb = jobs.n_bricks[blockIdx.x];
  if (threadIdx.x == 0) bad_s = 0;
  __syncthreads();
  float lo = INFINITY, hi = -INFINITY;
  int bad = 0;
  for (int64_t i = threadIdx.x; i < nb; i += blockDim.x) {
    const float2 v = r[i];
    if (v.x != v.x || v.y != v.y) bad = 1;
    lo = fminf(lo, v.x);
    hi = fmaxf(hi, v.y);
  }
  for (int o = 16; o > 0; o >>= 1) {
    lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, o));
    hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, o));
  }
  if (bad) atomicOr(&bad_s, 1);
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    lo_s[w] = lo;
    hi_s[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int i = 1; i < (int)(blockDim.x >> 5); ++i) {
      lo = fminf(lo, lo_s[i]);
      hi = fmaxf(hi, hi_s[i]);
    }
    *jobs.out[blockIdx.x] = bad_s ? make_float2(NAN, NAN) : make_float2(lo, hi);
  }
}

}  // namespace

cudaError_t launch_brick_device_many(int n, const float *const *srcs, const int (*dims)[3],
                                     float *const *bricks, const int (*nbrick)[3],
                                     float2 *const *brick_range, int *d_timed_out, cudaStream_t stream)
{
  if (n < 1 || n > kMaxDomains) return cudaErrorInvalidValue;
  StagedJobs jobs;
  std::memset(static_cast<void *>(&jobs), 0, sizeof(jobs));
  jobs.n = n;
  int64_t total = 0;
  for (int j = 0; j < n; ++j) {
    jobs.src[j] = srcs[j];
    jobs.bricks[j] = bricks[j];
    jobs.brick_range[j] = brick_range[j];
    jobs.n_src[j] = (int64_t)dims[j][0] * dims[j][1] * dims[j][2];
    for (int a = 0; a < 3; ++a) {
      jobs.dims[j][a] = dims[j][a];
      jobs.nbrick[j][a] = nbrick[j][a];
    }
    jobs.runs[j] = (nbrick[j][0] + kRunBricks - 1) / kRunBricks;
    jobs.first[j] = (int)total;
    total += (int64_t)jobs.runs[j] * nbrick[j][1] * nbrick[j][2];
    if (total >= ((int64_t)1 << 31)) return cudaErrorInvalidValue;
  }
  jobs.first[n] = (int)total;
  brick_staged_multi_kernel<<<(unsigned)total, 256, 0, stream>>>(jobs, d_timed_out, stage_first_polls());
  count_launch();
  return cudaGetLastError();
}

cudaError_t launch_brick_device(const void *dsrc, int dtype, int64_t stride, const int dims[3],
                                int bshift, float *d_bricks, const int nbrick[3],
                                float2 *d_brick_range, int *d_timed_out, cudaStream_t stream)
{
  return launch_bricks(dsrc, dtype, stride, dims, bshift, d_bricks, nbrick, d_brick_range,
                       d_timed_out, stream);
}

cudaError_t launch_ranges_of_bricks(int n, const float2 *const *brick_ranges,
                                    const int64_t *n_bricks, float2 *const *out,
                                    cudaStream_t stream)
{
  for (int j0 = 0; j0 < n; j0 += kRangeJobs) {
    RangeJobs jobs{};
    const int m = std::min(kRangeJobs, n - j0);
    for (int j = 0; j < m; ++j) {
      jobs.ranges[j] = brick_ranges[j0 + j];
      jobs.n_bricks[j] = n_bricks[j0 + j];
      jobs.out[j] = out[j0 + j];
    }
    range_of_bricks_kernel<<<m, 1024, 0, stream>>>(jobs);
    count_launch();
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t launch_cells_field(const void *src, int dtype, int64_t stride,
                               int src_on_device, int64_t n, float *d_cells,
                               double range_out[2], Staging &stg, cudaStream_t stream)
{
  const void *dsrc = nullptr;
  cudaError_t e = stage_source(src, dtype, stride, src_on_device, n, &dsrc, stg, stream);
  if (e != cudaSuccess) return e;
  int blocks = (int)((n + 255) / 256);
  if (blocks > 4096) blocks = 4096;
  if (!stg.block_range) {
    e = cudaMalloc(&stg.block_range, sizeof(float2) * 4096);
    if (e != cudaSuccess) return e;
  }
  float2 *d_br = stg.block_range;
  convert_kernel<<<blocks, 256, 0, stream>>>(dsrc, dtype, stride, n, d_cells, d_br);
  count_launch();
  e = cudaGetLastError();
  std::vector<float2> h(blocks);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(h.data(), d_br, sizeof(float2) * blocks, cudaMemcpyDeviceToHost, stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
  if (e != cudaSuccess) return e;
  double lo = INFINITY, hi = -INFINITY;
  for (const float2 &r : h) {
    if (r.x != r.x || r.y != r.y) { lo = NAN; hi = NAN; break; }
    lo = r.x < lo ? r.x : lo;
    hi = r.y > hi ? r.y : hi;
  }
  range_out[0] = lo;
  range_out[1] = hi;
  return cudaSuccess;
}

cudaError_t launch_empty_bricks(const float2 *brick_range, int64_t n_bricks,
                                const float4 *d_lut, int lut_size, int lut_filter,
                                float scalar_min, float inv_range,
                                uint8_t *brick_empty, int *any_empty, cudaStream_t stream)
{
  if (n_bricks == 0) return cudaSuccess;
  int blocks = (int)((n_bricks + 255) / 256);
  if (blocks > 1216) blocks = 1216;
  empty_kernel<<<blocks, 256, 0, stream>>>(brick_range, n_bricks, d_lut, lut_size,
                                           lut_filter, scalar_min, inv_range, brick_empty,
                                           any_empty);
  count_launch();
  return cudaGetLastError();
}

}  // namespace gvr
