// gvr_composite.cu — device partial compositing.
//
// Replaces PartialCompositor<VolumePartial<float>>::composite for partials a
// caller already holds (vtkh/compositing/PartialCompositor.cpp:244-547,
// BlendPartials :57-90, VolumePartial::blend VolumePartial.hpp:86-95):
//   1. sort the records by (pixel id, depth) — a stable device radix sort of
//      64-bit keys (pixel id, order-preserving bits of the depth), so records
//      with equal keys keep their input order;
//   2. flag segment heads: pixels with a single record ("unique") and the
//      first record of pixels with several;
//   3. exclusive scans of the two flags give every output slot: unique
//      pixels first, then blended pixels, each in pixel order — the order
//      composite_partials writes (:422-489);
//   4. one thread per multi-record pixel blends its records front to back
//      with VolumePartial::blend. Its arithmetic uses explicitly rounded
//      FP32 operations (no fused multiply-add), so the output is bit-identical
//      to the reference compiled without FMA contraction.
#include <cstdint>

#include "gvr_internal.h"

namespace gvr {
namespace {

using Partial = gvr_partial;
static_assert(sizeof(Partial) == 24, "VolumePartial<float> layout");

// Unsigned key with the order of float <; -0 and +0 compare equal there, so
// both map to the key of +0 (equal keys keep their input order).
__device__ __forceinline__ uint32_t order_bits(float f)
{
  uint32_t u = __float_as_uint(f);
  if (u == 0x80000000u) u = 0u;
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__global__ void key_kernel(const Partial *__restrict__ in, int64_t n, uint64_t *__restrict__ keys,
                           uint32_t *__restrict__ idx)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const Partial p = in[i];
    const uint32_t pid = (uint32_t)p.pixel_id ^ 0x80000000u;  // signed order
    keys[i] = ((uint64_t)pid << 32) | order_bits(p.depth);
    idx[i] = (uint32_t)i;
  }
}

// flags: uniq[i] = 1 for a pixel with one record, multi[i] = 1 for the first
// record of a pixel with several
__global__ void flag_kernel(const uint64_t *__restrict__ keys, int64_t n, uint32_t *__restrict__ uniq,
                            uint32_t *__restrict__ multi)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t pid = (uint32_t)(keys[i] >> 32);
    const bool head = i == 0 || (uint32_t)(keys[i - 1] >> 32) != pid;
    const bool last = i == n - 1 || (uint32_t)(keys[i + 1] >> 32) != pid;
    uniq[i] = head && last;
    multi[i] = head && !last;
  }
}

__global__ void emit_kernel(const Partial *__restrict__ in, const uint64_t *__restrict__ keys,
                            const uint32_t *__restrict__ idx, int64_t n,
                            const uint32_t *__restrict__ upos, const uint32_t *__restrict__ mpos,
                            const uint32_t *__restrict__ uniq, const uint32_t *__restrict__ multi,
                            uint32_t n_unique, Partial *__restrict__ out)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (uniq[i]) {
      out[upos[i]] = in[idx[i]];
    } else if (multi[i]) {
      Partial r = in[idx[i]];
      const uint32_t pid = (uint32_t)(keys[i] >> 32);
      for (int64_t j = i + 1; j < n && (uint32_t)(keys[j] >> 32) == pid; ++j) {
        const Partial o = in[idx[j]];
        // VolumePartial::blend
        if (r.alpha >= 1.f || o.alpha == 0.f) continue;
        const float op = __fsub_rn(1.f, r.alpha);
        r.rgb[0] = __fadd_rn(r.rgb[0], __fmul_rn(op, o.rgb[0]));
        r.rgb[1] = __fadd_rn(r.rgb[1], __fmul_rn(op, o.rgb[1]));
        r.rgb[2] = __fadd_rn(r.rgb[2], __fmul_rn(op, o.rgb[2]));
        r.alpha = __fadd_rn(r.alpha, __fmul_rn(op, o.alpha));
        r.alpha = r.alpha > 1.f ? 1.f : r.alpha;
      }
      out[n_unique + mpos[i]] = r;
    }
  }
}

int grid_of(int64_t n)
{
  const int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

}  // namespace
}  // namespace gvr

using namespace gvr;

extern "C" int gvr_composite_partials(const gvr_partial *partials, int64_t n, gvr_partial *out,
                                      int64_t *n_out, int location, void *stream)
{
  if (!n_out || n < 0 || (n > 0 && (!partials || !out)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad partial arrays");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad location");
  if (n >= ((int64_t)1 << 32) - 1) return set_error(GVR_ERR_UNSUPPORTED, "at most 2^32 - 2 partials");
  *n_out = 0;
  if (n == 0) return GVR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  Partial *d_in = nullptr, *d_out = nullptr;
  uint64_t *keys = nullptr, *keys_tmp = nullptr;
  uint32_t *idx = nullptr, *idx_tmp = nullptr, *scratch = nullptr;
  uint32_t *uniq = nullptr, *multi = nullptr, *upos = nullptr, *mpos = nullptr, *scan_tmp = nullptr;
  cudaError_t e = cudaSuccess;
  int rc = GVR_OK;
  uint32_t last[4] = {0, 0, 0, 0};
  const size_t words = sort_scratch_words(n);
  const size_t swords = scan_scratch_words(n);
#define CP_TRY(expr, what)                                        \
  do {                                                            \
    e = (expr);                                                   \
    if (e != cudaSuccess) { rc = cuda_error(e, what); goto done; } \
  } while (0)
  if (location == GVR_MEM_HOST) {
    CP_TRY(cudaMalloc(&d_in, sizeof(Partial) * n), "cudaMalloc partials");
    CP_TRY(cudaMalloc(&d_out, sizeof(Partial) * n), "cudaMalloc output");
    CP_TRY(cudaMemcpyAsync(d_in, partials, sizeof(Partial) * n, cudaMemcpyHostToDevice, st), "copy partials");
  } else {
    d_in = const_cast<Partial *>(partials);
    d_out = out;
  }
  CP_TRY(cudaMalloc(&keys, sizeof(uint64_t) * n), "cudaMalloc keys");
  CP_TRY(cudaMalloc(&keys_tmp, sizeof(uint64_t) * n), "cudaMalloc keys");
  CP_TRY(cudaMalloc(&idx, sizeof(uint32_t) * n), "cudaMalloc index");
  CP_TRY(cudaMalloc(&idx_tmp, sizeof(uint32_t) * n), "cudaMalloc index");
  CP_TRY(cudaMalloc(&scratch, sizeof(uint32_t) * words), "cudaMalloc sort scratch");
  CP_TRY(cudaMalloc(&uniq, sizeof(uint32_t) * n), "cudaMalloc flags");
  CP_TRY(cudaMalloc(&multi, sizeof(uint32_t) * n), "cudaMalloc flags");
  CP_TRY(cudaMalloc(&upos, sizeof(uint32_t) * n), "cudaMalloc positions");
  CP_TRY(cudaMalloc(&mpos, sizeof(uint32_t) * n), "cudaMalloc positions");
  CP_TRY(cudaMalloc(&scan_tmp, sizeof(uint32_t) * swords), "cudaMalloc scan scratch");
  key_kernel<<<grid_of(n), 256, 0, st>>>(d_in, n, keys, idx);
  count_launch();
  CP_TRY(radix_sort_pairs<uint64_t>(keys, idx, keys_tmp, idx_tmp, n, 64, scratch, st), "sort partials");
  flag_kernel<<<grid_of(n), 256, 0, st>>>(keys, n, uniq, multi);
  count_launch();
  CP_TRY(cudaMemcpyAsync(upos, uniq, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st), "copy flags");
  CP_TRY(cudaMemcpyAsync(mpos, multi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st), "copy flags");
  CP_TRY(exclusive_scan(upos, n, scan_tmp, st), "scan");
  CP_TRY(exclusive_scan(mpos, n, scan_tmp, st), "scan");
  // totals: last exclusive prefix + last flag
  CP_TRY(cudaMemcpyAsync(&last[0], upos + n - 1, 4, cudaMemcpyDeviceToHost, st), "read counts");
  CP_TRY(cudaMemcpyAsync(&last[1], uniq + n - 1, 4, cudaMemcpyDeviceToHost, st), "read counts");
  CP_TRY(cudaMemcpyAsync(&last[2], mpos + n - 1, 4, cudaMemcpyDeviceToHost, st), "read counts");
  CP_TRY(cudaMemcpyAsync(&last[3], multi + n - 1, 4, cudaMemcpyDeviceToHost, st), "read counts");
  CP_TRY(cudaStreamSynchronize(st), "composite");
  {
    const uint32_t n_unique = last[0] + last[1];
    const uint32_t n_multi = last[2] + last[3];
    emit_kernel<<<grid_of(n), 256, 0, st>>>(d_in, keys, idx, n, upos, mpos, uniq, multi, n_unique,
                                            d_out);
    count_launch();
    CP_TRY(cudaGetLastError(), "emit");
    if (location == GVR_MEM_HOST)
      CP_TRY(cudaMemcpyAsync(out, d_out, sizeof(Partial) * (n_unique + n_multi), cudaMemcpyDeviceToHost, st),
             "copy output");
    CP_TRY(cudaStreamSynchronize(st), "composite");
    *n_out = (int64_t)n_unique + n_multi;
  }
done:
#undef CP_TRY
  if (location == GVR_MEM_HOST) {
    cudaFree(d_in);
    cudaFree(d_out);
  }
  cudaFree(keys);
  cudaFree(keys_tmp);
  cudaFree(idx);
  cudaFree(idx_tmp);
  cudaFree(scratch);
  cudaFree(uniq);
  cudaFree(multi);
  cudaFree(upos);
  cudaFree(mpos);
  cudaFree(scan_tmp);
  return rc;
}
