// gvr_composite.cu — device partial compositing.
//
// Replaces PartialCompositor<VolumePartial<float>>::composite for partials a
// caller already holds (vtkh/compositing/PartialCompositor.cpp:244-547,
// BlendPartials :57-90, VolumePartial::blend VolumePartial.hpp:53-62). The
// result is the reference's: records ordered by (pixel id, depth) with
// equal keys in input order; pixels with one record are copied, the others
// blended front to back; output = single-record pixels in pixel order, then
// blended pixels in pixel order (composite_partials :422-489). The blend
// uses explicitly rounded FP32 operations (no fused multiply-add), so the
// output is bit-identical to the reference compiled without contraction.
//
// Two ways to group the records by pixel:
//   dense ids (pixel range <= 2 n + 64 Ki, the normal case: ids are y*W+x)
//     a per-pixel histogram whose atomics also hand every record its slot
//     in its pixel's bucket, scans over the pixel range for the bucket
//     offsets and for the output slots, and one thread per pixel that
//     orders its few records by (depth, input index) and blends them;
//   sparse ids
//     a stable device radix sort of 64-bit keys (pixel id, order-preserving
//     depth bits), segment flags and scans, one thread per blended pixel.
// Scratch comes from the library's stream-ordered memory pool
// (scratch_alloc), which keeps its memory between calls.
#include <algorithm>
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

__device__ __forceinline__ void blend_into(Partial &r, const Partial &o)
{
  // VolumePartial::blend
  if (r.alpha >= 1.f || o.alpha == 0.f) return;
  const float op = __fsub_rn(1.f, r.alpha);
  r.rgb[0] = __fadd_rn(r.rgb[0], __fmul_rn(op, o.rgb[0]));
  r.rgb[1] = __fadd_rn(r.rgb[1], __fmul_rn(op, o.rgb[1]));
  r.rgb[2] = __fadd_rn(r.rgb[2], __fmul_rn(op, o.rgb[2]));
  r.alpha = __fadd_rn(r.alpha, __fmul_rn(op, o.alpha));
  r.alpha = r.alpha > 1.f ? 1.f : r.alpha;
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

// Unique and blended pixel counts of the sorted path: last exclusive
// prefix plus last flag.
__global__ void sorted_totals_kernel(const uint32_t *upos, const uint32_t *uniq, const uint32_t *mpos,
                                     const uint32_t *multi, int64_t n, uint32_t *totals)
{
  if (threadIdx.x == 0) {
    totals[0] = upos[n - 1] + uniq[n - 1];
    totals[1] = mpos[n - 1] + multi[n - 1];
  }
}

__global__ void emit_kernel(const Partial *__restrict__ in, const uint64_t *__restrict__ keys,
                            const uint32_t *__restrict__ idx, int64_t n,
                            const uint32_t *__restrict__ upos, const uint32_t *__restrict__ mpos,
                            const uint32_t *__restrict__ uniq, const uint32_t *__restrict__ multi,
                            const uint32_t *__restrict__ totals, Partial *__restrict__ out)
{
  const uint32_t n_unique = totals[0];
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    if (uniq[i]) {
      out[upos[i]] = in[idx[i]];
    } else if (multi[i]) {
      Partial r = in[idx[i]];
      const uint32_t pid = (uint32_t)(keys[i] >> 32);
      for (int64_t j = i + 1; j < n && (uint32_t)(keys[j] >> 32) == pid; ++j) blend_into(r, in[idx[j]]);
      out[n_unique + mpos[i]] = r;
    }
  }
}

// Smallest and largest pixel id, as order-preserving unsigned values
// (mm[0] starts at 0xffffffff, mm[1] at 0).
__global__ void range_kernel(const Partial *__restrict__ in, int64_t n, unsigned *__restrict__ mm)
{
  unsigned lo = 0xffffffffu, hi = 0u;
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const unsigned u = (unsigned)in[i].pixel_id ^ 0x80000000u;
    lo = min(lo, u);
    hi = max(hi, u);
  }
  lo = __reduce_min_sync(0xffffffffu, lo);
  hi = __reduce_max_sync(0xffffffffu, hi);
  // one pair of atomics per block, not per warp (thousands of warps on two
  // addresses serialise at L2)
  __shared__ unsigned slo[32], shi[32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    slo[w] = lo;
    shi[w] = hi;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    const int nw = (int)(blockDim.x >> 5);
    lo = threadIdx.x < nw ? slo[threadIdx.x] : 0xffffffffu;
    hi = threadIdx.x < nw ? shi[threadIdx.x] : 0u;
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (threadIdx.x == 0) {
      atomicMin(mm, lo);
      atomicMax(mm + 1, hi);
    }
  }
}

// cnt[p] = records of pixel lo + p; pr[i] = {p, record i's slot in its
// bucket} (slots in arrival order; the emit kernel restores input order),
// so that the bucket pass reads 8 bytes per record instead of the 24-byte
// records again. A record whose id lies outside [lo, lo + r) (possible only
// when the caller gave the range) is left out (p = 0xffffffff) and sets
// *bad.
__global__ void count_kernel(const Partial *__restrict__ in, int64_t n, int lo, int64_t r,
                             uint32_t *__restrict__ cnt, uint2 *__restrict__ pr,
                             unsigned *__restrict__ bad)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const int64_t p = (int64_t)in[i].pixel_id - lo;
    if (p < 0 || p >= r) {
      atomicOr(bad, 1u);
      pr[i] = make_uint2(0xffffffffu, 0u);
      continue;
    }
    pr[i] = make_uint2((uint32_t)p, atomicAdd(cnt + p, 1u));
  }
}

__global__ void bucket_kernel(const uint2 *__restrict__ pr, int64_t n, int64_t r,
                              const uint32_t *__restrict__ off, uint32_t *__restrict__ order)
{
  for (int64_t i = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; i < n;
       i += (int64_t)gridDim.x * blockDim.x) {
    const uint2 v = pr[i];
    if ((int64_t)v.x >= r) continue;
    order[off[v.x] + v.y] = (uint32_t)i;
  }
}

// Output count of the caller-range path into the caller's device int64:
// -1 when a record's pixel id was outside the given range.
__global__ void count_out_kernel(const uint32_t *__restrict__ totals, const unsigned *__restrict__ bad,
                                 int64_t *__restrict__ n_out)
{
  if (threadIdx.x == 0) *n_out = *bad ? -1 : (int64_t)totals[0] + totals[1];
}

// upos[p] = 1 for pixels with one record, mpos[p] = 1 for pixels with more
// (scanned in place afterwards into output slots).
__global__ void pixel_flag_kernel(const uint32_t *__restrict__ cnt, int64_t r,
                                  uint32_t *__restrict__ upos, uint32_t *__restrict__ mpos)
{
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < r;
       p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cnt[p];
    upos[p] = c == 1;
    mpos[p] = c > 1;
  }
}

// The three pixel scans of the dense path in one pass over the counts:
// off = exclusive scan of cnt (bucket offsets), upos / mpos = exclusive
// scans of (cnt == 1) / (cnt > 1) (output slots). A tile of kTile3 pixels
// per block writes its local prefixes and its totals; one block scans the
// tile totals (at most kTile3 tiles, so r <= kTile3^2); a last pass adds
// each tile's base. Replaces a copy, a flag kernel and three three-launch
// scans (11 operations) by three launches.
constexpr int kTile3 = 1024;

__device__ __forceinline__ uint3 add3(uint3 a, uint3 b) { return make_uint3(a.x + b.x, a.y + b.y, a.z + b.z); }

// Inclusive block scan of one uint3 per thread (kTile3 threads); returns the
// thread's inclusive prefix, *tot receives the block total.
__device__ __forceinline__ uint3 block_scan3(uint3 v, uint3 *tot)
{
  __shared__ uint3 warp_tot[kTile3 / 32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint3 x = v;
  for (int o = 1; o < 32; o <<= 1) {
    uint3 y;
    y.x = __shfl_up_sync(0xffffffffu, x.x, o);
    y.y = __shfl_up_sync(0xffffffffu, x.y, o);
    y.z = __shfl_up_sync(0xffffffffu, x.z, o);
    if (lane >= o) x = add3(x, y);
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint3 t = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      uint3 y;
      y.x = __shfl_up_sync(0xffffffffu, t.x, o);
      y.y = __shfl_up_sync(0xffffffffu, t.y, o);
      y.z = __shfl_up_sync(0xffffffffu, t.z, o);
      if (lane >= o) t = add3(t, y);
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  if (warp > 0) x = add3(x, warp_tot[warp - 1]);
  *tot = warp_tot[kTile3 / 32 - 1];
  return x;
}

__global__ void __launch_bounds__(kTile3)
scan3_tile_kernel(const uint32_t *__restrict__ cnt, int64_t r, uint32_t *__restrict__ off,
                  uint32_t *__restrict__ upos, uint32_t *__restrict__ mpos, uint3 *__restrict__ sums)
{
  const int64_t p = (int64_t)blockIdx.x * kTile3 + threadIdx.x;
  const uint32_t c = p < r ? cnt[p] : 0u;
  const uint3 v = make_uint3(c, c == 1, c > 1);
  uint3 tot;
  const uint3 inc = block_scan3(v, &tot);
  if (p < r) {
    off[p] = inc.x - v.x;
    upos[p] = inc.y - v.y;
    mpos[p] = inc.z - v.z;
  }
  if (threadIdx.x == 0) sums[blockIdx.x] = tot;
}

// One block: exclusive scan of the tile totals in place.
__global__ void __launch_bounds__(kTile3) scan3_top_kernel(uint3 *__restrict__ sums, int tiles)
{
  const uint3 v = threadIdx.x < tiles ? sums[threadIdx.x] : make_uint3(0u, 0u, 0u);
  uint3 tot;
  const uint3 inc = block_scan3(v, &tot);
  if (threadIdx.x < tiles) sums[threadIdx.x] = make_uint3(inc.x - v.x, inc.y - v.y, inc.z - v.z);
}

__global__ void __launch_bounds__(kTile3)
scan3_add_kernel(int64_t r, uint32_t *__restrict__ off, uint32_t *__restrict__ upos,
                 uint32_t *__restrict__ mpos, const uint3 *__restrict__ sums)
{
  const int64_t p = (int64_t)blockIdx.x * kTile3 + threadIdx.x;
  if (p >= r) return;
  const uint3 b = sums[blockIdx.x];
  off[p] += b.x;
  upos[p] += b.y;
  mpos[p] += b.z;
}

constexpr int kLocalSort = 32;  // records per pixel ordered in thread-local arrays

__device__ __forceinline__ bool before(uint32_t ka, uint32_t ia, uint32_t kb, uint32_t ib)
{
  return ka < kb || (ka == kb && ia < ib);
}

// One thread per pixel: copy or blend its records in (depth, input index)
// order. totals[0..1] receive the unique and blended pixel counts.
__global__ void pixel_emit_kernel(const Partial *__restrict__ in, const uint32_t *__restrict__ cnt,
                                  const uint32_t *__restrict__ off, const uint32_t *__restrict__ upos,
                                  const uint32_t *__restrict__ mpos, uint32_t *__restrict__ order,
                                  int64_t r, Partial *__restrict__ out, uint32_t *__restrict__ totals)
{
  const uint32_t n_unique = upos[r - 1] + (cnt[r - 1] == 1);
  for (int64_t p = (int64_t)blockIdx.x * blockDim.x + threadIdx.x; p < r;
       p += (int64_t)gridDim.x * blockDim.x) {
    const uint32_t c = cnt[p];
    if (p == r - 1) {
      totals[0] = n_unique;
      totals[1] = mpos[p] + (c > 1);
    }
    if (c == 0) continue;
    uint32_t *seg = order + off[p];
    if (c == 1) {
      out[upos[p]] = in[seg[0]];
      continue;
    }
    Partial res;
    if (c <= 8) {
      // the common case (one record per partial image, at most 8 images):
      // keys and indices in registers, ordered by Batcher's odd-even merge
      // network for 8 inputs (19 compare-exchanges; padding sorts last)
      uint32_t key[8], idx[8];
#pragma unroll
      for (int j = 0; j < 8; ++j) {
        if ((uint32_t)j < c) {
          const uint32_t i = seg[j];
          key[j] = order_bits(in[i].depth);
          idx[j] = i;
        } else {
          key[j] = 0xffffffffu;
          idx[j] = 0xffffffffu;
        }
      }
      auto cx = [&](int a, int b) {
        if (before(key[b], idx[b], key[a], idx[a])) {
          const uint32_t tk = key[a], ti = idx[a];
          key[a] = key[b];
          idx[a] = idx[b];
          key[b] = tk;
          idx[b] = ti;
        }
      };
      cx(0, 1); cx(2, 3); cx(4, 5); cx(6, 7);
      cx(0, 2); cx(1, 3); cx(4, 6); cx(5, 7);
      cx(1, 2); cx(5, 6);
      cx(0, 4); cx(1, 5); cx(2, 6); cx(3, 7);
      cx(2, 4); cx(3, 5);
      cx(1, 2); cx(3, 4); cx(5, 6);
      res = in[idx[0]];
#pragma unroll
      for (int j = 1; j < 8; ++j)
        if ((uint32_t)j < c) blend_into(res, in[idx[j]]);
    } else if (c <= kLocalSort) {
      uint32_t key[kLocalSort], idx[kLocalSort];
      for (uint32_t j = 0; j < c; ++j) {
        const uint32_t i = seg[j];
        const uint32_t k = order_bits(in[i].depth);
        uint32_t q = j;
        while (q > 0 && before(k, i, key[q - 1], idx[q - 1])) {
          key[q] = key[q - 1];
          idx[q] = idx[q - 1];
          --q;
        }
        key[q] = k;
        idx[q] = i;
      }
      res = in[idx[0]];
      for (uint32_t j = 1; j < c; ++j) blend_into(res, in[idx[j]]);
    } else {
      // rare deep pixels: insertion sort of the bucket in place
      for (uint32_t j = 1; j < c; ++j) {
        const uint32_t i = seg[j];
        const uint32_t k = order_bits(in[i].depth);
        uint32_t q = j;
        while (q > 0) {
          const uint32_t pi = seg[q - 1];
          if (!before(k, i, order_bits(in[pi].depth), pi)) break;
          seg[q] = pi;
          --q;
        }
        seg[q] = i;
      }
      res = in[seg[0]];
      for (uint32_t j = 1; j < c; ++j) blend_into(res, in[seg[j]]);
    }
    out[n_unique + mpos[p]] = res;
  }
}

int grid_of(int64_t n)
{
  const int64_t b = (n + 255) / 256;
  return (int)(b < 1 ? 1 : (b > 152 * 32 ? 152 * 32 : b));
}

// Scratch of one call, carved from a single stream-ordered allocation.
struct Arena {
  char *base = nullptr;
  size_t used = 0;
  template <typename T>
  T *take(size_t count)
  {
    T *p = reinterpret_cast<T *>(base + used);
    used += (sizeof(T) * std::max<size_t>(count, 1) + 255) & ~(size_t)255;
    return p;
  }
};

size_t dense_bytes(int64_t n, int64_t r)
{
  return 256 * 9 + (4 * (size_t)r + 3 * (size_t)n + std::max<size_t>(scan_scratch_words(r), 3 * 1024) + 3) *
                       sizeof(uint32_t);
}

size_t sorted_bytes(int64_t n)
{
  return 256 * 12 + (2 * sizeof(uint64_t) + 6 * sizeof(uint32_t)) * (size_t)n +
         (sort_scratch_words(n) + scan_scratch_words(n) + 2) * sizeof(uint32_t);
}

// Dense pixel ids: histogram, bucket, per-pixel emit.
cudaError_t composite_dense(const Partial *in, int64_t n, int lo, int64_t r, Partial *out,
                            Arena &a, uint32_t *totals, unsigned *bad, cudaStream_t st)
{
  uint32_t *cnt = a.take<uint32_t>(r), *off = a.take<uint32_t>(r);
  uint32_t *upos = a.take<uint32_t>(r), *mpos = a.take<uint32_t>(r);
  uint2 *pr = a.take<uint2>(n);
  uint32_t *order = a.take<uint32_t>(n);
  uint32_t *scan_tmp = a.take<uint32_t>(std::max<size_t>(scan_scratch_words(r), 3 * (size_t)kTile3));
  cudaError_t e = cudaMemsetAsync(cnt, 0, sizeof(uint32_t) * r, st);
  if (e != cudaSuccess) return e;
  count_kernel<<<grid_of(n), 256, 0, st>>>(in, n, lo, r, cnt, pr, bad);
  count_launch();
  const int64_t tiles = (r + kTile3 - 1) / kTile3;
  if (tiles <= kTile3) {
    uint3 *sums = reinterpret_cast<uint3 *>(scan_tmp);   // 3 words per tile, within scan_tmp
    scan3_tile_kernel<<<(unsigned)tiles, kTile3, 0, st>>>(cnt, r, off, upos, mpos, sums);
    count_launch();
    if (tiles > 1) {
      scan3_top_kernel<<<1, kTile3, 0, st>>>(sums, (int)tiles);
      scan3_add_kernel<<<(unsigned)tiles, kTile3, 0, st>>>(r, off, upos, mpos, sums);
      count_launch(2);
    }
  } else {
    if ((e = cudaMemcpyAsync(off, cnt, sizeof(uint32_t) * r, cudaMemcpyDeviceToDevice, st)) != cudaSuccess)
      return e;
    if ((e = exclusive_scan(off, r, scan_tmp, st)) != cudaSuccess) return e;
    pixel_flag_kernel<<<grid_of(r), 256, 0, st>>>(cnt, r, upos, mpos);
    count_launch();
    if ((e = exclusive_scan(upos, r, scan_tmp, st)) != cudaSuccess) return e;
    if ((e = exclusive_scan(mpos, r, scan_tmp, st)) != cudaSuccess) return e;
  }
  bucket_kernel<<<grid_of(n), 256, 0, st>>>(pr, n, r, off, order);
  count_launch();
  pixel_emit_kernel<<<grid_of(r), 256, 0, st>>>(in, cnt, off, upos, mpos, order, r, out, totals);
  count_launch();
  return cudaGetLastError();
}

// Any pixel ids: stable radix sort by (pixel id, depth), segment scans.
cudaError_t composite_sorted(const Partial *in, int64_t n, Partial *out, Arena &a,
                             uint32_t *totals, cudaStream_t st)
{
  uint64_t *keys = a.take<uint64_t>(n), *keys_tmp = a.take<uint64_t>(n);
  uint32_t *idx = a.take<uint32_t>(n), *idx_tmp = a.take<uint32_t>(n);
  uint32_t *uniq = a.take<uint32_t>(n), *multi = a.take<uint32_t>(n);
  uint32_t *upos = a.take<uint32_t>(n), *mpos = a.take<uint32_t>(n);
  uint32_t *scratch = a.take<uint32_t>(sort_scratch_words(n));
  uint32_t *scan_tmp = a.take<uint32_t>(scan_scratch_words(n));
  key_kernel<<<grid_of(n), 256, 0, st>>>(in, n, keys, idx);
  count_launch();
  cudaError_t e = radix_sort_pairs<uint64_t>(keys, idx, keys_tmp, idx_tmp, n, 64, scratch, st);
  if (e != cudaSuccess) return e;
  flag_kernel<<<grid_of(n), 256, 0, st>>>(keys, n, uniq, multi);
  count_launch();
  if ((e = cudaMemcpyAsync(upos, uniq, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = cudaMemcpyAsync(mpos, multi, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, st)) != cudaSuccess) return e;
  if ((e = exclusive_scan(upos, n, scan_tmp, st)) != cudaSuccess) return e;
  if ((e = exclusive_scan(mpos, n, scan_tmp, st)) != cudaSuccess) return e;
  sorted_totals_kernel<<<1, 32, 0, st>>>(upos, uniq, mpos, multi, n, totals);
  count_launch();
  emit_kernel<<<grid_of(n), 256, 0, st>>>(in, keys, idx, n, upos, mpos, uniq, multi, totals, out);
  count_launch();
  return cudaGetLastError();
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
  if (n >= ((int64_t)1 << 31)) return set_error(GVR_ERR_UNSUPPORTED, "at most 2^31 - 1 partials");
  *n_out = 0;
  if (n == 0) return GVR_OK;
  cudaStream_t st = (cudaStream_t)stream;
  Partial *d_in = nullptr, *d_out = nullptr;
  unsigned *mm = nullptr;
  Arena arena;
  unsigned hm[2] = {0u, 0u};
  uint32_t ht[2] = {0u, 0u};
  uint32_t *totals = nullptr;
  cudaError_t e = cudaSuccess;
  int rc = GVR_OK;
#define CP_TRY(expr, what)                                        \
  do {                                                            \
    e = (expr);                                                   \
    if (e != cudaSuccess) { rc = cuda_error(e, what); goto done; } \
  } while (0)
  if (location == GVR_MEM_HOST) {
    CP_TRY(scratch_alloc((void **)&d_in, sizeof(Partial) * n, st), "allocate partials");
    CP_TRY(scratch_alloc((void **)&d_out, sizeof(Partial) * n, st), "allocate output");
    CP_TRY(cudaMemcpyAsync(d_in, partials, sizeof(Partial) * n, cudaMemcpyHostToDevice, st), "copy partials");
  } else {
    d_in = const_cast<Partial *>(partials);
    d_out = out;
  }
  // pixel-id range (merge computes the same, PartialCompositor.cpp:279-306)
  CP_TRY(scratch_alloc((void **)&mm, 2 * sizeof(unsigned), st), "allocate range");
  CP_TRY(cudaMemsetAsync(mm, 0xff, sizeof(unsigned), st), "range");
  CP_TRY(cudaMemsetAsync(mm + 1, 0, sizeof(unsigned), st), "range");
  range_kernel<<<grid_of(n), 256, 0, st>>>(d_in, n, mm);
  count_launch();
  CP_TRY(cudaMemcpyAsync(hm, mm, sizeof(hm), cudaMemcpyDeviceToHost, st), "read range");
  CP_TRY(cudaStreamSynchronize(st), "composite");
  {
    const int lo = (int)(hm[0] ^ 0x80000000u), hi = (int)(hm[1] ^ 0x80000000u);
    const int64_t r = (int64_t)hi - lo + 1;
    const bool dense = r <= 2 * n + 65536 && r < ((int64_t)1 << 31);
    const size_t bytes = dense ? dense_bytes(n, r) : sorted_bytes(n);
    CP_TRY(scratch_alloc((void **)&arena.base, bytes, st), "allocate scratch");
    totals = arena.take<uint32_t>(2);
    // the range was measured, so no record is outside it: mm[0] serves as
    // the (unused) flag word
    CP_TRY(dense ? composite_dense(d_in, n, lo, r, d_out, arena, totals, mm, st)
                 : composite_sorted(d_in, n, d_out, arena, totals, st),
           "composite");
    CP_TRY(cudaMemcpyAsync(ht, totals, sizeof(ht), cudaMemcpyDeviceToHost, st), "read counts");
    CP_TRY(cudaStreamSynchronize(st), "composite");
    const int64_t total = (int64_t)ht[0] + ht[1];
    if (location == GVR_MEM_HOST) {
      CP_TRY(cudaMemcpyAsync(out, d_out, sizeof(Partial) * total, cudaMemcpyDeviceToHost, st), "copy output");
      CP_TRY(cudaStreamSynchronize(st), "composite");
    }
    *n_out = total;
  }
done:
#undef CP_TRY
  if (location == GVR_MEM_HOST) {
    if (d_in) cudaFreeAsync(d_in, st);
    if (d_out) cudaFreeAsync(d_out, st);
  }
  if (mm) cudaFreeAsync(mm, st);
  if (arena.base) cudaFreeAsync(arena.base, st);
  return rc;
}

extern "C" int gvr_composite_partials_async(const gvr_partial *partials, int64_t n, int32_t pixel_lo,
                                            int32_t pixel_hi, gvr_partial *out, int64_t *n_out,
                                            void *stream)
{
  if (!n_out || n < 0 || (n > 0 && (!partials || !out)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad partial arrays");
  if (pixel_hi < pixel_lo) return set_error(GVR_ERR_INVALID_ARGUMENT, "pixel_hi < pixel_lo");
  if (n >= ((int64_t)1 << 31)) return set_error(GVR_ERR_UNSUPPORTED, "at most 2^31 - 1 partials");
  const int64_t r = (int64_t)pixel_hi - pixel_lo + 1;
  if (r > ((int64_t)1 << 30)) return set_error(GVR_ERR_UNSUPPORTED, "pixel range above 2^30");
  cudaStream_t st = (cudaStream_t)stream;
  cudaError_t e;
  if (n == 0) {
    e = cudaMemsetAsync(n_out, 0, sizeof(int64_t), st);
    return e == cudaSuccess ? GVR_OK : cuda_error(e, "composite");
  }
  Arena arena;
  e = scratch_alloc((void **)&arena.base, dense_bytes(n, r), st);
  if (e != cudaSuccess) return cuda_error(e, "allocate scratch");
  uint32_t *totals = arena.take<uint32_t>(2);
  unsigned *bad = arena.take<unsigned>(1);
  e = cudaMemsetAsync(bad, 0, sizeof(unsigned), st);
  if (e == cudaSuccess)
    e = composite_dense(reinterpret_cast<const Partial *>(partials), n, pixel_lo, r,
                        reinterpret_cast<Partial *>(out), arena, totals, bad, st);
  if (e == cudaSuccess) {
    count_out_kernel<<<1, 32, 0, st>>>(totals, bad, n_out);
    count_launch();
    e = cudaGetLastError();
  }
  cudaFreeAsync(arena.base, st);
  if (e != cudaSuccess) return cuda_error(e, "composite");
  return GVR_OK;
}
