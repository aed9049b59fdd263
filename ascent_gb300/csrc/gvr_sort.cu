// gvr_sort.cu — stable LSD radix sort of (key, index) pairs and an
// exclusive prefix sum, used by the LBVH build (Morton codes) and the
// partial compositor (pixel id, depth).
//
// Each pass sorts on 8 bits: per-block digit histograms (digit-major, so one
// exclusive scan of the whole table gives every block's start position per
// digit), then a scatter in which each block walks its chunk in order, tile
// by tile, ranking equal digits within a warp with __match_any_sync. Items
// keep their input order among equal digits, so the sort is stable and ties
// of the full key end up ordered by input position.
#include <cstdint>

#include "gvr_internal.h"

namespace gvr {
namespace {

constexpr int kSortThreads = 256;
constexpr int kItemsPerThread = 8;
constexpr int kChunk = kSortThreads * kItemsPerThread;  // items per block
constexpr int kScanTile = 1024;

template <typename K>
__global__ void __launch_bounds__(kSortThreads)
hist_kernel(const K *__restrict__ keys, int64_t n, int shift, int nblocks,
            uint32_t *__restrict__ hist)
{
  __shared__ uint32_t h[256];
  h[threadIdx.x] = 0;
  __syncthreads();
  const int64_t base = (int64_t)blockIdx.x * kChunk;
  for (int i = threadIdx.x; i < kChunk; i += kSortThreads) {
    const int64_t j = base + i;
    if (j < n) atomicAdd(&h[(unsigned)(keys[j] >> shift) & 255u], 1u);
  }
  __syncthreads();
  hist[(int64_t)threadIdx.x * nblocks + blockIdx.x] = h[threadIdx.x];
}

template <typename K>
__global__ void __launch_bounds__(kSortThreads)
scatter_kernel(const K *__restrict__ keys, const uint32_t *__restrict__ vals, int64_t n,
               int shift, int nblocks, const uint32_t *__restrict__ offsets,
               K *__restrict__ keys_out, uint32_t *__restrict__ vals_out)
{
  __shared__ uint32_t offs[256];
  __shared__ uint32_t wcnt[kSortThreads / 32][256];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  offs[threadIdx.x] = offsets[(int64_t)threadIdx.x * nblocks + blockIdx.x];
  for (int w = 0; w < kSortThreads / 32; ++w) wcnt[w][threadIdx.x] = 0;
  __syncthreads();
  const unsigned lt = (1u << lane) - 1u;
  const int64_t base = (int64_t)blockIdx.x * kChunk;
  for (int tile = 0; tile < kItemsPerThread; ++tile) {
    const int64_t j = base + (int64_t)tile * kSortThreads + threadIdx.x;
    const bool ok = j < n;
    K key = 0;
    uint32_t val = 0;
    unsigned d = 256u;  // sentinel digit for missing items
    if (ok) {
      key = keys[j];
      val = vals[j];
      d = (unsigned)(key >> shift) & 255u;
    }
    const unsigned peers = __match_any_sync(0xffffffffu, d);
    const int rank = __popc(peers & lt);
    if (ok && rank == 0) wcnt[warp][d] = __popc(peers);
    __syncthreads();
    if (ok) {
      uint32_t pre = 0;
      for (int w = 0; w < warp; ++w) pre += wcnt[w][d];
      const uint32_t pos = offs[d] + pre + (uint32_t)rank;
      keys_out[pos] = key;
      vals_out[pos] = val;
    }
    __syncthreads();
    {
      uint32_t tot = 0;
      for (int w = 0; w < kSortThreads / 32; ++w) {
        tot += wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = 0;
      }
      offs[threadIdx.x] += tot;
    }
    __syncthreads();
  }
}

// Exclusive scan of one tile of kScanTile values; tile totals to sums.
__global__ void __launch_bounds__(kScanTile)
scan_tile_kernel(uint32_t *__restrict__ data, int64_t n, uint32_t *__restrict__ sums)
{
  __shared__ uint32_t warp_tot[kScanTile / 32];
  const int64_t j = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  const uint32_t v = j < n ? data[j] : 0u;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  uint32_t x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) warp_tot[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t t = warp_tot[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
      if (lane >= o) t += y;
    }
    warp_tot[lane] = t;
  }
  __syncthreads();
  const uint32_t prefix = (warp > 0 ? warp_tot[warp - 1] : 0u) + x - v;
  if (j < n) data[j] = prefix;
  if (threadIdx.x == kScanTile - 1 && sums) sums[blockIdx.x] = warp_tot[kScanTile / 32 - 1];
}

__global__ void add_tile_kernel(uint32_t *__restrict__ data, int64_t n,
                                const uint32_t *__restrict__ sums)
{
  const int64_t j = (int64_t)blockIdx.x * kScanTile + threadIdx.x;
  if (j < n) data[j] += sums[blockIdx.x];
}

}  // namespace

size_t scan_scratch_words(int64_t n)
{
  size_t words = 0;
  while (n > kScanTile) {
    n = (n + kScanTile - 1) / kScanTile;
    words += (size_t)n;
  }
  return words + 1;
}

// In-place exclusive scan; tmp holds scan_scratch_words(n) words.
cudaError_t exclusive_scan(uint32_t *data, int64_t n, uint32_t *tmp, cudaStream_t stream)
{
  if (n <= 0) return cudaSuccess;
  const int64_t tiles = (n + kScanTile - 1) / kScanTile;
  if (tiles == 1) {
    scan_tile_kernel<<<1, kScanTile, 0, stream>>>(data, n, nullptr);
    count_launch();
    return cudaGetLastError();
  }
  scan_tile_kernel<<<(unsigned)tiles, kScanTile, 0, stream>>>(data, n, tmp);
  count_launch();
  cudaError_t e = exclusive_scan(tmp, tiles, tmp + tiles, stream);
  if (e != cudaSuccess) return e;
  add_tile_kernel<<<(unsigned)tiles, kScanTile, 0, stream>>>(data, n, tmp);
  count_launch();
  return cudaGetLastError();
}

int64_t sort_blocks(int64_t n) { return (n + kChunk - 1) / kChunk; }

size_t sort_scratch_words(int64_t n)
{
  const int64_t nb = sort_blocks(n);
  return (size_t)(256 * nb) + scan_scratch_words(256 * nb);
}

template <typename K>
cudaError_t radix_sort_pairs(K *keys, uint32_t *vals, K *keys_tmp, uint32_t *vals_tmp,
                             int64_t n, int key_bits, uint32_t *scratch, cudaStream_t stream)
{
  if (n <= 1) return cudaSuccess;
  if (n >= ((int64_t)1 << 32)) return cudaErrorInvalidValue;
  const int nb = (int)sort_blocks(n);
  uint32_t *hist = scratch;
  uint32_t *scan_tmp = scratch + (size_t)256 * nb;
  K *src_k = keys, *dst_k = keys_tmp;
  uint32_t *src_v = vals, *dst_v = vals_tmp;
  const int passes = (key_bits + 7) / 8;
  for (int p = 0; p < passes; ++p) {
    const int shift = 8 * p;
    hist_kernel<K><<<nb, kSortThreads, 0, stream>>>(src_k, n, shift, nb, hist);
    count_launch();
    cudaError_t e = exclusive_scan(hist, (int64_t)256 * nb, scan_tmp, stream);
    if (e != cudaSuccess) return e;
    scatter_kernel<K><<<nb, kSortThreads, 0, stream>>>(src_k, src_v, n, shift, nb, hist, dst_k,
                                                       dst_v);
    count_launch();
    e = cudaGetLastError();
    if (e != cudaSuccess) return e;
    K *tk = src_k; src_k = dst_k; dst_k = tk;
    uint32_t *tv = src_v; src_v = dst_v; dst_v = tv;
  }
  if (src_k != keys) {
    cudaError_t e = cudaMemcpyAsync(keys, src_k, sizeof(K) * n, cudaMemcpyDeviceToDevice, stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(vals, src_v, sizeof(uint32_t) * n, cudaMemcpyDeviceToDevice, stream);
    return e;
  }
  return cudaSuccess;
}

template cudaError_t radix_sort_pairs<uint32_t>(uint32_t *, uint32_t *, uint32_t *, uint32_t *,
                                                int64_t, int, uint32_t *, cudaStream_t);
template cudaError_t radix_sort_pairs<uint64_t>(uint64_t *, uint32_t *, uint64_t *, uint32_t *,
                                                int64_t, int, uint32_t *, cudaStream_t);

}  // namespace gvr
