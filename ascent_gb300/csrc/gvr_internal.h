// gvr_internal.h — types shared by the host library and the CUDA kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <map>
#include <string>
#include <vector>

#include "../../include/gvr.h"

namespace gvr {

// Bricked field layout: a brick covers 8^3 cells and stores the 9^3 nodes
// that bound them (one-node apron shared with the next brick), so every
// cell's eight corners sit in one brick at fixed offsets. Bricks are padded
// to 736 floats (2944 B, 23 x 128 B lines) so that each starts on a
// 128-byte boundary.
constexpr int kBrickCells = 8;
constexpr int kBrickNodes = kBrickCells + 1;
constexpr int kBrickFloats = 736;
static_assert(kBrickNodes * kBrickNodes * kBrickNodes <= kBrickFloats, "brick");

// A scene may brick its fields with 4^3, 8^3 (the default above) or 16^3
// cells per brick (gvr_scene_set_brick_cells; the autotuner picks one). A
// brick of 2^shift cells per axis stores (2^shift + 1)^3 nodes, padded to a
// multiple of 32 floats (128 bytes): 128, 736 or 4928 floats.
constexpr int kBrickShiftMin = 2, kBrickShiftMax = 4, kBrickShiftDefault = 3;
__host__ __device__ constexpr int brick_cells(int shift) { return 1 << shift; }
__host__ __device__ constexpr int brick_nodes(int shift) { return (1 << shift) + 1; }
__host__ __device__ constexpr int brick_floats(int shift)
{
  return (brick_nodes(shift) * brick_nodes(shift) * brick_nodes(shift) + 31) / 32 * 32;
}
static_assert(brick_floats(kBrickShiftDefault) == kBrickFloats, "default brick");

constexpr int kMaxDomains = 64;     // domains a single render can composite
constexpr int kMaxLut = 4096;
constexpr int kMarchTile = 16;      // march kernel: one CTA per 16x16-pixel tile

// Device view of one structured domain.
struct DomainDev {
  float lo[3];            // bounds
  float hi[3];
  float origin[3];        // uniform: node 0 position
  float inv_spacing[3];   // uniform: 1 / spacing
  int dims[3];            // node counts
  int nbrick[3];          // bricks per axis
  int kind;               // GVR_DOMAIN_UNIFORM / RECTILINEAR
  int assoc;              // GVR_ASSOC_VERTEX / ELEMENT
  const float *bricks;    // vertex fields: bricked nodes
  const float *cells;     // element fields: linear cell values
  const float *coord[3];  // rectilinear node coordinates
  const float2 *brick_range;  // per-brick {min, max} of the field
  const uint8_t *brick_empty; // per-brick 1 = LUT alpha is 0 over its range
  const int *any_empty;       // 1 if any brick of this domain is empty
  // hexahedral domains
  const float4 *hex_nodes;    // x, y, z, vertex field value
  const int4 *hex_conn;       // 8 node ids per cell (VTK hex order), 2 int4
  const float4 *hex_coef;     // 8 per cell: monomial coefficients of the trilinear map (xyz, field)
  const float4 *hex_bvh;      // 4 float4 per inner node (see gvr_hex.cu)
  const int *hex_ids;         // cell id of each sorted leaf
  const int *hex_nbr;         // 6 face neighbours per cell (r=0,r=1,s=0,s=1,t=0,t=1), -1 none
  int n_cells;
  int bshift;                 // vertex fields: 2^bshift cells per brick axis
};

// Launch shape of the march kernel (picked by the autotuner): pixel packet
// width per warp (4, 8 or 16; height 32 / width), samples located per loop
// iteration (1 or 2) and the CTAs per SM the register budget targets (3, 4).
struct Tuning {
  int packet_w = 8;
  int unroll = 2;
  int min_blocks = 4;
  int tiles_per_item = 1;   // batch path: 16x16 tiles per work-queue item
  int staged = 0;           // plain path: stage bricks in shared memory (uniform vertex scenes)
  int tile_order = 0;       // plain path: 0 = tiles nearest the image centre first,
                            // 1 = longest-first by the view's estimated tile cost
};

// Front-to-back order of a scene's domains for one view (staged march).
struct StageOrder {
  int n;
  unsigned char d[kMaxDomains];
};

// Everything the march kernel needs for one view.
struct ViewDev {
  float origin[3];        // camera position
  float look[3];          // unit view direction
  float ru[3];            // unit right
  float rv[3];            // unit up (orthogonalised)
  float dx_scale;         // world step per pixel along ru
  float dy_scale;         // world step per pixel along rv
  float xoff;             // pan, in pixels
  float yoff;
  float projview[16];     // row-major projection * view (image depth)
  double inv_projview[16]; // its inverse (opaque canvas depth -> distance)
};

struct MarchParams {
  int width;
  int height;
  int n_domains;
  int lut_size;
  int lut_filter;
  int quantize_uint8;
  int render_bg;
  int skip_empty;
  float sample_dist;
  float scalar_min;
  float inv_range;
  float alpha_cull;
  float early_term;
  float clear_depth;
  float bg[4];
  // opaque canvas the volume is drawn over (both NULL: a cleared canvas);
  // rays stop at its depth and partials blend over its colour
  const float4 *canvas_rgba = nullptr;
  const float *canvas_depth = nullptr;
};

// Reusable device buffers of one domain's field uploads: the staging copy
// of a host field and the per-CTA ranges of the element-field reduction.
struct Staging {
  void *buf = nullptr;
  size_t bytes = 0;
  float2 *block_range = nullptr;
};

// Host-side record of a domain owned by a scene.
struct Domain {
  DomainDev dev;
  double bounds[6];
  double range[2];
  size_t n_values = 0;             // field values
  float *d_bricks = nullptr;
  float *d_cells = nullptr;
  float *d_coord[3] = {nullptr, nullptr, nullptr};
  float2 *d_brick_range = nullptr;
  uint8_t *d_brick_empty = nullptr;
  int64_t n_bricks = 0;
  Staging stg;
  // hexahedral domains (device)
  int64_t n_nodes = 0;
  int64_t n_cells = 0;
  float4 *d_nodes = nullptr;
  int4 *d_conn = nullptr;
  float4 *d_coef = nullptr;         // 8 per cell (see hex_coef)
  float4 *d_bvh = nullptr;
  uint32_t *d_codes = nullptr;      // sorted Morton codes
  uint32_t *d_ids = nullptr;        // sorted leaf -> cell id
  int32_t *d_left = nullptr;        // Karras topology (n_cells - 1 inner nodes)
  int32_t *d_right = nullptr;
  int32_t *d_parent = nullptr;      // 2 n_cells - 1 entries, root's is -1
  float4 *d_inner_box = nullptr;    // 2 per inner node: lo, hi
  int *d_nbr = nullptr;             // 6 face neighbours per cell
  float bvh_build_ms = 0.f;
  float nbr_build_ms = 0.f;
};

}  // namespace gvr

struct gvr_scene {
  int device = 0;
  int brick_shift = gvr::kBrickShiftDefault;  // bricks of vertex fields added from now on
  std::vector<gvr::Domain> domains;
  gvr::DomainDev *d_domains = nullptr;   // device copy of the domain table
  int d_domains_cap = 0;
  float4 *d_lut = nullptr;               // LUT of the last render
  int *d_any_empty = nullptr;            // per-domain empty-brick flags
  bool has_hex = false;
  gvr::Tuning tuning;
  unsigned long long *d_counters = nullptr;  // [0] samples, [1] staged waits given up
  float4 *d_rgba_tmp = nullptr;          // device image for host outputs
  float *d_depth_tmp = nullptr;
  int64_t tmp_pixels = 0;
  bool table_dirty = true;
  // empty-brick classification of the last render, reused while the LUT,
  // its filter and the scalar range stay the same and no field changed
  bool classify_valid = false;
  std::vector<float> classify_lut;
  float classify_smin = 0.f, classify_inv_range = 0.f;
  int classify_filter = -1;
  // batched renders: per-view constants, per-(view, domain) screen rects,
  // the work-queue counter, and the captured graph of the last batch shape
  gvr::ViewDev *d_views = nullptr;
  int views_cap = 0;
  int4 *d_rects = nullptr;
  int rects_cap = 0;
  unsigned int *d_queue = nullptr;
  float4 *d_batch_rgba = nullptr;
  float *d_batch_depth = nullptr;
  int64_t batch_pixels = 0;
  cudaStream_t own_stream = nullptr;
  // batched field uploads: staging buffers (up to one per domain, at most
  // kStageMax, within ~1 GB) filled on a copy stream while earlier fields
  // are bricked, per-domain ranges on the device
  static constexpr int kStageMax = 8;
  void *stage[kStageMax] = {};
  int stage_count = 0;
  size_t stage_bytes = 0;
  cudaStream_t copy_stream = nullptr;
  cudaEvent_t copied[kStageMax] = {};
  cudaEvent_t consumed[kStageMax] = {};
  // per-domain ranges of a batched upload, then one int: the staged
  // kernel's timeout flag; read back in one copy into pinned h_ranges
  float2 *d_ranges = nullptr;
  float2 *h_ranges = nullptr;
  int ranges_cap = 0;
  int *d_flag = nullptr;  // timeout flag of single-field uploads
  cudaGraphExec_t batch_exec = nullptr;
  std::vector<unsigned char> batch_key;
  int batch_graph_builds = 0;
  // launch order of the march kernel's tiles per tile grid (linear tile
  // indices, nearest the image centre first); written once, then read only
  std::map<std::pair<int, int>, int *> tile_orders;
  // per-view longest-first tile order (tile_order 1), rewritten by every
  // render that uses it: the order (cap ints), the tile costs (cap words)
  // and the costs' maximum (one word, 0 between renders)
  int *d_cost_order = nullptr;
  int64_t cost_order_cap = 0;
};

namespace gvr {

// error plumbing (gvr_api.cpp)
int set_error(int code, const std::string &msg);
int cuda_error(cudaError_t e, const char *what);

// camera -> per-view constants (gvr_api.cpp)
void make_view(const gvr_camera &cam, int width, int height, ViewDev *v);

// stream-ordered scratch from this library's memory pool on the current
// device (kept between calls, unlike the default pool's); free it with
// cudaFreeAsync
cudaError_t scratch_alloc(void **ptr, size_t bytes, cudaStream_t stream);

// kernels launched by this library since it was loaded
void count_launch(int n = 1);
uint64_t launch_count();

// ingest kernels (gvr_ingest.cu)
// Brick a vertex field and read its range back (synchronises `stream`).
// *d_timed_out is a device int the staged kernel sets when a bulk copy did
// not complete within its bounded wait; *timed_out receives it.
cudaError_t launch_brick_field(const void *src, int dtype, int64_t stride,
                               int src_on_device, const int dims[3], int bshift,
                               float *d_bricks, const int nbrick[3],
                               float2 *d_brick_range, double range_out[2],
                               Staging &stg, int *d_timed_out, bool *timed_out,
                               cudaStream_t stream);
// Brick a vertex field that is already in device memory, with per-brick
// ranges (no host synchronisation); a staged copy that gives up waiting
// sets *d_timed_out.
cudaError_t launch_brick_device(const void *dsrc, int dtype, int64_t stride, const int dims[3],
                                int bshift, float *d_bricks, const int nbrick[3],
                                float2 *d_brick_range, int *d_timed_out, cudaStream_t stream);
// Brick n contiguous float32 fields in device memory into 8^3-cell bricks in
// one launch (the staged kernel's runs of all fields), with per-brick
// ranges; a staged copy that gives up waiting sets *d_timed_out.
cudaError_t launch_brick_device_many(int n, const float *const *srcs, const int (*dims)[3],
                                     float *const *bricks, const int (*nbrick)[3],
                                     float2 *const *brick_range, int *d_timed_out, cudaStream_t stream);
// Reduce n domains' per-brick ranges to one range each (*out[j]; NaN when a
// brick holds a non-finite value): one launch, one block per domain.
cudaError_t launch_ranges_of_bricks(int n, const float2 *const *brick_ranges,
                                    const int64_t *n_bricks, float2 *const *out,
                                    cudaStream_t stream);
cudaError_t launch_cells_field(const void *src, int dtype, int64_t stride,
                               int src_on_device, int64_t n, float *d_cells,
                               double range_out[2], Staging &stg,
                               cudaStream_t stream);
cudaError_t launch_empty_bricks(const float2 *brick_range, int64_t n_bricks,
                                const float4 *d_lut, int lut_size, int lut_filter,
                                float scalar_min, float inv_range,
                                uint8_t *brick_empty, int *any_empty,
                                cudaStream_t stream);

// sort / scan (gvr_sort.cu)
size_t scan_scratch_words(int64_t n);
cudaError_t exclusive_scan(uint32_t *data, int64_t n, uint32_t *tmp, cudaStream_t stream);
size_t sort_scratch_words(int64_t n);
template <typename K>
cudaError_t radix_sort_pairs(K *keys, uint32_t *vals, K *keys_tmp, uint32_t *vals_tmp,
                             int64_t n, int key_bits, uint32_t *scratch, cudaStream_t stream);

// hexahedral domains (gvr_hex.cu)
void free_hex(Domain &d);
int hex_update_field(Domain &d, const void *field, int dtype, int64_t stride, int location);

// march kernel (gvr_march.cu); CTA i renders tile d_order[i] (a linear
// tile index, row-major over the kMarchTile grid), or tile i when d_order is
// NULL
cudaError_t launch_march(const DomainDev *d_domains, const ViewDev &view,
                         const MarchParams &mp, const float4 *d_lut,
                         float4 *d_rgba, float *d_depth,
                         unsigned long long *d_samples, const Tuning &tuning,
                         bool has_hex, const int *d_order, cudaStream_t stream);
// longest-first tile order for one view (gvr_march.cu): writes a permutation
// of the view's kMarchTile tiles to d_order (one int per tile); d_keys holds
// one word per tile of scratch and *d_top a word that is 0 between calls;
// grids of more than kCostOrderTiles tiles are refused (cudaErrorInvalidValue)
constexpr int kCostOrderTiles = 48 * 1024;
cudaError_t launch_tile_cost_order(const DomainDev *d_domains, const ViewDev &view, const MarchParams &mp,
                                   int *d_order, unsigned *d_keys, unsigned *d_top, cudaStream_t stream);
// staged march (gvr_march.cu): uniform vertex-field domains only, taken in
// `order`; *d_stage_fail counts CTAs whose bounded wait for their bulk
// copies gave up (they finish from global memory)
cudaError_t launch_staged(const DomainDev *d_domains, const ViewDev &view, const MarchParams &mp,
                          const float4 *d_lut, float4 *d_rgba, float *d_depth,
                          unsigned long long *d_samples, const Tuning &tuning, const int *d_order,
                          const StageOrder &order, unsigned long long *d_stage_fail,
                          cudaStream_t stream);
cudaError_t batch_grid(const MarchParams &mp, int n_views, const Tuning &tuning, bool has_hex,
                       int *grid);
cudaError_t launch_batch(const DomainDev *d_domains, const ViewDev *d_views, const int4 *d_rects,
                         const MarchParams &mp, int n_views, const float4 *d_lut, float4 *d_rgba,
                         float *d_depth, unsigned long long *d_samples, unsigned int *d_queue,
                         const Tuning &tuning, bool has_hex, int grid, cudaStream_t stream);

}  // namespace gvr
