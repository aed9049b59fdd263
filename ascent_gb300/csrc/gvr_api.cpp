// gvr_api.cpp — host side of the C ABI declared in include/gvr.h.
//
// This is the part of vtkh::VolumeRenderer / vtkh::Renderer / Ascent's
// rendering filters that runs on the host (opacity correction, sample
// distance, transfer-function sampling, cameras, visibility order, domain
// bookkeeping) plus the orchestration of the device kernels.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include "gvr_internal.h"

namespace {
thread_local std::string g_last_error;
std::atomic<uint64_t> g_launches{0};
constexpr double kPi = 3.14159265358979323846;
}  // namespace

namespace gvr {

int set_error(int code, const std::string &msg)
{
  g_last_error = msg;
  return code;
}

void count_launch(int n) { g_launches.fetch_add((uint64_t)n, std::memory_order_relaxed); }

uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }

int cuda_error(cudaError_t e, const char *what)
{
  const int code = e == cudaErrorMemoryAllocation ? GVR_ERR_OUT_OF_MEMORY : GVR_ERR_CUDA;
  return set_error(code, std::string(what) + ": " + cudaGetErrorString(e));
}

namespace {
constexpr int kMaxPoolDevices = 64;
std::mutex g_pool_mu;
cudaMemPool_t g_pools[kMaxPoolDevices] = {};
}  // namespace

// The device's default memory pool gives its free memory back to the
// system at every synchronisation (release threshold 0), so a call that
// allocates tens of MB of scratch and synchronises would map fresh pages
// every time. This library's own pool keeps what it has allocated (up to
// its high-water mark, held until the process exits) and leaves the
// default pool, which other libraries in the process may use, as it is.
cudaError_t scratch_alloc(void **ptr, size_t bytes, cudaStream_t stream)
{
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) return e;
  if (device < 0 || device >= kMaxPoolDevices) return cudaMallocAsync(ptr, bytes, stream);
  cudaMemPool_t pool;
  {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    if (!g_pools[device]) {
      cudaMemPoolProps props{};
      props.allocType = cudaMemAllocationTypePinned;
      props.location.type = cudaMemLocationTypeDevice;
      props.location.id = device;
      cudaMemPool_t created = nullptr;
      if ((e = cudaMemPoolCreate(&created, &props)) != cudaSuccess) return e;
      uint64_t keep = UINT64_MAX;
      if ((e = cudaMemPoolSetAttribute(created, cudaMemPoolAttrReleaseThreshold, &keep)) !=
          cudaSuccess) {
        cudaMemPoolDestroy(created);
        return e;
      }
      g_pools[device] = created;
    }
    pool = g_pools[device];
  }
  return cudaMallocFromPoolAsync(ptr, bytes, pool, stream);
}

}  // namespace gvr

int gvr_scratch_trim(int device, uint64_t keep_bytes, uint64_t *reserved_out)
{
  using namespace gvr;
  if (device < 0) return set_error(GVR_ERR_INVALID_ARGUMENT, "negative device");
  cudaMemPool_t pool = nullptr;
  if (device < kMaxPoolDevices) {
    std::lock_guard<std::mutex> lock(g_pool_mu);
    pool = g_pools[device];
  }
  uint64_t reserved = 0;
  if (pool) {
    // blocks still in use are kept whatever keep_bytes says; memory freed
    // on a stream is returned once that free has completed
    cudaError_t e = cudaMemPoolTrimTo(pool, (size_t)keep_bytes);
    if (e != cudaSuccess) return cuda_error(e, "cudaMemPoolTrimTo");
    e = cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &reserved);
    if (e != cudaSuccess) return cuda_error(e, "cudaMemPoolGetAttribute");
  }
  if (reserved_out) *reserved_out = reserved;
  return GVR_OK;
}

namespace gvr {
namespace {

struct V3 {
  double x, y, z;
};
V3 v3(const float *p) { return {p[0], p[1], p[2]}; }
V3 operator-(V3 a, V3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
V3 operator+(V3 a, V3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
V3 operator*(V3 a, double s) { return {a.x * s, a.y * s, a.z * s}; }
double dot(V3 a, V3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
V3 cross(V3 a, V3 b) { return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x}; }
V3 unit(V3 a)
{
  const double m = std::sqrt(dot(a, a));
  return m > 0 ? a * (1.0 / m) : a;
}
V3 rotate(V3 v, V3 k, double deg)
{
  const double th = deg * kPi / 180.0, c = std::cos(th), s = std::sin(th);
  return v * c + cross(k, v) * s + k * (dot(k, v) * (1 - c));
}

bool finite3(const float *p) { return std::isfinite(p[0]) && std::isfinite(p[1]) && std::isfinite(p[2]); }

int check_camera(const gvr_camera *c)
{
  if (!c) return set_error(GVR_ERR_INVALID_ARGUMENT, "camera is NULL");
  if (!finite3(c->position) || !finite3(c->look_at) || !finite3(c->up))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "camera has non-finite vectors");
  V3 d = v3(c->look_at) - v3(c->position);
  if (dot(d, d) == 0) return set_error(GVR_ERR_INVALID_ARGUMENT, "camera position equals look_at");
  if (!(c->fov_y > 0 && c->fov_y < 180))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "camera fov_y must be in (0, 180)");
  V3 r = cross(d, v3(c->up));
  if (dot(r, r) == 0) return set_error(GVR_ERR_INVALID_ARGUMENT, "camera up is parallel to the view direction");
  return GVR_OK;
}

double piecewise(int n, const double *pos, const double *val, int stride, int c, double x,
                 double dflt)
{
  if (n <= 0) return dflt;
  if (x <= pos[0]) return val[c];
  if (x >= pos[n - 1]) return val[(size_t)(n - 1) * stride + c];
  const double *it = std::upper_bound(pos, pos + n, x);
  const int hi = (int)(it - pos), lo = hi - 1;
  const double w = (x - pos[lo]) / (pos[hi] - pos[lo]);
  return val[(size_t)lo * stride + c] * (1 - w) + val[(size_t)hi * stride + c] * w;
}

// Inverse of a row-major 4x4 matrix by Gauss-Jordan elimination with
// partial pivoting (identity when singular).
void invert4(const double *m, double *inv)
{
  double a[4][8];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 8; ++j) a[i][j] = j < 4 ? m[i * 4 + j] : (j - 4 == i ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (std::fabs(a[r][c]) > std::fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) {
      for (int i = 0; i < 16; ++i) inv[i] = (i % 5) == 0 ? 1.0 : 0.0;
      return;
    }
    if (piv != c)
      for (int j = 0; j < 8; ++j) std::swap(a[c][j], a[piv][j]);
    const double d = 1.0 / a[c][c];
    for (int j = 0; j < 8; ++j) a[c][j] *= d;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      const double f = a[r][c];
      for (int j = 0; j < 8; ++j) a[r][j] -= f * a[c][j];
    }
  }
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) inv[i * 4 + j] = a[i][j + 4];
}

}  // namespace

// Per-view constants of the pinhole model the reference's partials_to_canvas
// inverts (VolumeRenderer.cpp:303-335): look, ru = look x up, rv = ru x look,
// per-pixel steps 2 tan(fov/2) / size divided by zoom; fov_x is derived from
// fov_y through the aspect ratio when the image is not square.
void make_view(const gvr_camera &cam, int width, int height, ViewDev *v)
{
  const V3 origin = v3(cam.position);
  const V3 look = unit(v3(cam.look_at) - origin);
  const V3 ru = unit(cross(look, v3(cam.up)));
  const V3 rv = unit(cross(ru, look));
  const float fov_y = cam.fov_y;
  float fov_x = fov_y;
  if (width != height) {
    const float fovy_rad = fov_y * (float)(kPi / 180.0);
    const float vd = std::tan(0.5f * fovy_rad);
    const float hd = ((float)width / (float)height) * vd;
    fov_x = 2.0f * std::atan(hd) / (float)(kPi / 180.0);
  }
  const float thx = std::tan((fov_x * (float)(kPi / 180.0)) * 0.5f);
  const float thy = std::tan((fov_y * (float)(kPi / 180.0)) * 0.5f);
  float dxs = 2 * thx / (float)width, dys = 2 * thy / (float)height;
  if (cam.zoom > 0) {
    dxs /= cam.zoom;
    dys /= cam.zoom;
  }
  const double o[3] = {origin.x, origin.y, origin.z};
  const double l[3] = {look.x, look.y, look.z};
  const double r[3] = {ru.x, ru.y, ru.z};
  const double u[3] = {rv.x, rv.y, rv.z};
  for (int a = 0; a < 3; ++a) {
    v->origin[a] = (float)o[a];
    v->look[a] = (float)l[a];
    v->ru[a] = (float)r[a];
    v->rv[a] = (float)u[a];
  }
  v->dx_scale = dxs;
  v->dy_scale = dys;
  v->xoff = cam.xpan * (float)width * 0.5f;
  v->yoff = cam.ypan * (float)height * 0.5f;
  // projection * view (standard perspective look-at camera)
  const V3 f = look;
  const V3 s = unit(cross(f, v3(cam.up)));
  const V3 uu = cross(s, f);
  const double V[4][4] = {{s.x, s.y, s.z, -dot(s, origin)},
                          {uu.x, uu.y, uu.z, -dot(uu, origin)},
                          {-f.x, -f.y, -f.z, dot(f, origin)},
                          {0, 0, 0, 1}};
  const double n = cam.near_plane, fa = cam.far_plane;
  const double aspect = (double)width / (double)height;
  const double ff = 1.0 / std::tan(0.5 * (double)cam.fov_y * kPi / 180.0);
  const double z = cam.zoom > 0 ? (double)cam.zoom : 1.0;
  const double P[4][4] = {{ff / aspect * z, 0, 0, 0},
                          {0, ff * z, 0, 0},
                          {0, 0, (fa + n) / (n - fa), 2 * fa * n / (n - fa)},
                          {0, 0, -1, 0}};
  double M[16];
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) {
      double acc = 0;
      for (int k = 0; k < 4; ++k) acc += P[i][k] * V[k][j];
      M[i * 4 + j] = acc;
      v->projview[i * 4 + j] = (float)acc;
    }
  invert4(M, v->inv_projview);
}

}  // namespace gvr

using namespace gvr;

extern "C" {

const char *gvr_last_error(void) { return g_last_error.c_str(); }

int gvr_launch_count(uint64_t *n)
{
  if (!n) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = launch_count();
  return GVR_OK;
}

int gvr_version(void) { return GVR_VERSION; }

int gvr_correct_opacity(const double *alpha_in, int n, int num_samples, double *alpha_out)
{
  if (num_samples < 1)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "Volume rendering samples must be greater than 0");
  if (n < 0 || (n > 0 && (!alpha_in || !alpha_out)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad alpha arrays");
  const float ratio = 10.f / (float)num_samples;
  for (int i = 0; i < n; ++i) alpha_out[i] = 1. - std::pow(1. - alpha_in[i], (double)ratio);
  return GVR_OK;
}

int gvr_sample_distance(const double bounds[6], int num_samples, float *sample_dist)
{
  if (!bounds || !sample_dist) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (num_samples < 1)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "Volume rendering samples must be greater than 0");
  const float e[3] = {(float)(bounds[1] - bounds[0]), (float)(bounds[3] - bounds[2]),
                      (float)(bounds[5] - bounds[4])};
  const float mag = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
  *sample_dist = mag / (float)num_samples;
  return GVR_OK;
}

int gvr_color_table_sample(const gvr_color_table *t, int n, int uint8_mode, float *out)
{
  if (!t || !out || n < 2) return set_error(GVR_ERR_INVALID_ARGUMENT, "bad colour table arguments");
  if (uint8_mode < GVR_UINT8_NONE || uint8_mode > GVR_UINT8_TRUNCATE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad uint8 mode");
  for (int i = 1; i < t->n_rgb; ++i)
    if (!(t->rgb_pos[i] > t->rgb_pos[i - 1]))
      return set_error(GVR_ERR_INVALID_ARGUMENT, "rgb control points must be strictly increasing");
  for (int i = 1; i < t->n_alpha; ++i)
    if (!(t->alpha_pos[i] > t->alpha_pos[i - 1]))
      return set_error(GVR_ERR_INVALID_ARGUMENT, "alpha control points must be strictly increasing");
  for (int i = 0; i < n; ++i) {
    const double x = (double)i / (double)(n - 1);
    double c[4];
    for (int k = 0; k < 3; ++k) c[k] = piecewise(t->n_rgb, t->rgb_pos, t->rgb, 3, k, x, 0.0);
    c[3] = piecewise(t->n_alpha, t->alpha_pos, t->alpha, 1, 0, x, 1.0);
    for (int k = 0; k < 4; ++k) {
      double v = std::min(1.0, std::max(0.0, c[k]));
      if (uint8_mode == GVR_UINT8_NONE) {
        out[i * 4 + k] = (float)c[k];
      } else {
        const double s = v * 255.0;
        unsigned u = uint8_mode == GVR_UINT8_TRUNCATE ? (unsigned)s : (unsigned)(s + 0.5);
        out[i * 4 + k] = (float)std::min(u, 255u) * (1.0f / 255.0f);
      }
    }
  }
  return GVR_OK;
}

int gvr_camera_reset_to_bounds(gvr_camera *c, const double b[6])
{
  if (!c || !b) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  const double cx = 0.5 * (b[0] + b[1]), cy = 0.5 * (b[2] + b[3]), cz = 0.5 * (b[4] + b[5]);
  const double ex = b[1] - b[0], ey = b[3] - b[2], ez = b[5] - b[4];
  double diag = std::sqrt(ex * ex + ey * ey + ez * ez);
  if (!(diag > 0)) diag = 1.0;
  const double fov = 30.0;
  const double dist = 0.5 * diag / std::tan(0.5 * fov * kPi / 180.0);
  c->look_at[0] = (float)cx; c->look_at[1] = (float)cy; c->look_at[2] = (float)cz;
  c->position[0] = (float)cx; c->position[1] = (float)cy; c->position[2] = (float)(cz + dist);
  c->up[0] = 0.f; c->up[1] = 1.f; c->up[2] = 0.f;
  c->fov_y = (float)fov;
  c->zoom = 1.f;
  c->xpan = 0.f;
  c->ypan = 0.f;
  c->near_plane = (float)(0.01 * diag);
  c->far_plane = (float)(100.0 * diag);
  return GVR_OK;
}

int gvr_camera_azimuth(gvr_camera *c, double deg)
{
  if (!c) return set_error(GVR_ERR_INVALID_ARGUMENT, "camera is NULL");
  const V3 k = unit(v3(c->up));
  const V3 at = v3(c->look_at);
  const V3 p = at + rotate(v3(c->position) - at, k, deg);
  c->position[0] = (float)p.x; c->position[1] = (float)p.y; c->position[2] = (float)p.z;
  return GVR_OK;
}

int gvr_camera_elevation(gvr_camera *c, double deg)
{
  if (!c) return set_error(GVR_ERR_INVALID_ARGUMENT, "camera is NULL");
  const V3 at = v3(c->look_at);
  const V3 off = v3(c->position) - at;
  const V3 k = unit(cross(off, v3(c->up)));
  const V3 p = at + rotate(off, k, deg);
  c->position[0] = (float)p.x; c->position[1] = (float)p.y; c->position[2] = (float)p.z;
  return GVR_OK;
}

int gvr_cinema_cameras(const double b[6], const float *pt, int n, gvr_camera *out)
{
  if (!b || (n > 0 && (!pt || !out)) || n < 0)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad cinema arguments");
  const float center[3] = {(float)(0.5 * (b[0] + b[1])), (float)(0.5 * (b[2] + b[3])),
                           (float)(0.5 * (b[4] + b[5]))};
  const float ext[3] = {(float)(b[1] - b[0]), (float)(b[3] - b[2]), (float)(b[5] - b[4])};
  const float radius = std::sqrt(ext[0] * ext[0] + ext[1] * ext[1] + ext[2] * ext[2]) * 2.5f / 2.0f;
  for (int a = 0; a < n; ++a) {
    gvr_camera c;
    gvr_camera_reset_to_bounds(&c, b);
    const float phi = pt[2 * a] * (float)(kPi / 180.0);
    const float th = pt[2 * a + 1] * (float)(kPi / 180.0);
    const float cp = std::cos(phi), sp = std::sin(phi), ct = std::cos(th), st = std::sin(th);
    // columns 1 (image of up = +y) and 2 (image of +z) of Rz(phi) Rx(theta)
    const float up[3] = {-sp * ct, cp * ct, st};
    const float pos[3] = {sp * st, -cp * st, ct};
    const float um = std::sqrt(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
    for (int i = 0; i < 3; ++i) {
      c.up[i] = up[i] / um;
      c.position[i] = pos[i] * radius + center[i];
      c.look_at[i] = center[i];
    }
    out[a] = c;
  }
  return GVR_OK;
}

int gvr_visibility_order(const gvr_camera *c, const double *bounds, int n, int *order)
{
  if (!c || n < 0 || (n > 0 && (!bounds || !order)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad visibility-order arguments");
  std::vector<float> dist(n);
  for (int d = 0; d < n; ++d) {
    const double *bb = bounds + 6 * d;
    const float dx = (float)(0.5 * (bb[0] + bb[1])) - c->position[0];
    const float dy = (float)(0.5 * (bb[2] + bb[3])) - c->position[1];
    const float dz = (float)(0.5 * (bb[4] + bb[5])) - c->position[2];
    dist[d] = std::sqrt(dx * dx + dy * dy + dz * dz);
  }
  std::vector<int> idx(n);
  for (int d = 0; d < n; ++d) idx[d] = d;
  std::stable_sort(idx.begin(), idx.end(), [&](int a, int b2) { return dist[a] < dist[b2]; });
  for (int r = 0; r < n; ++r) order[idx[r]] = r;
  return GVR_OK;
}

// ---------------------------------------------------------------------------
// Scene
// ---------------------------------------------------------------------------

int gvr_scene_create(int device, gvr_scene **out)
{
  if (!out) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene_out is NULL");
  *out = nullptr;
  int count = 0;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return cuda_error(e, "cudaGetDeviceCount");
  if (device < 0 || device >= count)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "device " + std::to_string(device) + " does not exist");
  gvr_scene *s = new gvr_scene();
  s->device = device;
  *out = s;
  return GVR_OK;
}

static void free_domain(Domain &d)
{
  cudaFree(d.d_bricks);
  cudaFree(d.d_cells);
  for (int a = 0; a < 3; ++a) cudaFree(d.d_coord[a]);
  cudaFree(d.d_brick_range);
  cudaFree(d.d_brick_empty);
  cudaFree(d.stg.buf);
  cudaFree(d.stg.block_range);
  free_hex(d);
  d = Domain();
}

int gvr_scene_destroy(gvr_scene *s)
{
  if (!s) return GVR_OK;
  cudaSetDevice(s->device);
  for (Domain &d : s->domains) free_domain(d);
  cudaFree(s->d_domains);
  cudaFree(s->d_lut);
  cudaFree(s->d_any_empty);
  cudaFree(s->d_counters);
  cudaFree(s->d_rgba_tmp);
  cudaFree(s->d_depth_tmp);
  cudaFree(s->d_views);
  cudaFree(s->d_rects);
  cudaFree(s->d_queue);
  for (auto &t : s->tile_orders) cudaFree(t.second);
  cudaFree(s->d_cost_order);
  cudaFree(s->d_batch_rgba);
  cudaFree(s->d_batch_depth);
  if (s->batch_exec) cudaGraphExecDestroy(s->batch_exec);
  if (s->own_stream) cudaStreamDestroy(s->own_stream);
  if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
  for (int b = 0; b < gvr_scene::kStageMax; ++b) {
    cudaFree(s->stage[b]);
    if (s->copied[b]) cudaEventDestroy(s->copied[b]);
    if (s->consumed[b]) cudaEventDestroy(s->consumed[b]);
  }
  cudaFree(s->d_ranges);
  cudaFreeHost(s->h_ranges);
  cudaFree(s->d_flag);
  delete s;
  return GVR_OK;
}

static int upload_field(gvr_scene *s, Domain &d, const void *field, int dtype, int64_t stride,
                        int location)
{
  if (!field) return set_error(GVR_ERR_INVALID_ARGUMENT, "field is NULL");
  if (dtype != GVR_DTYPE_FLOAT32 && dtype != GVR_DTYPE_FLOAT64)
    return set_error(GVR_ERR_UNSUPPORTED, "field dtype must be float32 or float64");
  if (stride < 1) return set_error(GVR_ERR_INVALID_ARGUMENT, "field stride must be >= 1");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad field location");
  cudaError_t e;
  if (d.dev.kind == GVR_DOMAIN_HEX) {
    const int rc = hex_update_field(d, field, dtype, stride, location);
    if (rc != GVR_OK) return rc;
    s->table_dirty = true;
    s->classify_valid = false;
    return GVR_OK;
  }
  bool timed_out = false;
  if (d.dev.assoc == GVR_ASSOC_VERTEX) {
    if (!s->d_flag && (e = cudaMalloc(&s->d_flag, sizeof(int))) != cudaSuccess)
      return cuda_error(e, "cudaMalloc flag");
    e = launch_brick_field(field, dtype, stride, location == GVR_MEM_DEVICE, d.dev.dims, d.dev.bshift,
                           d.d_bricks, d.dev.nbrick, d.d_brick_range, d.range, d.stg, s->d_flag,
                           &timed_out, 0);
  } else {
    e = launch_cells_field(field, dtype, stride, location == GVR_MEM_DEVICE, (int64_t)d.n_values,
                           d.d_cells, d.range, d.stg, 0);
  }
  if (e != cudaSuccess) return cuda_error(e, "field upload");
  s->table_dirty = true;
  s->classify_valid = false;
  if (timed_out) {
    // the bricks were rewritten with non-finite ranges: the domain's range
    // is unknown until the field is published again
    d.range[0] = d.range[1] = std::nan("");
    return set_error(GVR_ERR_TIMEOUT, "field staging copy did not complete");
  }
  if (!(std::isfinite(d.range[0]) && std::isfinite(d.range[1])))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "field contains non-finite values");
  s->table_dirty = true;
  s->classify_valid = false;
  return GVR_OK;
}

static int add_structured(gvr_scene *s, int kind, const int dims[3], const double origin[3],
                          const double spacing[3], const double *coords[3], const void *field,
                          int dtype, int64_t stride, int assoc, int location, int *domain_id)
{
  if (!s || !dims) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if ((int)s->domains.size() >= kMaxDomains)
    return set_error(GVR_ERR_UNSUPPORTED, "a scene holds at most 64 structured domains");
  for (int a = 0; a < 3; ++a)
    if (dims[a] < 2) return set_error(GVR_ERR_INVALID_ARGUMENT, "every dimension needs >= 2 nodes");
  if (assoc != GVR_ASSOC_VERTEX && assoc != GVR_ASSOC_ELEMENT)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad field association");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  Domain d;
  std::memset(&d.dev, 0, sizeof(d.dev));
  d.dev.kind = kind;
  d.dev.assoc = assoc;
  d.dev.bshift = s->brick_shift;
  for (int a = 0; a < 3; ++a) {
    d.dev.dims[a] = dims[a];
    d.dev.nbrick[a] = (dims[a] - 1 + brick_cells(s->brick_shift) - 1) / brick_cells(s->brick_shift);
  }
  if (kind == GVR_DOMAIN_UNIFORM) {
    for (int a = 0; a < 3; ++a) {
      const float o = (float)origin[a], sp = (float)spacing[a];
      if (!(sp > 0) || !std::isfinite(o))
        return set_error(GVR_ERR_INVALID_ARGUMENT, "uniform spacing must be > 0 and origin finite");
      d.dev.origin[a] = o;
      d.dev.inv_spacing[a] = 1.0f / sp;
      d.dev.lo[a] = o;
      d.dev.hi[a] = (float)((double)o + (double)(dims[a] - 1) * (double)sp);
      d.bounds[2 * a] = d.dev.lo[a];
      d.bounds[2 * a + 1] = d.dev.hi[a];
    }
  } else {
    for (int a = 0; a < 3; ++a) {
      if (!coords[a]) return set_error(GVR_ERR_INVALID_ARGUMENT, "rectilinear coordinates are NULL");
      std::vector<float> c(dims[a]);
      for (int i = 0; i < dims[a]; ++i) {
        c[i] = (float)coords[a][i];
        if (i > 0 && !(c[i] > c[i - 1]))
          return set_error(GVR_ERR_INVALID_ARGUMENT, "rectilinear coordinates must increase");
      }
      e = cudaMalloc(&d.d_coord[a], sizeof(float) * dims[a]);
      if (e != cudaSuccess) { free_domain(d); return cuda_error(e, "cudaMalloc coords"); }
      e = cudaMemcpy(d.d_coord[a], c.data(), sizeof(float) * dims[a], cudaMemcpyHostToDevice);
      if (e != cudaSuccess) { free_domain(d); return cuda_error(e, "copy coords"); }
      d.dev.coord[a] = d.d_coord[a];
      d.dev.lo[a] = c.front();
      d.dev.hi[a] = c.back();
      d.dev.origin[a] = c.front();
      d.dev.inv_spacing[a] = 1.f;
      d.bounds[2 * a] = c.front();
      d.bounds[2 * a + 1] = c.back();
    }
  }
  if (assoc == GVR_ASSOC_VERTEX) {
    d.n_values = (size_t)dims[0] * dims[1] * dims[2];
    d.n_bricks = (int64_t)d.dev.nbrick[0] * d.dev.nbrick[1] * d.dev.nbrick[2];
    if (d.n_bricks * brick_floats(d.dev.bshift) >= (int64_t)1 << 31) {
      free_domain(d);
      return set_error(GVR_ERR_UNSUPPORTED,
                       "a domain's bricked field must hold < 2^31 floats (about 1290^3 nodes); "
                       "split it into more domains");
    }
    e = cudaMalloc(&d.d_bricks, sizeof(float) * brick_floats(d.dev.bshift) * d.n_bricks);
    if (e == cudaSuccess) e = cudaMalloc(&d.d_brick_range, sizeof(float2) * d.n_bricks);
    if (e == cudaSuccess) e = cudaMalloc(&d.d_brick_empty, d.n_bricks);
    if (e == cudaSuccess) e = cudaMemset(d.d_brick_empty, 0, d.n_bricks);
  } else {
    d.n_values = (size_t)(dims[0] - 1) * (dims[1] - 1) * (dims[2] - 1);
    e = cudaMalloc(&d.d_cells, sizeof(float) * d.n_values);
  }
  if (e != cudaSuccess) { free_domain(d); return cuda_error(e, "cudaMalloc field"); }
  d.dev.bricks = d.d_bricks;
  d.dev.cells = d.d_cells;
  d.dev.brick_range = d.d_brick_range;
  d.dev.brick_empty = d.d_brick_empty;
  int rc = upload_field(s, d, field, dtype, stride, location);
  if (rc != GVR_OK) { free_domain(d); return rc; }
  s->domains.push_back(d);
  s->table_dirty = true;
  if (domain_id) *domain_id = (int)s->domains.size() - 1;
  return GVR_OK;
}

int gvr_scene_add_uniform(gvr_scene *s, const int dims[3], const double origin[3],
                          const double spacing[3], const void *field, int dtype, int64_t stride,
                          int association, int location, int *domain_id)
{
  if (!origin || !spacing) return set_error(GVR_ERR_INVALID_ARGUMENT, "origin/spacing is NULL");
  const double *coords[3] = {nullptr, nullptr, nullptr};
  return add_structured(s, GVR_DOMAIN_UNIFORM, dims, origin, spacing, coords, field, dtype, stride,
                        association, location, domain_id);
}

int gvr_scene_add_rectilinear(gvr_scene *s, const int dims[3], const double *x, const double *y,
                              const double *z, const void *field, int dtype, int64_t stride,
                              int association, int location, int *domain_id)
{
  const double *coords[3] = {x, y, z};
  return add_structured(s, GVR_DOMAIN_RECTILINEAR, dims, nullptr, nullptr, coords, field, dtype,
                        stride, association, location, domain_id);
}

int gvr_scene_update_field(gvr_scene *s, int domain_id, const void *field, int dtype,
                           int64_t stride, int location)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (domain_id < 0 || domain_id >= (int)s->domains.size())
    return set_error(GVR_ERR_NOT_FOUND, "no such domain");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  return upload_field(s, s->domains[domain_id], field, dtype, stride, location);
}

int gvr_scene_update_fields(gvr_scene *s, int n, const int *domain_ids, const void *const *fields,
                            int dtype, int64_t stride, int location, void *stream)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (n < 0 || (n > 0 && (!domain_ids || !fields)))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad domain or field arrays");
  if (dtype != GVR_DTYPE_FLOAT32 && dtype != GVR_DTYPE_FLOAT64)
    return set_error(GVR_ERR_UNSUPPORTED, "field dtype must be float32 or float64");
  if (stride < 1) return set_error(GVR_ERR_INVALID_ARGUMENT, "field stride must be >= 1");
  if (location != GVR_MEM_HOST && location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad field location");
  for (int k = 0; k < n; ++k) {
    if (domain_ids[k] < 0 || domain_ids[k] >= (int)s->domains.size())
      return set_error(GVR_ERR_NOT_FOUND, "no such domain");
    if (!fields[k]) return set_error(GVR_ERR_INVALID_ARGUMENT, "field is NULL");
  }
  if (n == 0) return GVR_OK;
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const size_t esz = dtype == GVR_DTYPE_FLOAT64 ? 8 : 4;
  auto piped = [&](const Domain &d) {
    return d.dev.kind != GVR_DOMAIN_HEX && d.dev.assoc == GVR_ASSOC_VERTEX;
  };
  auto src_bytes = [&](const Domain &d) {
    return (size_t)((int64_t)(d.n_values - 1) * stride + 1) * esz;
  };
  if (n > s->ranges_cap) {
    cudaFree(s->d_ranges);
    cudaFreeHost(s->h_ranges);
    s->d_ranges = nullptr;
    s->h_ranges = nullptr;
    s->ranges_cap = 0;
    if ((e = cudaMalloc(&s->d_ranges, sizeof(float2) * (n + 1))) != cudaSuccess)
      return cuda_error(e, "cudaMalloc ranges");
    if ((e = cudaMallocHost(&s->h_ranges, sizeof(float2) * (n + 1))) != cudaSuccess)
      return cuda_error(e, "cudaMallocHost ranges");
    s->ranges_cap = n;
  }
  // the timeout flag sits after the n ranges
  int *d_timed_out = reinterpret_cast<int *>(s->d_ranges + n);
  if ((e = cudaMemsetAsync(d_timed_out, 0, sizeof(int), st)) != cudaSuccess)
    return cuda_error(e, "clear flag");
  if (location == GVR_MEM_HOST) {
    size_t need = 0;
    int jobs = 0;
    for (int k = 0; k < n; ++k)
      if (piped(s->domains[domain_ids[k]])) {
        need = std::max(need, src_bytes(s->domains[domain_ids[k]]));
        ++jobs;
      }
    if (!s->copy_stream) {
      if ((e = cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking)) != cudaSuccess)
        return cuda_error(e, "copy stream");
      for (int b = 0; b < gvr_scene::kStageMax && e == cudaSuccess; ++b) {
        e = cudaEventCreateWithFlags(&s->copied[b], cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&s->consumed[b], cudaEventDisableTiming);
      }
      if (e != cudaSuccess) return cuda_error(e, "copy events");
    }
    // one buffer per field up to kStageMax within ~1 GB (at least two): a
    // copy then never waits for the bricking of an earlier field, which
    // may be held back by other work on the GPU
    const int want = (int)std::min<int64_t>(
        std::min(gvr_scene::kStageMax, std::max(jobs, 1)),
        std::max<int64_t>(2, ((int64_t)1 << 30) / (int64_t)std::max<size_t>(need, 1)));
    if (jobs > 0 && (need > s->stage_bytes || want > s->stage_count)) {
      // the old buffers may still be read by bricking from an earlier call
      if ((e = cudaDeviceSynchronize()) != cudaSuccess) return cuda_error(e, "staging");
      for (int b = 0; b < gvr_scene::kStageMax; ++b) {
        cudaFree(s->stage[b]);
        s->stage[b] = nullptr;
      }
      const size_t bytes = std::max(need, s->stage_bytes);
      s->stage_bytes = 0;
      s->stage_count = 0;
      for (int b = 0; b < want; ++b)
        if ((e = cudaMalloc(&s->stage[b], bytes)) != cudaSuccess) return cuda_error(e, "staging");
      s->stage_bytes = bytes;
      s->stage_count = want;
    }
  }
  // copies run ahead of the bricking by up to stage_count fields; the
  // domains' ranges are reduced in one launch after the last field
  int j = 0;
  std::vector<const float2 *> job_ranges;
  std::vector<int64_t> job_bricks;
  std::vector<float2 *> job_out;
  // device-resident contiguous float32 fields in 8^3-cell bricks: every
  // field's bricking in one launch, so that the domains' tails overlap
  bool merged = location == GVR_MEM_DEVICE && dtype == GVR_DTYPE_FLOAT32 && stride == 1;
  for (int k = 0; k < n && merged; ++k) {
    const Domain &d = s->domains[domain_ids[k]];
    if (piped(d) && d.dev.bshift != kBrickShiftDefault) merged = false;
  }
  if (merged) {
    std::vector<const float *> srcs;
    std::vector<float *> bricks;
    std::vector<float2 *> ranges;
    std::vector<std::array<int, 3>> dims, nbrick;
    for (int k = 0; k < n; ++k) {
      Domain &d = s->domains[domain_ids[k]];
      if (!piped(d)) continue;
      srcs.push_back(static_cast<const float *>(fields[k]));
      bricks.push_back(d.d_bricks);
      ranges.push_back(d.d_brick_range);
      dims.push_back({d.dev.dims[0], d.dev.dims[1], d.dev.dims[2]});
      nbrick.push_back({d.dev.nbrick[0], d.dev.nbrick[1], d.dev.nbrick[2]});
      job_ranges.push_back(d.d_brick_range);
      job_bricks.push_back(d.n_bricks);
      job_out.push_back(s->d_ranges + k);
      ++j;
    }
    if (j > 0) {
      e = launch_brick_device_many(j, srcs.data(), reinterpret_cast<const int(*)[3]>(dims.data()),
                                   bricks.data(), reinterpret_cast<const int(*)[3]>(nbrick.data()),
                                   ranges.data(), d_timed_out, st);
      if (e != cudaSuccess) return cuda_error(e, "field bricking");
    }
  }
  for (int k = 0; k < n && !merged; ++k) {
    Domain &d = s->domains[domain_ids[k]];
    if (!piped(d)) continue;
    const void *dsrc = fields[k];
    const int b = s->stage_count > 0 ? j % s->stage_count : 0;
    if (location == GVR_MEM_HOST) {
      e = cudaStreamWaitEvent(s->copy_stream, s->consumed[b], 0);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(s->stage[b], fields[k], src_bytes(d), cudaMemcpyHostToDevice, s->copy_stream);
      if (e == cudaSuccess) e = cudaEventRecord(s->copied[b], s->copy_stream);
      if (e == cudaSuccess) e = cudaStreamWaitEvent(st, s->copied[b], 0);
      if (e != cudaSuccess) return cuda_error(e, "field copy");
      dsrc = s->stage[b];
    }
    e = launch_brick_device(dsrc, dtype, stride, d.dev.dims, d.dev.bshift, d.d_bricks, d.dev.nbrick,
                            d.d_brick_range, d_timed_out, st);
    if (e == cudaSuccess && location == GVR_MEM_HOST) e = cudaEventRecord(s->consumed[b], st);
    if (e != cudaSuccess) return cuda_error(e, "field bricking");
    job_ranges.push_back(d.d_brick_range);
    job_bricks.push_back(d.n_bricks);
    job_out.push_back(s->d_ranges + k);
    ++j;
  }
  if (j > 0) {
    e = launch_ranges_of_bricks(j, job_ranges.data(), job_bricks.data(), job_out.data(), st);
    if (e != cudaSuccess) return cuda_error(e, "field ranges");
  }
  s->table_dirty = true;
  s->classify_valid = false;
  if (j > 0) {
    // ranges and the timeout flag in one copy
    const float2 *r = s->h_ranges;
    e = cudaMemcpyAsync(s->h_ranges, s->d_ranges, sizeof(float2) * (n + 1), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "field ranges");
    if (reinterpret_cast<const int *>(s->h_ranges + n)[0] != 0) {
      // some bricks were rewritten with non-finite ranges: the ranges of
      // this call's domains are unknown until they are published again
      for (int k = 0; k < n; ++k) {
        Domain &d = s->domains[domain_ids[k]];
        if (piped(d)) d.range[0] = d.range[1] = std::nan("");
      }
      return set_error(GVR_ERR_TIMEOUT, "field staging copy did not complete");
    }
    bool bad = false;
    for (int k = 0; k < n; ++k) {
      Domain &d = s->domains[domain_ids[k]];
      if (!piped(d)) continue;
      d.range[0] = r[k].x;
      d.range[1] = r[k].y;
      bad = bad || !(std::isfinite(d.range[0]) && std::isfinite(d.range[1]));
    }
    if (bad) return set_error(GVR_ERR_INVALID_ARGUMENT, "field contains non-finite values");
  }
  // element fields and hexahedral domains: one at a time
  for (int k = 0; k < n; ++k) {
    Domain &d = s->domains[domain_ids[k]];
    if (piped(d)) continue;
    const int rc = upload_field(s, d, fields[k], dtype, stride, location);
    if (rc != GVR_OK) return rc;
  }
  return GVR_OK;
}

int gvr_scene_set_batch_granularity(gvr_scene *s, int tiles_per_item)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (tiles_per_item < 1 || tiles_per_item > 64)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "tiles_per_item must be in [1, 64]");
  s->tuning.tiles_per_item = tiles_per_item;
  return GVR_OK;
}

int gvr_scene_set_tuning(gvr_scene *s, int packet_w, int unroll, int min_blocks)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if ((packet_w != 4 && packet_w != 8 && packet_w != 16) || unroll < 1 || unroll > 4 ||
      (min_blocks != 3 && min_blocks != 4) || (unroll == 4 && packet_w == 16) ||
      (unroll == 3 && min_blocks == 3 && packet_w == 16))
    return set_error(GVR_ERR_INVALID_ARGUMENT,
                     "tuning: packet_w in {4,8,16}, unroll in {1,2,3,4}, min_blocks in {3,4}; "
                     "16-wide packets take at most 3 samples per iteration, and 3 only at 4 CTAs per SM");
  s->tuning.packet_w = packet_w;
  s->tuning.unroll = unroll;
  s->tuning.min_blocks = min_blocks;
  return GVR_OK;
}

int gvr_scene_num_domains(const gvr_scene *s, int *n)
{
  if (!s || !n) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = (int)s->domains.size();
  return GVR_OK;
}

int gvr_scene_bounds(const gvr_scene *s, int domain_id, double b[6])
{
  if (!s || !b) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (domain_id >= (int)s->domains.size() || domain_id < -1)
    return set_error(GVR_ERR_NOT_FOUND, "no such domain");
  if (domain_id >= 0) {
    std::memcpy(b, s->domains[domain_id].bounds, sizeof(double) * 6);
    return GVR_OK;
  }
  if (s->domains.empty()) return set_error(GVR_ERR_NOT_FOUND, "scene has no domains");
  for (int a = 0; a < 3; ++a) {
    b[2 * a] = INFINITY;
    b[2 * a + 1] = -INFINITY;
  }
  for (const Domain &d : s->domains)
    for (int a = 0; a < 3; ++a) {
      b[2 * a] = std::min(b[2 * a], d.bounds[2 * a]);
      b[2 * a + 1] = std::max(b[2 * a + 1], d.bounds[2 * a + 1]);
    }
  return GVR_OK;
}

int gvr_scene_range(const gvr_scene *s, double r[2])
{
  if (!s || !r) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  if (s->domains.empty()) return set_error(GVR_ERR_NOT_FOUND, "scene has no domains");
  r[0] = INFINITY;
  r[1] = -INFINITY;
  for (const Domain &d : s->domains) {
    if (!(std::isfinite(d.range[0]) && std::isfinite(d.range[1]))) {
      // a domain whose field publish did not complete: range unknown
      r[0] = r[1] = std::nan("");
      return GVR_OK;
    }
    r[0] = std::min(r[0], d.range[0]);
    r[1] = std::max(r[1], d.range[1]);
  }
  return GVR_OK;
}

// ---------------------------------------------------------------------------
// Render
// ---------------------------------------------------------------------------

static int check_params(const gvr_render_params *p)
{
  if (!p) return set_error(GVR_ERR_INVALID_ARGUMENT, "params is NULL");
  if (p->width < 1 || p->height < 1 || (int64_t)p->width * p->height > (1ll << 28))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "image size must be >= 1 and <= 2^28 pixels");
  if (!(p->sample_dist > 0) || !std::isfinite(p->sample_dist))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "sample_dist must be > 0");
  if (!p->lut_rgba || p->lut_size < 2 || p->lut_size > kMaxLut)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "lut_size must be in [2, 4096]");
  if (p->lut_filter != GVR_LUT_NEAREST && p->lut_filter != GVR_LUT_LINEAR)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad lut_filter");
  if (!std::isfinite(p->scalar_min) || !std::isfinite(p->scalar_max))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "scalar range must be finite");
  return GVR_OK;
}

static int ensure_buffers(gvr_scene *s, int64_t pixels, int lut_size)
{
  cudaError_t e;
  if (s->table_dirty || s->d_domains_cap < (int)s->domains.size()) {
    if (s->d_domains_cap < (int)s->domains.size()) {
      cudaFree(s->d_domains);
      s->d_domains = nullptr;
      e = cudaMalloc(&s->d_domains, sizeof(DomainDev) * kMaxDomains);
      if (e != cudaSuccess) return cuda_error(e, "cudaMalloc domain table");
      s->d_domains_cap = kMaxDomains;
    }
    if (!s->d_any_empty) {
      e = cudaMalloc(&s->d_any_empty, sizeof(int) * kMaxDomains);
      if (e == cudaSuccess) e = cudaMemset(s->d_any_empty, 0, sizeof(int) * kMaxDomains);
      if (e != cudaSuccess) return cuda_error(e, "cudaMalloc empty flags");
    }
    std::vector<DomainDev> h(s->domains.size());
    for (size_t i = 0; i < h.size(); ++i) {
      h[i] = s->domains[i].dev;
      h[i].any_empty = s->d_any_empty + i;
    }
    if (!h.empty()) {
      e = cudaMemcpy(s->d_domains, h.data(), sizeof(DomainDev) * h.size(), cudaMemcpyHostToDevice);
      if (e != cudaSuccess) return cuda_error(e, "copy domain table");
    }
    s->table_dirty = false;
  }
  if (!s->d_lut) {
    e = cudaMalloc(&s->d_lut, sizeof(float4) * kMaxLut);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc LUT");
  }
  if (!s->d_counters) {
    e = cudaMalloc(&s->d_counters, sizeof(unsigned long long) * 4);
    if (e == cudaSuccess) e = cudaMemset(s->d_counters, 0, sizeof(unsigned long long) * 4);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc counters");
  }
  if (pixels > s->tmp_pixels) {
    cudaFree(s->d_rgba_tmp);
    cudaFree(s->d_depth_tmp);
    s->d_rgba_tmp = nullptr;
    s->d_depth_tmp = nullptr;
    s->tmp_pixels = 0;
    e = cudaMalloc(&s->d_rgba_tmp, sizeof(float4) * pixels);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_depth_tmp, sizeof(float) * pixels);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc image");
    s->tmp_pixels = pixels;
  }
  (void)lut_size;
  return GVR_OK;
}

// MarchParams of one render, plus the empty-brick classification of every
// vertex-field domain against this transfer function, reused while the LUT,
// its filter, the range and the fields stay those of the last render.
static int prepare_march(gvr_scene *s, const gvr_render_params *p, cudaStream_t st, MarchParams &mp)
{
  cudaError_t e;
  // zeroed bytewise, padding included: the batch path compares launch
  // parameters bytewise to decide whether its captured graph still applies
  std::memset(static_cast<void *>(&mp), 0, sizeof(mp));
  mp.width = p->width;
  mp.height = p->height;
  mp.n_domains = (int)s->domains.size();
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

  // empty-space skipping: classify bricks against this transfer function,
  // unless the LUT, filter, range and fields are those of the last render
  mp.skip_empty = 1;
  const size_t lut_floats = (size_t)p->lut_size * 4;
  const bool same = s->classify_valid && s->classify_lut.size() == lut_floats &&
                    s->classify_filter == p->lut_filter && s->classify_smin == mp.scalar_min &&
                    s->classify_inv_range == mp.inv_range &&
                    std::memcmp(s->classify_lut.data(), p->lut_rgba, lut_floats * sizeof(float)) == 0;
  if (!same) {
    e = cudaMemcpyAsync(s->d_lut, p->lut_rgba, sizeof(float4) * p->lut_size, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_any_empty, 0, sizeof(int) * kMaxDomains, st);
    if (e != cudaSuccess) return cuda_error(e, "copy LUT");
    for (size_t i = 0; i < s->domains.size(); ++i) {
      Domain &d = s->domains[i];
      if (d.dev.assoc != GVR_ASSOC_VERTEX) continue;
      e = launch_empty_bricks(d.d_brick_range, d.n_bricks, s->d_lut, p->lut_size, p->lut_filter,
                              mp.scalar_min, mp.inv_range, d.d_brick_empty, s->d_any_empty + i, st);
      if (e != cudaSuccess) return cuda_error(e, "empty-brick pass");
    }
    s->classify_lut.assign(p->lut_rgba, p->lut_rgba + lut_floats);
    s->classify_filter = p->lut_filter;
    s->classify_smin = mp.scalar_min;
    s->classify_inv_range = mp.inv_range;
    s->classify_valid = true;
  }
  return GVR_OK;
}

static int render_one(gvr_scene *s, const gvr_camera *camera, const gvr_render_params *p,
                      float *rgba, float *depth, int out_location, void *stream,
                      uint64_t *samples_out, bool over);

// Launch order of the march kernel's tiles: by increasing distance from the
// centre of the image. The hardware starts CTAs in launch order as SM slots
// free up, so the costliest tiles (the longest rays, where a volume framed by
// the camera projects) start first and the cheap tiles at the border of the
// image fill the end of the launch, instead of a last wave of long rays
// keeping a few SMs busy while the others idle. The order changes no pixel.
// One table per tile grid, built once (a counting sort by squared distance in
// tiles) and uploaded with a synchronous copy, then never written again, so
// renders on any stream may read it. *out is NULL (row-major launch order)
// when the grid is too large for a table.
static int tile_order(gvr_scene *s, int W, int H, const int **out)
{
  *out = nullptr;
  const int tx = (W + kMarchTile - 1) / kMarchTile, ty = (H + kMarchTile - 1) / kMarchTile;
  const int64_t n = (int64_t)tx * ty;
  if (n > (1 << 20)) return GVR_OK;
  const auto it = s->tile_orders.find({tx, ty});
  if (it != s->tile_orders.end()) {
    *out = it->second;
    return GVR_OK;
  }
  // distances in half tiles from the image centre (integers for any parity)
  auto key = [&](int x, int y) {
    const int64_t dx = 2 * x + 1 - tx, dy = 2 * y + 1 - ty;
    return dx * dx + dy * dy;
  };
  const int64_t max_key = key(0, 0);
  if (max_key > (1 << 24)) return GVR_OK;
  std::vector<int> cnt(max_key + 2, 0), ord(n);
  for (int y = 0; y < ty; ++y)
    for (int x = 0; x < tx; ++x) ++cnt[key(x, y) + 1];
  for (size_t k = 1; k < cnt.size(); ++k) cnt[k] += cnt[k - 1];
  for (int y = 0; y < ty; ++y)
    for (int x = 0; x < tx; ++x) ord[cnt[key(x, y)]++] = y * tx + x;
  int *d = nullptr;
  cudaError_t e = cudaMalloc(&d, sizeof(int) * n);
  if (e != cudaSuccess) return cuda_error(e, "cudaMalloc tile order");
  e = cudaMemcpy(d, ord.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    cudaFree(d);
    return cuda_error(e, "copy tile order");
  }
  s->tile_orders[{tx, ty}] = d;
  *out = d;
  return GVR_OK;
}

// Front-to-back order of the domains for rays from `eye`, for the staged
// march: domain i goes before domain j when a plane between their boxes
// (i's upper face below j's lower face on some axis, or the reverse) has
// the eye on i's side; every ray from the eye that crosses both boxes then
// crosses i first. Pairs the eye sees along no such plane (it lies between
// them, on a face plane, or the planes disagree) no ray crosses in a fixed
// order, so they are left free. A topological sort, lowest index first
// among the ready domains, gives the order; false when the scene is not
// eligible (not all uniform vertex fields) or the relation has a cycle.
static bool staged_order(const gvr_scene *s, const float eye[3], StageOrder &out)
{
  const int n = (int)s->domains.size();
  if (s->has_hex || n < 1 || n > kMaxDomains) return false;
  for (const Domain &d : s->domains)
    if (d.dev.kind != GVR_DOMAIN_UNIFORM || d.dev.assoc != GVR_ASSOC_VERTEX ||
        d.dev.bshift != kBrickShiftDefault)
      return false;
  std::vector<uint64_t> before(n, 0);   // before[j]: bits of domains that must precede j
  for (int i = 0; i < n; ++i) {
    for (int j = i + 1; j < n; ++j) {
      const double *bi = s->domains[i].bounds, *bj = s->domains[j].bounds;
      int vote = 0;          // +1: i first, -1: j first
      bool conflict = false;
      for (int a = 0; a < 3; ++a) {
        int v = 0;
        if (bi[2 * a + 1] <= bj[2 * a]) {          // i below j on axis a
          if (eye[a] < bi[2 * a + 1]) v = 1;
          else if (eye[a] > bj[2 * a]) v = -1;
        } else if (bj[2 * a + 1] <= bi[2 * a]) {   // j below i
          if (eye[a] < bj[2 * a + 1]) v = -1;
          else if (eye[a] > bi[2 * a]) v = 1;
        }
        if (v != 0) {
          if (vote != 0 && vote != v) conflict = true;
          vote = v;
        }
      }
      if (conflict || vote == 0) continue;
      if (vote > 0) before[j] |= 1ull << i;
      else before[i] |= 1ull << j;
    }
  }
  uint64_t done = 0;
  out.n = n;
  for (int k = 0; k < n; ++k) {
    int pick = -1;
    for (int j = 0; j < n && pick < 0; ++j)
      if (!(done >> j & 1) && (before[j] & ~done) == 0) pick = j;
    if (pick < 0) return false;   // a cycle
    out.d[k] = (unsigned char)pick;
    done |= 1ull << pick;
  }
  return true;
}

int gvr_scene_set_brick_cells(gvr_scene *s, int cells)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (cells != 4 && cells != 8 && cells != 16)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "brick cells must be 4, 8 or 16");
  for (const Domain &d : s->domains)
    if (d.dev.kind != GVR_DOMAIN_HEX && d.dev.assoc == GVR_ASSOC_VERTEX)
      return set_error(GVR_ERR_INVALID_ARGUMENT,
                       "set the brick size before adding vertex-field domains");
  s->brick_shift = cells == 4 ? 2 : (cells == 16 ? 4 : 3);
  return GVR_OK;
}

int gvr_scene_set_staging(gvr_scene *s, int mode)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (mode < 0 || mode > 2) return set_error(GVR_ERR_INVALID_ARGUMENT, "staging mode must be 0, 1 or 2");
  s->tuning.staged = mode;
  return GVR_OK;
}

int gvr_scene_set_tile_order(gvr_scene *s, int mode)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (mode != 0 && mode != 1) return set_error(GVR_ERR_INVALID_ARGUMENT, "tile order mode must be 0 or 1");
  s->tuning.tile_order = mode;
  return GVR_OK;
}

int gvr_scene_staging_failures(const gvr_scene *s, uint64_t *n)
{
  if (!s || !n) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = 0;
  if (!s->d_counters) return GVR_OK;
  cudaError_t e = cudaSetDevice(s->device);
  unsigned long long c = 0;
  if (e == cudaSuccess) e = cudaMemcpy(&c, s->d_counters + 1, sizeof(c), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return cuda_error(e, "read staging counter");
  *n = c;
  return GVR_OK;
}

int gvr_render_volume(gvr_scene *s, const gvr_camera *camera, const gvr_render_params *p,
                      float *rgba, float *depth, int out_location, void *stream,
                      uint64_t *samples_out)
{
  return render_one(s, camera, p, rgba, depth, out_location, stream, samples_out, false);
}

int gvr_render_volume_over(gvr_scene *s, const gvr_camera *camera, const gvr_render_params *p,
                           float *rgba, float *depth, int location, void *stream,
                           uint64_t *samples_out)
{
  return render_one(s, camera, p, rgba, depth, location, stream, samples_out, true);
}

static int render_one(gvr_scene *s, const gvr_camera *camera, const gvr_render_params *p,
                      float *rgba, float *depth, int out_location, void *stream,
                      uint64_t *samples_out, bool over)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  int rc = check_camera(camera);
  if (rc != GVR_OK) return rc;
  if ((rc = check_params(p)) != GVR_OK) return rc;
  if (!rgba || !depth) return set_error(GVR_ERR_INVALID_ARGUMENT, "output buffers are NULL");
  if (out_location != GVR_MEM_HOST && out_location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad out_location");
  if (s->domains.empty()) return set_error(GVR_ERR_NOT_FOUND, "scene has no domains");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  cudaStream_t st = (cudaStream_t)stream;
  const int64_t pixels = (int64_t)p->width * p->height;
  if ((rc = ensure_buffers(s, out_location == GVR_MEM_HOST ? pixels : 0, p->lut_size)) != GVR_OK)
    return rc;

  MarchParams mp;
  if ((rc = prepare_march(s, p, st, mp)) != GVR_OK) return rc;
  if (samples_out) {
    e = cudaMemsetAsync(s->d_counters, 0, sizeof(unsigned long long), st);
    if (e != cudaSuccess) return cuda_error(e, "clear counters");
  }
  ViewDev view;
  make_view(*camera, p->width, p->height, &view);
  float4 *d_rgba = out_location == GVR_MEM_DEVICE ? (float4 *)rgba : s->d_rgba_tmp;
  float *d_depth = out_location == GVR_MEM_DEVICE ? depth : s->d_depth_tmp;
  if (over) {
    // the canvas is read and written in place, one pixel per thread
    if (out_location == GVR_MEM_HOST) {
      e = cudaMemcpyAsync(d_rgba, rgba, sizeof(float4) * pixels, cudaMemcpyHostToDevice, st);
      if (e == cudaSuccess)
        e = cudaMemcpyAsync(d_depth, depth, sizeof(float) * pixels, cudaMemcpyHostToDevice, st);
      if (e != cudaSuccess) return cuda_error(e, "copy canvas to device");
    }
    mp.canvas_rgba = d_rgba;
    mp.canvas_depth = d_depth;
  }
  const int *d_order = nullptr;
  const int64_t n_tiles = (int64_t)((p->width + kMarchTile - 1) / kMarchTile) *
                          ((p->height + kMarchTile - 1) / kMarchTile);
  if (s->tuning.tile_order == 1 && n_tiles <= kCostOrderTiles) {
    if (s->cost_order_cap < n_tiles) {
      // order, costs, and the costs' maximum (zeroed here, then by every
      // sort launch)
      if (s->d_cost_order && (e = cudaStreamSynchronize(st)) != cudaSuccess)
        return cuda_error(e, "tile cost order");
      cudaFree(s->d_cost_order);
      s->d_cost_order = nullptr;
      s->cost_order_cap = 0;
      e = cudaMalloc(&s->d_cost_order, sizeof(int) * (2 * n_tiles + 1));
      if (e == cudaSuccess) e = cudaMemsetAsync(s->d_cost_order + 2 * n_tiles, 0, sizeof(int), st);
      if (e != cudaSuccess) return cuda_error(e, "cudaMalloc tile cost order");
      s->cost_order_cap = n_tiles;
    }
    e = launch_tile_cost_order(s->d_domains, view, mp, s->d_cost_order,
                               reinterpret_cast<unsigned *>(s->d_cost_order + s->cost_order_cap),
                               reinterpret_cast<unsigned *>(s->d_cost_order + 2 * s->cost_order_cap), st);
    if (e != cudaSuccess) return cuda_error(e, "tile cost order launch");
    d_order = s->d_cost_order;
  } else if ((rc = tile_order(s, p->width, p->height, &d_order)) != GVR_OK) {
    return rc;
  }
  StageOrder order;
  if (s->tuning.staged && staged_order(s, camera->position, order)) {
    e = launch_staged(s->d_domains, view, mp, s->d_lut, d_rgba, d_depth,
                      samples_out ? s->d_counters : nullptr, s->tuning, d_order, order,
                      s->d_counters + 1, st);
  } else {
    e = launch_march(s->d_domains, view, mp, s->d_lut, d_rgba, d_depth,
                     samples_out ? s->d_counters : nullptr, s->tuning, s->has_hex, d_order, st);
  }
  if (e != cudaSuccess) return cuda_error(e, "march kernel launch");
  if (out_location == GVR_MEM_HOST) {
    e = cudaMemcpyAsync(rgba, d_rgba, sizeof(float4) * pixels, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(depth, d_depth, sizeof(float) * pixels, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_error(e, "copy image to host");
  }
  if (samples_out) {
    unsigned long long n = 0;
    e = cudaMemcpyAsync(&n, s->d_counters, sizeof(n), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "read sample counter");
    *samples_out = n;
  } else if (out_location == GVR_MEM_HOST) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "render");
  }
  return GVR_OK;
}


// Conservative pixel rectangle {x0, y0, x1, y1} (inclusive) of a box seen by a
// view: the projections of its 8 corners through the same pinhole model the
// rays use, widened by one pixel; the whole image when a corner is not in
// front of the camera.
static int4 screen_rect(const ViewDev &v, const double b[6], int W, int H)
{
  double lo_x = 1e30, lo_y = 1e30, hi_x = -1e30, hi_y = -1e30;
  for (int k = 0; k < 8; ++k) {
    const double P[3] = {b[(k & 1) ? 1 : 0], b[(k & 2) ? 3 : 2], b[(k & 4) ? 5 : 4]};
    double d[3];
    for (int a = 0; a < 3; ++a) d[a] = P[a] - v.origin[a];
    const double z = d[0] * v.look[0] + d[1] * v.look[1] + d[2] * v.look[2];
    if (!(z > 1e-6)) return make_int4(0, 0, W - 1, H - 1);
    const double a = d[0] * v.ru[0] + d[1] * v.ru[1] + d[2] * v.ru[2];
    const double c = d[0] * v.rv[0] + d[1] * v.rv[1] + d[2] * v.rv[2];
    const double x = a / (z * v.dx_scale) + 0.5 * W + v.xoff;
    const double y = c / (z * v.dy_scale) + 0.5 * H + v.yoff;
    lo_x = std::min(lo_x, x); hi_x = std::max(hi_x, x);
    lo_y = std::min(lo_y, y); hi_y = std::max(hi_y, y);
  }
  const double cx0 = std::floor(lo_x) - 1, cy0 = std::floor(lo_y) - 1;
  const double cx1 = std::ceil(hi_x) + 1, cy1 = std::ceil(hi_y) + 1;
  if (cx1 < 0 || cy1 < 0 || cx0 > W - 1 || cy0 > H - 1) return make_int4(1, 1, 0, 0);  // empty
  return make_int4((int)std::max(0.0, cx0), (int)std::max(0.0, cy0), (int)std::min<double>(W - 1, cx1),
                   (int)std::min<double>(H - 1, cy1));
}

int gvr_render_volume_batch(gvr_scene *s, const gvr_camera *cameras, int n_views,
                            const gvr_render_params *p, float *rgba, float *depth,
                            int out_location, void *stream, uint64_t *samples_out)
{
  if (!s) return set_error(GVR_ERR_INVALID_ARGUMENT, "scene is NULL");
  if (n_views < 1 || !cameras) return set_error(GVR_ERR_INVALID_ARGUMENT, "need >= 1 camera");
  int rc;
  for (int i = 0; i < n_views; ++i)
    if ((rc = check_camera(cameras + i)) != GVR_OK) return rc;
  if ((rc = check_params(p)) != GVR_OK) return rc;
  if (!rgba || !depth) return set_error(GVR_ERR_INVALID_ARGUMENT, "output buffers are NULL");
  if (out_location != GVR_MEM_HOST && out_location != GVR_MEM_DEVICE)
    return set_error(GVR_ERR_INVALID_ARGUMENT, "bad out_location");
  if (s->domains.empty()) return set_error(GVR_ERR_NOT_FOUND, "scene has no domains");
  const int64_t pixels = (int64_t)p->width * p->height;
  if (pixels * n_views > (1ll << 30))
    return set_error(GVR_ERR_INVALID_ARGUMENT, "views x pixels must be <= 2^30");
  cudaError_t e = cudaSetDevice(s->device);
  if (e != cudaSuccess) return cuda_error(e, "cudaSetDevice");
  if ((rc = ensure_buffers(s, 0, p->lut_size)) != GVR_OK) return rc;
  cudaStream_t st = (cudaStream_t)stream;
  if (!st) {
    if (!s->own_stream) {
      e = cudaStreamCreate(&s->own_stream);  // blocking: ordered with the legacy stream
      if (e != cudaSuccess) return cuda_error(e, "cudaStreamCreate");
    }
    st = s->own_stream;
  }
  const int nd = (int)s->domains.size();
  if (n_views > s->views_cap) {
    cudaFree(s->d_views);
    s->d_views = nullptr;
    s->views_cap = 0;
    if ((e = cudaMalloc(&s->d_views, sizeof(ViewDev) * n_views)) != cudaSuccess)
      return cuda_error(e, "cudaMalloc views");
    s->views_cap = n_views;
  }
  if (n_views * nd > s->rects_cap) {
    cudaFree(s->d_rects);
    s->d_rects = nullptr;
    s->rects_cap = 0;
    if ((e = cudaMalloc(&s->d_rects, sizeof(int4) * n_views * nd)) != cudaSuccess)
      return cuda_error(e, "cudaMalloc rects");
    s->rects_cap = n_views * nd;
  }
  if (!s->d_queue && (e = cudaMalloc(&s->d_queue, 256)) != cudaSuccess)
    return cuda_error(e, "cudaMalloc queue");
  if (out_location == GVR_MEM_HOST && pixels * n_views > s->batch_pixels) {
    cudaFree(s->d_batch_rgba);
    cudaFree(s->d_batch_depth);
    s->d_batch_rgba = nullptr;
    s->d_batch_depth = nullptr;
    s->batch_pixels = 0;
    e = cudaMalloc(&s->d_batch_rgba, sizeof(float4) * pixels * n_views);
    if (e == cudaSuccess) e = cudaMalloc(&s->d_batch_depth, sizeof(float) * pixels * n_views);
    if (e != cudaSuccess) return cuda_error(e, "cudaMalloc batch images");
    s->batch_pixels = pixels * n_views;
  }
  MarchParams mp;
  if ((rc = prepare_march(s, p, st, mp)) != GVR_OK) return rc;
  std::vector<ViewDev> views(n_views);
  std::vector<int4> rects((size_t)n_views * nd);
  for (int v = 0; v < n_views; ++v) {
    make_view(cameras[v], p->width, p->height, &views[v]);
    for (int d = 0; d < nd; ++d)
      rects[(size_t)v * nd + d] = screen_rect(views[v], s->domains[d].bounds, p->width, p->height);
  }
  e = cudaMemcpyAsync(s->d_views, views.data(), sizeof(ViewDev) * n_views, cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(s->d_rects, rects.data(), sizeof(int4) * rects.size(), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess && samples_out) e = cudaMemsetAsync(s->d_counters, 0, sizeof(unsigned long long), st);
  if (e != cudaSuccess) return cuda_error(e, "batch set-up copies");
  float4 *d_rgba = out_location == GVR_MEM_DEVICE ? (float4 *)rgba : s->d_batch_rgba;
  float *d_depth = out_location == GVR_MEM_DEVICE ? depth : s->d_batch_depth;
  unsigned long long *d_samples = samples_out ? s->d_counters : nullptr;

  // The memset of the work counter and the persistent launch are captured
  // once per launch configuration and replayed as a CUDA graph.
  struct Key {
    MarchParams mp;
    int n_views, packet_w, unroll, min_blocks, tpi, has_hex;
    const void *ptrs[6];
  } key;
  std::memset(static_cast<void *>(&key), 0, sizeof(key));  // padding too: compared bytewise
  key.mp = mp;
  key.n_views = n_views;
  key.packet_w = s->tuning.packet_w;
  key.unroll = s->tuning.unroll;
  key.min_blocks = s->tuning.min_blocks;
  key.tpi = s->tuning.tiles_per_item;
  key.has_hex = s->has_hex ? 1 : 0;
  const void *ptrs[6] = {d_rgba, d_depth, d_samples, s->d_views, s->d_rects, s->d_domains};
  std::memcpy(key.ptrs, ptrs, sizeof(ptrs));
  const unsigned char *kb = reinterpret_cast<const unsigned char *>(&key);
  if (!s->batch_exec || s->batch_key.size() != sizeof(key) ||
      std::memcmp(s->batch_key.data(), kb, sizeof(key)) != 0) {
    if (s->batch_exec) {
      cudaGraphExecDestroy(s->batch_exec);
      s->batch_exec = nullptr;
    }
    int grid = 0;
    if ((e = batch_grid(mp, n_views, s->tuning, s->has_hex, &grid)) != cudaSuccess)
      return cuda_error(e, "batch launch shape");
    cudaGraph_t graph = nullptr;
    e = cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal);
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamBeginCapture");
    cudaError_t le = launch_batch(s->d_domains, s->d_views, s->d_rects, mp, n_views, s->d_lut, d_rgba,
                                  d_depth, d_samples, s->d_queue, s->tuning, s->has_hex, grid, st);
    e = cudaStreamEndCapture(st, &graph);
    if (le != cudaSuccess) { if (graph) cudaGraphDestroy(graph); return cuda_error(le, "batch capture"); }
    if (e != cudaSuccess) return cuda_error(e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&s->batch_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { s->batch_exec = nullptr; return cuda_error(e, "cudaGraphInstantiate"); }
    s->batch_key.assign(kb, kb + sizeof(key));
    ++s->batch_graph_builds;
  }
  e = cudaGraphLaunch(s->batch_exec, st);
  if (e != cudaSuccess) return cuda_error(e, "cudaGraphLaunch");
  count_launch();
  if (out_location == GVR_MEM_HOST) {
    e = cudaMemcpyAsync(rgba, d_rgba, sizeof(float4) * pixels * n_views, cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(depth, d_depth, sizeof(float) * pixels * n_views, cudaMemcpyDeviceToHost, st);
    if (e != cudaSuccess) return cuda_error(e, "copy images to host");
  }
  if (samples_out) {
    unsigned long long n = 0;
    e = cudaMemcpyAsync(&n, s->d_counters, sizeof(n), cudaMemcpyDeviceToHost, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "read sample counter");
    *samples_out = n;
  } else if (out_location == GVR_MEM_HOST || !stream) {
    e = cudaStreamSynchronize(st);
    if (e != cudaSuccess) return cuda_error(e, "batch render");
  }
  return GVR_OK;
}

int gvr_scene_batch_graph_builds(const gvr_scene *s, int *n)
{
  if (!s || !n) return set_error(GVR_ERR_INVALID_ARGUMENT, "NULL argument");
  *n = s->batch_graph_builds;
  return GVR_OK;
}

}  // extern "C"
