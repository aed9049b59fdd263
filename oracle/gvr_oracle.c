/*
 * gvr_oracle.c — CPU restatement of Ascent's volume-plot path.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the oracle that the CUDA product
 * is compared against; it is never linked into, loaded by, or called from
 * the product library. Only tests/, __graft_entry__.smoke() and bench.py's
 * CPU-baseline arm load it.
 *
 * Built twice from this one source (oracle/Makefile):
 *   liboracle64.so  REAL = double : the FP64 accuracy oracle.
 *   liboracle32.so  REAL = float  : the timed CPU port ("cpu_baseline").
 * OpenMP parallelises over image rows when compiled with -fopenmp.
 *
 * What it restates, and from where (paths relative to Ascent's src/libs):
 *   - opacity correction      vtkh/rendering/VolumeRenderer.cpp:448-466
 *   - sample distance         vtkh/rendering/VolumeRenderer.cpp:600-612
 *   - uint8 LUT conversion    vtkh/rendering/VolumeRenderer.cpp:65-90
 *   - per-domain partials     vtkh/rendering/VolumeRenderer.cpp:223-284
 *                             (alpha < 0.001 culled, depth = ray exit)
 *   - partial compositing     vtkh/compositing/PartialCompositor.cpp:57-90,
 *                             331-490; VolumePartial.hpp:74-95
 *   - partials -> canvas      vtkh/rendering/VolumeRenderer.cpp:287-391
 *                             (ray rebuild, image depth 0.5 z/w + 0.49)
 *   - uint8 image round trip  vtkh/compositing/Image.hpp:80-113,
 *                             vtkh/rendering/Renderer.cpp:265-283
 *   - visibility order        vtkh/rendering/VolumeRenderer.cpp:638-650,
 *                             691-831, 834-866
 *   - cinema cameras          ascent/runtimes/flow_filters/
 *                             ascent_runtime_rendering_filters.cpp:906-960
 *
 * The ray march itself lives in VTK-m v2.1.0, which is not available. It is
 * written here from the emission-absorption model with these named,
 * switchable assumptions (each is a parameter of or_render):
 *   A1 ray i,j direction = normalize(look + dx (i - W/2) + dy (j - H/2)),
 *      the same pinhole model partials_to_canvas inverts (:341-344);
 *   A2 samples at t_k = t_entry + k * sample_dist while t_k < t_exit, where
 *      [t_entry, t_exit] is the ray's slab interval with the domain bounds
 *      and t_entry is clamped at 0;
 *   A3 trilinear interpolation of nodal values (cell value for element
 *      fields), scalar normalised over [scalar_min, scalar_max] and clamped;
 *   A4 LUT lookup nearest: idx = (int)(s (N-1)); linear: lerp at s (N-1);
 *   A5 front-to-back blend C += (1-A) a c, A += (1-A) a;
 *   A6 optional early termination once the composited alpha reaches
 *      early_term (>= 1 disables it);
 *   A7 domains do not overlap (Ascent strips ghost zones before plots):
 *      along a ray they are visited in order of entry distance and each is
 *      marched from the furthest exit reached so far, so every point is
 *      covered once even where rounding makes neighbouring intervals overlap
 *      (rays in a shared face); for disjoint boxes this is the order of the
 *      reference's (pixel, exit depth) sort.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gvr.h"

#ifndef REAL
#define REAL double
#endif

#define OR_PI 3.14159265358979323846

/* ------------------------------------------------------------------ */
/* Small vector helpers                                                 */
/* ------------------------------------------------------------------ */
typedef struct { REAL x, y, z; } v3;

static v3 mk(REAL x, REAL y, REAL z) { v3 r = {x, y, z}; return r; }
static v3 add(v3 a, v3 b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
static v3 sub(v3 a, v3 b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
static v3 scl(v3 a, REAL s) { return mk(a.x * s, a.y * s, a.z * s); }
static REAL dot(v3 a, v3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static v3 cross(v3 a, v3 b)
{
  return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
}
static v3 normalize(v3 a)
{
  REAL m = (REAL)sqrt((double)dot(a, a));
  return m > 0 ? scl(a, (REAL)1 / m) : a;
}
static v3 fromf(const float *p) { return mk(p[0], p[1], p[2]); }

/* ------------------------------------------------------------------ */
/* Host logic                                                           */
/* ------------------------------------------------------------------ */

/* VolumeRenderer::CorrectOpacity (VolumeRenderer.cpp:448-466): the ratio is
 * a float (10.f / samples), the power is taken in double. */
int or_correct_opacity(const double *alpha_in, int n, int num_samples,
                       double *alpha_out)
{
  if (num_samples < 1 || n < 0) return GVR_ERR_INVALID_ARGUMENT;
  float ratio = 10.f / (float)num_samples;
  for (int i = 0; i < n; ++i)
    alpha_out[i] = 1. - pow(1. - alpha_in[i], (double)ratio);
  return GVR_OK;
}

/* VolumeRenderer::PreExecute (VolumeRenderer.cpp:600-612): float extent,
 * magnitude divided by the float sample count. */
float or_sample_distance(const double bounds[6], int num_samples)
{
  float e0 = (float)(bounds[1] - bounds[0]);
  float e1 = (float)(bounds[3] - bounds[2]);
  float e2 = (float)(bounds[5] - bounds[4]);
  float mag = sqrtf(e0 * e0 + e1 * e1 + e2 * e2);
  return mag / (float)num_samples;
}

static double pl_eval(int n, const double *pos, const double *val, int stride,
                      int c, double x, double dflt)
{
  if (n <= 0) return dflt;
  if (x <= pos[0]) return val[c];
  if (x >= pos[n - 1]) return val[(n - 1) * stride + c];
  int lo = 0, hi = n - 1;
  while (hi - lo > 1) {
    int mid = (lo + hi) / 2;
    if (pos[mid] <= x) lo = mid; else hi = mid;
  }
  double w = (x - pos[lo]) / (pos[hi] - pos[lo]);
  return val[lo * stride + c] * (1. - w) + val[hi * stride + c] * w;
}

static float to_u8_and_back(double v, int mode)
{
  if (v < 0) v = 0;
  if (v > 1) v = 1;
  double s = v * 255.0;
  unsigned u = (mode == GVR_UINT8_TRUNCATE) ? (unsigned)s : (unsigned)(s + 0.5);
  if (u > 255) u = 255;
  return (float)u * (1.0f / 255.0f);
}

/* Transfer-function sampling at positions i/(n-1), piecewise linear in RGB
 * between control points and clamped outside them; through uint8 for the
 * multi-domain LUT (detail::convert_table, VolumeRenderer.cpp:65-90). */
int or_color_table_sample(const gvr_color_table *t, int n, int uint8_mode,
                          float *out)
{
  if (!t || n < 2 || !out) return GVR_ERR_INVALID_ARGUMENT;
  for (int i = 0; i < n; ++i) {
    double x = (double)i / (double)(n - 1);
    double rgba[4];
    for (int c = 0; c < 3; ++c)
      rgba[c] = pl_eval(t->n_rgb, t->rgb_pos, t->rgb, 3, c, x, 0.0);
    rgba[3] = pl_eval(t->n_alpha, t->alpha_pos, t->alpha, 1, 0, x, 1.0);
    for (int c = 0; c < 4; ++c)
      out[i * 4 + c] = uint8_mode ? to_u8_and_back(rgba[c], uint8_mode)
                                  : (float)rgba[c];
  }
  return GVR_OK;
}

/* Camera defaults for given bounds: look at the centre from +z, view up +y,
 * 30 degree vertical field of view, at the distance where the bounding
 * sphere fills the view height; clip range [0.01, 100] x diagonal. */
int or_camera_reset_to_bounds(gvr_camera *c, const double b[6])
{
  double cx = 0.5 * (b[0] + b[1]), cy = 0.5 * (b[2] + b[3]),
         cz = 0.5 * (b[4] + b[5]);
  double dx = b[1] - b[0], dy = b[3] - b[2], dz = b[5] - b[4];
  double diag = sqrt(dx * dx + dy * dy + dz * dz);
  if (!(diag > 0)) diag = 1.0;
  double fov = 30.0;
  double dist = 0.5 * diag / tan(0.5 * fov * OR_PI / 180.0);
  c->look_at[0] = (float)cx; c->look_at[1] = (float)cy; c->look_at[2] = (float)cz;
  c->position[0] = (float)cx; c->position[1] = (float)cy;
  c->position[2] = (float)(cz + dist);
  c->up[0] = 0.f; c->up[1] = 1.f; c->up[2] = 0.f;
  c->fov_y = (float)fov;
  c->zoom = 1.f;
  c->xpan = 0.f; c->ypan = 0.f;
  c->near_plane = (float)(0.01 * diag);
  c->far_plane = (float)(100.0 * diag);
  return GVR_OK;
}

/* Rodrigues rotation of v about the unit axis k by `deg` degrees. */
static void rotate(double v[3], const double k[3], double deg)
{
  double th = deg * OR_PI / 180.0, c = cos(th), s = sin(th);
  double kv = k[0] * v[0] + k[1] * v[1] + k[2] * v[2];
  double kx[3] = {k[1] * v[2] - k[2] * v[1], k[2] * v[0] - k[0] * v[2],
                  k[0] * v[1] - k[1] * v[0]};
  for (int i = 0; i < 3; ++i)
    v[i] = v[i] * c + kx[i] * s + k[i] * kv * (1 - c);
}

static void unit(double v[3])
{
  double m = sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  if (m > 0) { v[0] /= m; v[1] /= m; v[2] /= m; }
}

/* Azimuth: position rotates about view-up through look_at. */
int or_camera_azimuth(gvr_camera *c, double deg)
{
  double k[3] = {c->up[0], c->up[1], c->up[2]};
  unit(k);
  double v[3] = {c->position[0] - c->look_at[0], c->position[1] - c->look_at[1],
                 c->position[2] - c->look_at[2]};
  rotate(v, k, deg);
  for (int i = 0; i < 3; ++i) c->position[i] = (float)(c->look_at[i] + v[i]);
  return GVR_OK;
}

/* Elevation: position rotates about cross(position - look_at, up) through
 * look_at (positive angles raise the camera); view-up is unchanged. */
int or_camera_elevation(gvr_camera *c, double deg)
{
  double v[3] = {c->position[0] - c->look_at[0], c->position[1] - c->look_at[1],
                 c->position[2] - c->look_at[2]};
  double u[3] = {c->up[0], c->up[1], c->up[2]};
  double k[3] = {v[1] * u[2] - v[2] * u[1], v[2] * u[0] - v[0] * u[2],
                 v[0] * u[1] - v[1] * u[0]};
  unit(k);
  rotate(v, k, deg);
  for (int i = 0; i < 3; ++i) c->position[i] = (float)(c->look_at[i] + v[i]);
  return GVR_OK;
}

/* CinemaManager::create_cinema_cameras (rendering_filters.cpp:906-960), in
 * float like the reference: rot = RotZ(phi) RotX(theta) applied to
 * (0,0,1) and up (0,1,0); position = rot(pos) * radius + centre with
 * radius = |extent| * 2.5 / 2. */
int or_cinema_cameras(const double b[6], const float *pt, int n, gvr_camera *out)
{
  float center[3] = {(float)(0.5 * (b[0] + b[1])), (float)(0.5 * (b[2] + b[3])),
                     (float)(0.5 * (b[4] + b[5]))};
  float ext[3] = {(float)(b[1] - b[0]), (float)(b[3] - b[2]), (float)(b[5] - b[4])};
  float radius = sqrtf(ext[0] * ext[0] + ext[1] * ext[1] + ext[2] * ext[2]) *
                 2.5f / 2.0f;
  for (int a = 0; a < n; ++a) {
    gvr_camera c;
    or_camera_reset_to_bounds(&c, b);
    float phi = pt[2 * a] * (float)(OR_PI / 180.0);
    float th = pt[2 * a + 1] * (float)(OR_PI / 180.0);
    float cp = cosf(phi), sp = sinf(phi), ct = cosf(th), st = sinf(th);
    /* R = Rz(phi) * Rx(theta) */
    float R[3][3] = {{cp, -sp * ct, sp * st},
                     {sp, cp * ct, -cp * st},
                     {0.f, st, ct}};
    float up[3], pos[3];
    for (int i = 0; i < 3; ++i) {
      up[i] = R[i][1];
      pos[i] = R[i][2];
    }
    float um = sqrtf(up[0] * up[0] + up[1] * up[1] + up[2] * up[2]);
    for (int i = 0; i < 3; ++i) {
      c.up[i] = up[i] / um;
      c.position[i] = pos[i] * radius + center[i];
      c.look_at[i] = center[i];
    }
    out[a] = c;
  }
  return GVR_OK;
}

/* FindMinDepth + serial DepthSort: order[d] = rank of domain d by the float
 * distance from the camera to its bounds centre (ties: lower index first). */
int or_visibility_order(const gvr_camera *c, const double *bounds, int n,
                        int *order)
{
  float *dist = (float *)malloc(sizeof(float) * (n > 0 ? n : 1));
  for (int d = 0; d < n; ++d) {
    const double *b = bounds + 6 * d;
    float cx = (float)(0.5 * (b[0] + b[1])) - c->position[0];
    float cy = (float)(0.5 * (b[2] + b[3])) - c->position[1];
    float cz = (float)(0.5 * (b[4] + b[5])) - c->position[2];
    dist[d] = sqrtf(cx * cx + cy * cy + cz * cz);
  }
  for (int d = 0; d < n; ++d) {
    int r = 0;
    for (int e = 0; e < n; ++e)
      if (dist[e] < dist[d] || (dist[e] == dist[d] && e < d)) ++r;
    order[d] = r;
  }
  free(dist);
  return GVR_OK;
}

/* ------------------------------------------------------------------ */
/* Z-buffer compositing of opaque canvases                              */
/* ------------------------------------------------------------------ */

/* Image::Init (vtkh/compositing/Image.hpp:80-113): 8-bit colour by a
 * truncating cast of value * 255 (float arithmetic), depth made positive. */
static unsigned char or_u8(float v)
{
  float s = v * 255.f;
  if (s < 0.f) s = 0.f;
  if (s > 255.f) s = 255.f;
  return (unsigned char)s;
}

/* Renderer::Composite in Z_BUFFER_SURFACE mode for n canvases (Renderer.cpp:
 * 111-142): the first canvas is kept (Compositor::AddImage, Compositor.cpp:
 * 86-125), each later one composited into it by ImageCompositor::
 * ZBufferComposite (ImageCompositor.hpp:49-76: skip where its depth > 1 or
 * the kept depth is nearer, else take its pixel and |depth|), and the result
 * converted back by Renderer::ImageToCanvas (Renderer.cpp:271-289). */
int or_zbuffer_composite(int n, const float *const *rgba, const float *const *depth,
                         int width, int height, float *out_rgba, float *out_depth)
{
  if (n < 1 || width < 1 || height < 1) return GVR_ERR_INVALID_ARGUMENT;
  const long long size = (long long)width * height;
  for (long long i = 0; i < size; ++i) {
    unsigned char px[4];
    for (int c = 0; c < 4; ++c) px[c] = or_u8(rgba[0][4 * i + c]);
    float d = depth[0][i] < 0.f ? -depth[0][i] : depth[0][i];
    for (int k = 1; k < n; ++k) {
      float dk = depth[k][i] < 0.f ? -depth[k][i] : depth[k][i];
      if (dk > 1.f || d < dk) continue;
      d = dk;
      for (int c = 0; c < 4; ++c) px[c] = or_u8(rgba[k][4 * i + c]);
    }
    const float one_over_255 = 1.f / 255.f;
    for (int c = 0; c < 4; ++c) out_rgba[4 * i + c] = (float)px[c] * one_over_255;
    out_depth[i] = d;
  }
  return GVR_OK;
}

/* ------------------------------------------------------------------ */
/* Partial compositing (PartialCompositor::composite_partials and       */
/* BlendPartials, VolumePartial::blend)                                 */
/* ------------------------------------------------------------------ */
typedef struct {
  int pixel_id;
  float depth;
  float rgb[3];
  float alpha;
} or_partial;

typedef struct {
  REAL rgb[3];
  REAL alpha;
  REAL depth;
  int dom;
} or_rpartial;

/* VolumePartial::blend (VolumePartial.hpp:86-95). */
static void blend_partial(REAL *rgb, REAL *a, const REAL *orgb, REAL oa)
{
  if (*a >= 1 || oa == 0) return;
  REAL op = 1 - *a;
  rgb[0] += op * orgb[0];
  rgb[1] += op * orgb[1];
  rgb[2] += op * orgb[2];
  *a += op * oa;
  if (*a > 1) *a = 1;
}

static int cmp_partial(const void *pa, const void *pb)
{
  const or_partial *a = (const or_partial *)pa, *b = (const or_partial *)pb;
  if (a->pixel_id != b->pixel_id) return a->pixel_id < b->pixel_id ? -1 : 1;
  if (a->depth != b->depth) return a->depth < b->depth ? -1 : 1;
  return 0;
}

typedef struct {
  or_partial v;
  int idx;
} or_tagged;

/* (pixel id, depth) order of VolumePartial::operator< with the input index
 * as the final key, so that equal records keep their input order. */
static int cmp_tagged(const void *pa, const void *pb)
{
  const or_tagged *a = (const or_tagged *)pa, *b = (const or_tagged *)pb;
  int c = cmp_partial(&a->v, &b->v);
  if (c) return c;
  return a->idx < b->idx ? -1 : (a->idx > b->idx ? 1 : 0);
}

/* Composite n_images lists of partials (counts[i] records each, laid end to
 * end in `in`) into one list sorted by pixel id; returns the output count.
 * Partials of one pixel are blended in increasing depth order
 * (composite_partials + BlendPartials, PartialCompositor.cpp:57-90,
 * 331-490); the output record keeps the front partial's depth. */
int or_composite_partials(int n_images, const int *counts, const or_partial *in,
                          or_partial *out)
{
  int total = 0;
  for (int i = 0; i < n_images; ++i) total += counts[i];
  if (total == 0) return 0;
  or_tagged *t = (or_tagged *)malloc(sizeof(or_tagged) * total);
  for (int i = 0; i < total; ++i) { t[i].v = in[i]; t[i].idx = i; }
  qsort(t, total, sizeof(or_tagged), cmp_tagged);
  int n_out = 0;
  int i = 0;
  while (i < total) {
    int j = i + 1;
    REAL rgb[3] = {t[i].v.rgb[0], t[i].v.rgb[1], t[i].v.rgb[2]};
    REAL a = t[i].v.alpha;
    while (j < total && t[j].v.pixel_id == t[i].v.pixel_id) {
      REAL orgb[3] = {t[j].v.rgb[0], t[j].v.rgb[1], t[j].v.rgb[2]};
      blend_partial(rgb, &a, orgb, t[j].v.alpha);
      ++j;
    }
    or_partial r = t[i].v;
    r.rgb[0] = (float)rgb[0]; r.rgb[1] = (float)rgb[1]; r.rgb[2] = (float)rgb[2];
    r.alpha = (float)a;
    out[n_out++] = r;
    i = j;
  }
  free(t);
  return n_out;
}

/* ------------------------------------------------------------------ */
/* Scene                                                                */
/* ------------------------------------------------------------------ */
typedef struct {
  int kind;           /* GVR_DOMAIN_UNIFORM / RECTILINEAR */
  int dims[3];        /* node counts */
  float origin[3], spacing[3];
  REAL *coord[3];     /* rectilinear node coordinates */
  REAL lo[3], hi[3];  /* bounds */
  const float *field; /* caller-owned */
  int assoc;
  /* hexahedral domains */
  int64_t n_nodes, n_cells;
  const float *hx, *hy, *hz; /* caller-owned node coordinates */
  const int *conn;           /* caller-owned, 8 per cell */
  float *leaf_lo, *leaf_hi;  /* 3 per cell */
  uint32_t *codes, *ids;     /* sorted Morton codes, leaf -> cell */
  int *left, *right, *parent;
  float *inner_box;          /* 6 per inner node */
} or_domain;

typedef struct {
  int n;
  or_domain *d;
} or_scene;

or_scene *or_scene_new(void)
{
  or_scene *s = (or_scene *)calloc(1, sizeof(or_scene));
  return s;
}

void or_scene_free(or_scene *s)
{
  if (!s) return;
  for (int i = 0; i < s->n; ++i) {
    or_domain *d = &s->d[i];
    for (int a = 0; a < 3; ++a) free(d->coord[a]);
    free(d->leaf_lo); free(d->leaf_hi); free(d->codes); free(d->ids);
    free(d->left); free(d->right); free(d->parent); free(d->inner_box);
  }
  free(s->d);
  free(s);
}

static or_domain *push(or_scene *s)
{
  s->d = (or_domain *)realloc(s->d, sizeof(or_domain) * (s->n + 1));
  or_domain *d = &s->d[s->n++];
  memset(d, 0, sizeof(*d));
  return d;
}

/* Uniform domain: origin/spacing are taken as float32, like the Blueprint
 * adapter's cast (ascent_vtkh_data_adapter.cpp:1264-1270). */
int or_scene_add_uniform(or_scene *s, const int dims[3], const double origin[3],
                         const double spacing[3], const float *field, int assoc)
{
  or_domain *d = push(s);
  d->kind = GVR_DOMAIN_UNIFORM;
  for (int a = 0; a < 3; ++a) {
    d->dims[a] = dims[a];
    d->origin[a] = (float)origin[a];
    d->spacing[a] = (float)spacing[a];
    d->lo[a] = (REAL)d->origin[a];
    d->hi[a] = (REAL)d->origin[a] + (REAL)(dims[a] - 1) * (REAL)d->spacing[a];
  }
  d->field = field;
  d->assoc = assoc;
  return s->n - 1;
}

int or_scene_add_rectilinear(or_scene *s, const int dims[3], const double *x,
                             const double *y, const double *z, const float *field,
                             int assoc)
{
  or_domain *d = push(s);
  d->kind = GVR_DOMAIN_RECTILINEAR;
  const double *c[3] = {x, y, z};
  for (int a = 0; a < 3; ++a) {
    d->dims[a] = dims[a];
    d->coord[a] = (REAL *)malloc(sizeof(REAL) * dims[a]);
    /* VTK-m's default coordinate type is float32 */
    for (int i = 0; i < dims[a]; ++i) d->coord[a][i] = (REAL)(float)c[a][i];
    d->lo[a] = d->coord[a][0];
    d->hi[a] = d->coord[a][dims[a] - 1];
  }
  d->field = field;
  d->assoc = assoc;
  return s->n - 1;
}


/* ------------------------------------------------------------------ */
/* Hexahedral domains: CPU rebuild of the LBVH (Devil Ray's             */
/* LinearBVHBuilder, src/libs/dray/linear_bvh_builder.cpp:60-520) and   */
/* point location (DeviceMesh::locate, data_model/device_mesh.hpp:      */
/* 250-360, NewtonSolve, newton_solver.hpp:33-110).                     */
/* The box, centre and Morton arithmetic is float32 with every rounding */
/* step explicit (this file is built with -ffp-contract=off), so codes, */
/* order and topology match the device build bit for bit. Equal codes   */
/* are ordered by cell id (the reference's std::sort leaves that order  */
/* unspecified).                                                        */
/* ------------------------------------------------------------------ */
static uint32_t spread3(uint32_t x)
{
  x &= 0x3ffu;
  x = (x | (x << 16)) & 0x030000FFu;
  x = (x | (x << 8)) & 0x0300F00Fu;
  x = (x | (x << 4)) & 0x030C30C3u;
  x = (x | (x << 2)) & 0x09249249u;
  return x;
}

static uint32_t quant10(float u)
{
  float q = u * 1024.0f;
  q = q < 0.0f ? 0.0f : q;
  q = q > 1023.0f ? 1023.0f : q;
  return (uint32_t)q;
}

static const uint32_t *g_sort_codes;
static int cmp_code(const void *a, const void *b)
{
  uint32_t ia = *(const uint32_t *)a, ib = *(const uint32_t *)b;
  uint32_t ca = g_sort_codes[ia], cb = g_sort_codes[ib];
  if (ca != cb) return ca < cb ? -1 : 1;
  return ia < ib ? -1 : (ia > ib ? 1 : 0);
}

static int prefix_len(const uint32_t *codes, int n, int a, int b)
{
  if (b < 0 || b >= n) return -1;
  uint32_t x = codes[a] ^ codes[b];
  if (x) return __builtin_clz(x);
  return 32 + __builtin_clz((uint32_t)a ^ (uint32_t)b);
}

static void hex_build(or_domain *d)
{
  const int64_t nc = d->n_cells;
  d->leaf_lo = (float *)malloc(sizeof(float) * 3 * nc);
  d->leaf_hi = (float *)malloc(sizeof(float) * 3 * nc);
  float bl[3] = {INFINITY, INFINITY, INFINITY}, bh[3] = {-INFINITY, -INFINITY, -INFINITY};
  const float *xyz[3] = {d->hx, d->hy, d->hz};
  for (int64_t c = 0; c < nc; ++c) {
    for (int a = 0; a < 3; ++a) {
      float l = INFINITY, h = -INFINITY;
      for (int k = 0; k < 8; ++k) {
        float v = xyz[a][d->conn[8 * c + k]];
        l = v < l ? v : l;
        h = v > h ? v : h;
      }
      d->leaf_lo[3 * c + a] = l;
      d->leaf_hi[3 * c + a] = h;
      bl[a] = l < bl[a] ? l : bl[a];
      bh[a] = h > bh[a] ? h : bh[a];
    }
  }
  float inv[3];
  for (int a = 0; a < 3; ++a) {
    float ext = bh[a] - bl[a];
    inv[a] = ext == 0.0f ? 0.0f : 1.0f / ext;
    d->lo[a] = bl[a];
    d->hi[a] = bh[a];
  }
  uint32_t *codes = (uint32_t *)malloc(sizeof(uint32_t) * nc);
  for (int64_t c = 0; c < nc; ++c) {
    uint32_t q[3];
    for (int a = 0; a < 3; ++a) {
      float cen = 0.5f * (d->leaf_lo[3 * c + a] + d->leaf_hi[3 * c + a]);
      float u = (cen - bl[a]) * inv[a];
      q[a] = quant10(u);
    }
    codes[c] = (spread3(q[2]) << 2) | (spread3(q[1]) << 1) | spread3(q[0]);
  }
  d->ids = (uint32_t *)malloc(sizeof(uint32_t) * nc);
  for (int64_t c = 0; c < nc; ++c) d->ids[c] = (uint32_t)c;
  g_sort_codes = codes;
  qsort(d->ids, nc, sizeof(uint32_t), cmp_code);
  d->codes = (uint32_t *)malloc(sizeof(uint32_t) * nc);
  for (int64_t k = 0; k < nc; ++k) d->codes[k] = codes[d->ids[k]];
  free(codes);
  if (nc < 2) return;
  const int n = (int)nc, ni = n - 1;
  d->left = (int *)malloc(sizeof(int) * ni);
  d->right = (int *)malloc(sizeof(int) * ni);
  d->parent = (int *)malloc(sizeof(int) * (2 * n - 1));
  d->inner_box = (float *)malloc(sizeof(float) * 6 * ni);
  const uint32_t *k = d->codes;
  /* Karras 2012, "Maximizing parallelism in the construction of BVHs,
   * octrees, and k-d trees", Figure 4 */
  for (int i = 0; i < ni; ++i) {
    int dd = prefix_len(k, n, i, i + 1) - prefix_len(k, n, i, i - 1) < 0 ? -1 : 1;
    int dmin = prefix_len(k, n, i, i - dd);
    int lmax = 2;
    while (prefix_len(k, n, i, i + lmax * dd) > dmin) lmax *= 2;
    int l = 0;
    for (int t = lmax / 2; t >= 1; t /= 2)
      if (prefix_len(k, n, i, i + (l + t) * dd) > dmin) l += t;
    int j = i + l * dd;
    int dnode = prefix_len(k, n, i, j);
    int sidx = 0;
    for (int e = 1;; ++e) {
      int t = (l + (1 << e) - 1) >> e;
      if (prefix_len(k, n, i, i + (sidx + t) * dd) > dnode) sidx += t;
      if (t <= 1) break;
    }
    int split = i + sidx * dd + (dd < 0 ? dd : 0);
    int lo = i < j ? i : j, hi = i < j ? j : i;
    int lc = lo == split ? ni + split : split;
    int rc = hi == split + 1 ? ni + split + 1 : split + 1;
    d->left[i] = lc;
    d->right[i] = rc;
    d->parent[lc] = i;
    d->parent[rc] = i;
  }
  d->parent[0] = -1;
  /* boxes of inner nodes, children before parents: post-order by explicit stack */
  int *stack = (int *)malloc(sizeof(int) * 2 * n);
  char *done = (char *)calloc(ni, 1);
  int sp = 0;
  stack[sp++] = 0;
  while (sp) {
    int node = stack[sp - 1];
    int ch[2] = {d->left[node], d->right[node]};
    int pushed = 0;
    for (int q = 0; q < 2; ++q)
      if (ch[q] < ni && !done[ch[q]]) { stack[sp++] = ch[q]; pushed = 1; }
    if (pushed) continue;
    --sp;
    float *b = d->inner_box + 6 * node;
    for (int a = 0; a < 3; ++a) { b[a] = INFINITY; b[3 + a] = -INFINITY; }
    for (int q = 0; q < 2; ++q) {
      const float *cl, *chh;
      if (ch[q] >= ni) {
        uint32_t cell = d->ids[ch[q] - ni];
        cl = d->leaf_lo + 3 * cell;
        chh = d->leaf_hi + 3 * cell;
      } else {
        cl = d->inner_box + 6 * ch[q];
        chh = cl + 3;
      }
      for (int a = 0; a < 3; ++a) {
        b[a] = cl[a] < b[a] ? cl[a] : b[a];
        b[3 + a] = chh[a] > b[3 + a] ? chh[a] : b[3 + a];
      }
    }
    done[node] = 1;
  }
  free(stack);
  free(done);
}

int or_scene_add_hex(or_scene *s, int64_t n_nodes, const float *x, const float *y,
                     const float *z, int64_t n_cells, const int *conn, const float *field,
                     int assoc)
{
  if (n_cells < 1 || n_nodes < 8) return -1;
  or_domain *d = push(s);
  d->kind = GVR_DOMAIN_HEX;
  d->n_nodes = n_nodes;
  d->n_cells = n_cells;
  d->hx = x; d->hy = y; d->hz = z;
  d->conn = conn;
  d->field = field;
  d->assoc = assoc;
  hex_build(d);
  return s->n - 1;
}

/* Copy the LBVH of a hex domain (same layout as gvr_scene_hex_bvh). */
int or_hex_bvh(const or_scene *s, int dom, uint32_t *codes, uint32_t *ids, int *left,
               int *right, int *parent, float *inner_box)
{
  const or_domain *d = &s->d[dom];
  const int64_t nc = d->n_cells;
  memcpy(codes, d->codes, sizeof(uint32_t) * nc);
  memcpy(ids, d->ids, sizeof(uint32_t) * nc);
  if (nc > 1) {
    memcpy(left, d->left, sizeof(int) * (nc - 1));
    memcpy(right, d->right, sizeof(int) * (nc - 1));
    memcpy(parent, d->parent, sizeof(int) * (2 * nc - 1));
    memcpy(inner_box, d->inner_box, sizeof(float) * 6 * (nc - 1));
  }
  return GVR_OK;
}

/* Newton's method on the trilinear map of cell c (VTK hex order). */
static int hex_newton(const or_domain *d, int64_t c, const REAL p[3], REAL rst[3])
{
  REAL X[8][3];
  for (int i = 0; i < 8; ++i) {
    int nid = d->conn[8 * c + i];
    X[i][0] = d->hx[nid]; X[i][1] = d->hy[nid]; X[i][2] = d->hz[nid];
  }
  const REAL tol = sizeof(REAL) == 8 ? (REAL)1e-10 : (REAL)1e-5;
  const REAL in_tol = (REAL)2e-4; /* the device's inside tolerance */
  REAL r = rst[0], sv = rst[1], t = rst[2];
  int conv = 0;
  for (int it = 0; it < 10; ++it) {
    REAL r0 = 1 - r, s0 = 1 - sv, t0 = 1 - t;
    REAL n[8] = {r0 * s0 * t0, r * s0 * t0, r * sv * t0, r0 * sv * t0,
                 r0 * s0 * t, r * s0 * t, r * sv * t, r0 * sv * t};
    REAL dr[8] = {-s0 * t0, s0 * t0, sv * t0, -sv * t0, -s0 * t, s0 * t, sv * t, -sv * t};
    REAL ds[8] = {-r0 * t0, -r * t0, r * t0, r0 * t0, -r0 * t, -r * t, r * t, r0 * t};
    REAL dt[8] = {-r0 * s0, -r * s0, -r * sv, -r0 * sv, r0 * s0, r * s0, r * sv, r0 * sv};
    REAL F[3] = {-p[0], -p[1], -p[2]}, J[3][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
    for (int i = 0; i < 8; ++i)
      for (int a = 0; a < 3; ++a) {
        F[a] += n[i] * X[i][a];
        J[a][0] += dr[i] * X[i][a];
        J[a][1] += ds[i] * X[i][a];
        J[a][2] += dt[i] * X[i][a];
      }
    REAL c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    REAL c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    REAL c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    REAL det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    if (!(det > 0 || det < 0)) return 0;
    REAL c10 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    REAL c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    REAL c12 = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    REAL c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    REAL c21 = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    REAL c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    REAL d0 = (c00 * F[0] + c10 * F[1] + c20 * F[2]) / det;
    REAL d1 = (c01 * F[0] + c11 * F[1] + c21 * F[2]) / det;
    REAL d2 = (c02 * F[0] + c12 * F[1] + c22 * F[2]) / det;
    r -= d0; sv -= d1; t -= d2;
    if (!(fabs((double)r) < 1e3 && fabs((double)sv) < 1e3 && fabs((double)t) < 1e3)) return 0;
    REAL m = fabs((double)d0);
    if (fabs((double)d1) > m) m = fabs((double)d1);
    if (fabs((double)d2) > m) m = fabs((double)d2);
    if (m < tol) { conv = 1; break; }
  }
  rst[0] = r; rst[1] = sv; rst[2] = t;
  return conv && r >= -in_tol && r <= 1 + in_tol && sv >= -in_tol && sv <= 1 + in_tol &&
         t >= -in_tol && t <= 1 + in_tol;
}

static int in_box(const REAL p[3], const float *lo, const float *hi)
{
  return !(p[0] < lo[0] || p[1] < lo[1] || p[2] < lo[2] || p[0] > hi[0] || p[1] > hi[1] ||
           p[2] > hi[2]);
}

/* First cell containing p in left-first traversal order, or -1. */
static int64_t hex_locate(const or_domain *d, const REAL p[3], REAL rst[3])
{
  const int64_t nc = d->n_cells;
  if (nc == 1) {
    rst[0] = rst[1] = rst[2] = (REAL)0.5;
    return hex_newton(d, 0, p, rst) ? 0 : -1;
  }
  const int ni = (int)nc - 1;
  int stack[128];
  int sp = 0, node = 0; /* node < ni: inner, else leaf node - ni */
  for (;;) {
    if (node < ni) {
      int ch[2] = {d->left[node], d->right[node]};
      int in[2];
      for (int q = 0; q < 2; ++q) {
        const float *lo, *hi;
        if (ch[q] >= ni) {
          uint32_t cell = d->ids[ch[q] - ni];
          lo = d->leaf_lo + 3 * cell;
          hi = d->leaf_hi + 3 * cell;
        } else {
          lo = d->inner_box + 6 * ch[q];
          hi = lo + 3;
        }
        in[q] = in_box(p, lo, hi);
      }
      if (!in[0] && !in[1]) {
        if (!sp) return -1;
        node = stack[--sp];
        continue;
      }
      if (in[0] && in[1]) {
        if (sp < 128) stack[sp++] = ch[1];
        node = ch[0];
      } else {
        node = in[0] ? ch[0] : ch[1];
      }
    } else {
      int64_t cell = d->ids[node - ni];
      rst[0] = rst[1] = rst[2] = (REAL)0.5;
      if (hex_newton(d, cell, p, rst)) return cell;
      if (!sp) return -1;
      node = stack[--sp];
    }
  }
}

int or_hex_locate(const or_scene *s, int dom, const float *pts, int n, int *cells, float *rst)
{
  const or_domain *d = &s->d[dom];
#pragma omp parallel for schedule(dynamic, 64)
  for (int i = 0; i < n; ++i) {
    REAL p[3] = {pts[3 * i], pts[3 * i + 1], pts[3 * i + 2]}, r[3];
    cells[i] = (int)hex_locate(d, p, r);
    for (int a = 0; a < 3; ++a) rst[3 * i + a] = (float)r[a];
  }
  return GVR_OK;
}

/* ------------------------------------------------------------------ */
/* March                                                                */
/* ------------------------------------------------------------------ */

/* Slab test of the ray o + t dir against [lo, hi]; returns 1 on a hit with
 * t_exit > t_entry >= 0. */
static int slab(const REAL lo[3], const REAL hi[3], v3 o, v3 dir, REAL *t0, REAL *t1)
{
  REAL tmin = -INFINITY, tmax = INFINITY;
  REAL oo[3] = {o.x, o.y, o.z}, dd[3] = {dir.x, dir.y, dir.z};
  for (int a = 0; a < 3; ++a) {
    if (dd[a] != 0) {
      REAL inv = (REAL)1 / dd[a];
      REAL ta = (lo[a] - oo[a]) * inv, tb = (hi[a] - oo[a]) * inv;
      if (ta > tb) { REAL t = ta; ta = tb; tb = t; }
      if (ta > tmin) tmin = ta;
      if (tb < tmax) tmax = tb;
    } else if (oo[a] < lo[a] || oo[a] > hi[a]) {
      return 0;
    }
  }
  if (tmin < 0) tmin = 0;
  if (!(tmax > tmin)) return 0;
  *t0 = tmin;
  *t1 = tmax;
  return 1;
}

/* Locate one axis coordinate: cell index i in [0, n-2] and weight w. */
static void locate_axis(const or_domain *d, int a, REAL p, int *i, REAL *w)
{
  int n = d->dims[a];
  if (d->kind == GVR_DOMAIN_UNIFORM) {
    REAL g = (p - (REAL)d->origin[a]) / (REAL)d->spacing[a];
    if (g < 0) g = 0;
    if (g > (REAL)(n - 1)) g = (REAL)(n - 1);
    int c = (int)floor((double)g);
    if (c > n - 2) c = n - 2;
    *i = c;
    *w = g - (REAL)c;
  } else {
    const REAL *x = d->coord[a];
    int lo = 0, hi = n - 1;
    if (p <= x[0]) { *i = 0; *w = 0; return; }
    if (p >= x[n - 1]) { *i = n - 2; *w = 1; return; }
    while (hi - lo > 1) {
      int mid = (lo + hi) / 2;
      if (x[mid] <= p) lo = mid; else hi = mid;
    }
    *i = lo;
    *w = (p - x[lo]) / (x[lo + 1] - x[lo]);
  }
}

static REAL sample_field(const or_domain *d, v3 p, int *found)
{
  *found = 1;
  if (d->kind == GVR_DOMAIN_HEX) {
    REAL q[3] = {p.x, p.y, p.z}, rst[3];
    int64_t c = hex_locate(d, q, rst);
    if (c < 0) { *found = 0; return 0; }
    if (d->assoc == GVR_ASSOC_ELEMENT) return (REAL)d->field[c];
    for (int a = 0; a < 3; ++a) rst[a] = rst[a] < 0 ? 0 : (rst[a] > 1 ? 1 : rst[a]);
    REAL r = rst[0], sv = rst[1], t = rst[2], r0 = 1 - r, s0 = 1 - sv, t0 = 1 - t;
    REAL n[8] = {r0 * s0 * t0, r * s0 * t0, r * sv * t0, r0 * sv * t0,
                 r0 * s0 * t, r * s0 * t, r * sv * t, r0 * sv * t};
    REAL v = 0;
    for (int i = 0; i < 8; ++i) v += n[i] * (REAL)d->field[d->conn[8 * c + i]];
    return v;
  }
  int i[3];
  REAL w[3];
  REAL pp[3] = {p.x, p.y, p.z};
  for (int a = 0; a < 3; ++a) locate_axis(d, a, pp[a], &i[a], &w[a]);
  const int nx = d->dims[0], ny = d->dims[1];
  if (d->assoc == GVR_ASSOC_ELEMENT) {
    const int cx = nx - 1, cy = ny - 1;
    return (REAL)d->field[((int64_t)i[2] * cy + i[1]) * cx + i[0]];
  }
  const float *f = d->field;
  int64_t base = ((int64_t)i[2] * ny + i[1]) * nx + i[0];
  int64_t sy = nx, sz = (int64_t)nx * ny;
  REAL c000 = f[base], c100 = f[base + 1], c010 = f[base + sy],
       c110 = f[base + sy + 1], c001 = f[base + sz], c101 = f[base + sz + 1],
       c011 = f[base + sz + sy], c111 = f[base + sz + sy + 1];
  REAL c00 = c000 + (c100 - c000) * w[0];
  REAL c10 = c010 + (c110 - c010) * w[0];
  REAL c01 = c001 + (c101 - c001) * w[0];
  REAL c11 = c011 + (c111 - c011) * w[0];
  REAL c0 = c00 + (c10 - c00) * w[1];
  REAL c1 = c01 + (c11 - c01) * w[1];
  return c0 + (c1 - c0) * w[2];
}

static void lut_lookup(const float *lut, int n, int filter, REAL s, REAL out[4])
{
  if (filter == GVR_LUT_LINEAR) {
    REAL x = s * (REAL)(n - 1);
    int i0 = (int)floor((double)x);
    if (i0 > n - 2) i0 = n - 2;
    if (i0 < 0) i0 = 0;
    REAL w = x - (REAL)i0;
    for (int c = 0; c < 4; ++c)
      out[c] = (REAL)lut[i0 * 4 + c] * (1 - w) + (REAL)lut[(i0 + 1) * 4 + c] * w;
  } else {
    int i = (int)(s * (REAL)(n - 1));
    if (i < 0) i = 0;
    if (i > n - 1) i = n - 1;
    for (int c = 0; c < 4; ++c) out[c] = (REAL)lut[i * 4 + c];
  }
}

/* March one domain along o + t dir over [t0, t1). acc holds the partial of
 * this domain; a_front is the alpha already composited in front of it. */
static int64_t march(const or_domain *d, v3 o, v3 dir, REAL t0, REAL t1,
                     const gvr_render_params *p, REAL a_front, REAL acc[4])
{
  const REAL dt = (REAL)p->sample_dist;
  const REAL smin = (REAL)p->scalar_min, smax = (REAL)p->scalar_max;
  const REAL inv_range = smax > smin ? (REAL)1 / (smax - smin) : (REAL)0;
  int64_t count = 0;
  for (int64_t k = 0;; ++k) {
    REAL t = t0 + (REAL)k * dt;
    if (!(t < t1)) break;
    ++count;
    v3 pos = add(o, scl(dir, t));
    int found;
    REAL v = sample_field(d, pos, &found);
    if (!found) continue;
    REAL s = (v - smin) * inv_range;
    if (s < 0) s = 0;
    if (s > 1) s = 1;
    REAL c[4];
    lut_lookup(p->lut_rgba, p->lut_size, p->lut_filter, s, c);
    REAL om = 1 - acc[3];
    REAL wa = om * c[3];
    acc[0] += wa * c[0];
    acc[1] += wa * c[1];
    acc[2] += wa * c[2];
    acc[3] += wa;
    if (p->early_term < 1 && a_front + (1 - a_front) * acc[3] >= (REAL)p->early_term)
      break;
  }
  return count;
}

typedef struct {
  v3 look, ru, rv, origin;
  REAL dx_scale, dy_scale; /* world step per pixel along ru / rv */
  REAL xoff, yoff;         /* pan offsets in pixels */
} or_basis;

static or_basis make_basis(const gvr_camera *c, int W, int H)
{
  or_basis b;
  b.origin = fromf(c->position);
  b.look = normalize(sub(fromf(c->look_at), b.origin));
  v3 up = fromf(c->up);
  b.ru = normalize(cross(b.look, up));
  b.rv = normalize(cross(b.ru, b.look));
  REAL fov_y = (REAL)c->fov_y;
  REAL fov_x = fov_y;
  if (W != H) {
    REAL fovy_rad = fov_y * (REAL)(OR_PI / 180.0);
    REAL vd = (REAL)tan((double)((REAL)0.5 * fovy_rad));
    REAL hd = ((REAL)W / (REAL)H) * vd;
    fov_x = (REAL)2 * (REAL)atan((double)hd) / (REAL)(OR_PI / 180.0);
  }
  REAL thx = (REAL)tan((double)(fov_x * (REAL)(OR_PI / 180.0) * (REAL)0.5));
  REAL thy = (REAL)tan((double)(fov_y * (REAL)(OR_PI / 180.0) * (REAL)0.5));
  b.dx_scale = (REAL)2 * thx / (REAL)W;
  b.dy_scale = (REAL)2 * thy / (REAL)H;
  if (c->zoom > 0) {
    b.dx_scale /= (REAL)c->zoom;
    b.dy_scale /= (REAL)c->zoom;
  }
  b.xoff = (REAL)c->xpan * (REAL)W * (REAL)0.5;
  b.yoff = (REAL)c->ypan * (REAL)H * (REAL)0.5;
  return b;
}

/* column-major-free 4x4 helpers for the projection (row-major M[r][c]) */
static void projview(const gvr_camera *c, int W, int H, double M[4][4])
{
  double e[3] = {c->position[0], c->position[1], c->position[2]};
  double f[3] = {c->look_at[0] - e[0], c->look_at[1] - e[1], c->look_at[2] - e[2]};
  unit(f);
  double u0[3] = {c->up[0], c->up[1], c->up[2]};
  double s[3] = {f[1] * u0[2] - f[2] * u0[1], f[2] * u0[0] - f[0] * u0[2],
                 f[0] * u0[1] - f[1] * u0[0]};
  unit(s);
  double u[3] = {s[1] * f[2] - s[2] * f[1], s[2] * f[0] - s[0] * f[2],
                 s[0] * f[1] - s[1] * f[0]};
  double V[4][4] = {{s[0], s[1], s[2], -(s[0] * e[0] + s[1] * e[1] + s[2] * e[2])},
                    {u[0], u[1], u[2], -(u[0] * e[0] + u[1] * e[1] + u[2] * e[2])},
                    {-f[0], -f[1], -f[2], (f[0] * e[0] + f[1] * e[1] + f[2] * e[2])},
                    {0, 0, 0, 1}};
  double n = c->near_plane, fa = c->far_plane;
  double aspect = (double)W / (double)H;
  double ff = 1.0 / tan(0.5 * (double)c->fov_y * OR_PI / 180.0);
  double z = c->zoom > 0 ? (double)c->zoom : 1.0;
  double P[4][4] = {{ff / aspect * z, 0, 0, 0},
                    {0, ff * z, 0, 0},
                    {0, 0, (fa + n) / (n - fa), 2 * fa * n / (n - fa)},
                    {0, 0, -1, 0}};
  for (int r = 0; r < 4; ++r)
    for (int cc = 0; cc < 4; ++cc) {
      double acc = 0;
      for (int k = 0; k < 4; ++k) acc += P[r][k] * V[k][cc];
      M[r][cc] = acc;
    }
}

/* Image depth of a partial (partials_to_canvas, VolumeRenderer.cpp:287-391).
 * The reference rebuilds the ray with delta_y along ru, not rv
 * (VolumeRenderer.cpp:325); that is kept so that depths match. */
static REAL image_depth(const or_basis *b, const double M[4][4], int W, int H,
                        int i, int j, REAL world_depth)
{
  v3 dx = scl(b->ru, b->dx_scale);
  v3 dy = scl(b->ru, b->dy_scale);
  v3 dir = add(b->look, add(scl(dx, ((REAL)2 * (REAL)i - (REAL)W) / (REAL)2),
                            scl(dy, ((REAL)2 * (REAL)j - (REAL)H) / (REAL)2)));
  dir = normalize(dir);
  v3 pos = add(b->origin, scl(dir, world_depth));
  double pt[4] = {pos.x, pos.y, pos.z, 1.0}, np[4];
  for (int r = 0; r < 4; ++r)
    np[r] = M[r][0] * pt[0] + M[r][1] * pt[1] + M[r][2] * pt[2] + M[r][3] * pt[3];
  return (REAL)(0.5 * (np[2] / np[3]) + 0.49);
}

/* Domain order along a ray: entry distance (stashed in .alpha), then index. */
static int cmp_rpartial(const void *pa, const void *pb)
{
  const or_rpartial *a = (const or_rpartial *)pa, *b = (const or_rpartial *)pb;
  if (a->alpha != b->alpha) return a->alpha < b->alpha ? -1 : 1;
  return a->dom - b->dom;
}

/* Inverse of a row-major 4x4 matrix (Gauss-Jordan, partial pivoting);
 * identity when singular. */
static void invert4(const double M[4][4], double I[4][4])
{
  double a[4][8];
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 8; ++c) a[r][c] = c < 4 ? M[r][c] : (c - 4 == r ? 1.0 : 0.0);
  for (int c = 0; c < 4; ++c) {
    int piv = c;
    for (int r = c + 1; r < 4; ++r)
      if (fabs(a[r][c]) > fabs(a[piv][c])) piv = r;
    if (a[piv][c] == 0.0) {
      for (int r = 0; r < 4; ++r)
        for (int k = 0; k < 4; ++k) I[r][k] = r == k;
      return;
    }
    for (int k = 0; k < 8; ++k) { double t = a[c][k]; a[c][k] = a[piv][k]; a[piv][k] = t; }
    double d = 1.0 / a[c][c];
    for (int k = 0; k < 8; ++k) a[c][k] *= d;
    for (int r = 0; r < 4; ++r) {
      if (r == c) continue;
      double f = a[r][c];
      for (int k = 0; k < 8; ++k) a[r][k] -= f * a[c][k];
    }
  }
  for (int r = 0; r < 4; ++r)
    for (int k = 0; k < 4; ++k) I[r][k] = a[r][k + 4];
}

static int render_rows(const or_scene *s, const gvr_camera *cam, const gvr_render_params *p,
                       int row0, int row1, float *rgba, float *depth, int over,
                       uint64_t *samples_out);

/* Render image rows [row0, row1) of the scene for one camera into full-size
 * buffers (rgba: 4*W*H floats, depth: W*H floats; other rows untouched).
 * *samples_out (if non-NULL) receives the number of samples taken. */
int or_render_rows(const or_scene *s, const gvr_camera *cam, const gvr_render_params *p,
                   int row0, int row1, float *rgba, float *depth, uint64_t *samples_out)
{
  return render_rows(s, cam, p, row0, row1, rgba, depth, 0, samples_out);
}

/* Render over an opaque canvas held in rgba/depth (image depth 0.5 z + 0.5,
 * 1 = empty): every ray ends at the world point its pixel's canvas depth
 * unprojects to (assumption A11: pixel (i, j) at NDC (2i/W - 1, 2j/H - 1,
 * 2d - 1) through the inverse projection * view, the distance from the
 * camera becomes the ray's MaxDistance as in RayOperations::MapCanvasToRays,
 * VolumeRenderer.cpp:243-247), and partials blend over the canvas colour
 * (partials_to_canvas, VolumeRenderer.cpp:366-385). */
int or_render_over(const or_scene *s, const gvr_camera *cam, const gvr_render_params *p,
                   float *rgba, float *depth, uint64_t *samples_out)
{
  return render_rows(s, cam, p, 0, p->height, rgba, depth, 1, samples_out);
}

static int render_rows(const or_scene *s, const gvr_camera *cam, const gvr_render_params *p,
                       int row0, int row1, float *rgba, float *depth, int over,
                       uint64_t *samples_out)
{
  const int W = p->width, H = p->height;
  if (W < 1 || H < 1 || !p->lut_rgba || p->lut_size < 2) return GVR_ERR_INVALID_ARGUMENT;
  if (row0 < 0) row0 = 0;
  if (row1 > H) row1 = H;
  or_basis b = make_basis(cam, W, H);
  double M[4][4], IM[4][4];
  projview(cam, W, H, M);
  invert4(M, IM);
  const int nd = s->n;
  uint64_t total = 0;
#pragma omp parallel for schedule(dynamic, 1) reduction(+ : total)
  for (int j = row0; j < row1; ++j) {
    or_rpartial *parts = (or_rpartial *)malloc(sizeof(or_rpartial) * (nd > 0 ? nd : 1));
    for (int i = 0; i < W; ++i) {
      v3 dir = add(b.look,
                   add(scl(b.ru, b.dx_scale * ((REAL)i - (REAL)W / 2 - b.xoff)),
                       scl(b.rv, b.dy_scale * ((REAL)j - (REAL)H / 2 - b.yoff))));
      dir = normalize(dir);
      /* domain order along this ray: increasing exit distance */
      int np = 0;
      for (int d = 0; d < nd; ++d) {
        REAL t0, t1;
        if (slab(s->d[d].lo, s->d[d].hi, b.origin, dir, &t0, &t1)) {
          parts[np].depth = t1;
          parts[np].dom = d;
          parts[np].alpha = t0; /* stash entry distance */
          ++np;
        }
      }
      qsort(parts, np, sizeof(or_rpartial), cmp_rpartial);
      const int64_t pix = (int64_t)j * W + i;
      REAL cin[4] = {0, 0, 0, 0};
      REAL din = (REAL)p->clear_depth;
      REAL t_max = INFINITY;
      if (over) {
        for (int c = 0; c < 4; ++c) cin[c] = rgba[pix * 4 + c];
        din = depth[pix];
        double q[4] = {2.0 * i / W - 1.0, 2.0 * j / H - 1.0, 2.0 * (double)depth[pix] - 1.0, 1.0}, P[4];
        for (int r = 0; r < 4; ++r)
          P[r] = IM[r][0] * q[0] + IM[r][1] * q[1] + IM[r][2] * q[2] + IM[r][3] * q[3];
        if (P[3] != 0.0) {
          double ex = P[0] / P[3] - b.origin.x, ey = P[1] / P[3] - b.origin.y, ez = P[2] / P[3] - b.origin.z;
          t_max = (REAL)(float)sqrt(ex * ex + ey * ey + ez * ez);
        }
      }
      REAL rgb[3] = {0, 0, 0}, a = 0, front_depth = 0;
      int have = 0;
      REAL covered = -INFINITY;
      for (int k = 0; k < np; ++k) {
        REAL acc[4] = {0, 0, 0, 0};
        REAL t0 = parts[k].alpha, t1 = parts[k].depth;
        /* A7: domains in entry order, each marched from the furthest exit
         * reached so far */
        if (t0 < covered) t0 = covered;
        if (t1 > t_max) t1 = t_max;
        if (t1 > covered) covered = t1;
        if (p->early_term < 1 && a >= (REAL)p->early_term) break;
        total += (uint64_t)march(&s->d[parts[k].dom], b.origin, dir, t0, t1, p, a, acc);
        if (acc[3] < (REAL)p->alpha_cull) continue;
        if (!have) {
          /* the front partial is taken as-is (BlendPartials, :66-67) */
          rgb[0] = acc[0]; rgb[1] = acc[1]; rgb[2] = acc[2]; a = acc[3];
          front_depth = t1;
          have = 1;
        } else {
          blend_partial(rgb, &a, acc, acc[3]);
        }
      }
      REAL out[4] = {cin[0], cin[1], cin[2], cin[3]};
      REAL dep = din;
      if (have) {
        /* composited partial in front of the canvas (a cleared canvas is 0) */
        REAL om = 1 - a;
        out[0] = rgb[0] + cin[0] * om; out[1] = rgb[1] + cin[1] * om;
        out[2] = rgb[2] + cin[2] * om; out[3] = cin[3] * om + a;
        dep = image_depth(&b, M, W, H, i, j, front_depth);
      }
      if (p->quantize_uint8) {
        /* vtkh::Image::Init truncation, then ImageToCanvas x 1/255 */
        for (int c = 0; c < 4; ++c) {
          float f = (float)out[c] * 255.f;
          unsigned char u = (unsigned char)(f < 0 ? 0 : (f > 255.f ? 255.f : f));
          out[c] = (REAL)((float)u * (1.f / 255.f));
        }
        if (dep < 0) dep = -dep;
      }
      if (p->render_bg) {
        REAL om = 1 - out[3];
        for (int c = 0; c < 4; ++c) out[c] += (REAL)p->bg_color[c] * om;
      }
      for (int c = 0; c < 4; ++c) rgba[pix * 4 + c] = (float)out[c];
      depth[pix] = (float)dep;
    }
    free(parts);
  }
  if (samples_out) *samples_out = total;
  return GVR_OK;
}

/* Render the whole image. */
int or_render(const or_scene *s, const gvr_camera *cam, const gvr_render_params *p,
              float *rgba, float *depth, uint64_t *samples_out)
{
  return or_render_rows(s, cam, p, 0, p->height, rgba, depth, samples_out);
}

/* Number of OpenMP threads the render loop uses (1 without OpenMP). */
int or_num_threads(void)
{
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
