// gvr_march.cu — fused structured ray march + partial compositing.
//
// One thread per ray; a warp marches an 8x4-pixel packet and a CTA a 16x16
// tile, so neighbouring lanes read neighbouring bricks. For every pixel the
// kernel does what the reference spreads over several host passes:
//   - per-domain ray setup and march        (StructuredWrapper::render,
//     VolumeRenderer.cpp:223-284; the march itself is VTK-m's
//     VolumeRendererStructured),
//   - partial extraction with the alpha < alpha_cull drop and depth = the
//     ray's exit distance of the domain    (VolumeRenderer.cpp:262-283),
//   - compositing of the partials of all domains in increasing depth with
//     VolumePartial::blend                  (PartialCompositor.cpp:57-90,
//     331-490; VolumePartial.hpp:86-95),
//   - partials_to_canvas: blend over the cleared canvas and image depth
//     0.5 z/w + 0.49                        (VolumeRenderer.cpp:287-391),
//   - the uint8 round trip of the single-domain path (Image.hpp:102-105,
//     Renderer.cpp:265-283) and the background blend.
// Domains are visited in increasing entry distance along each ray, which for
// disjoint boxes is the order the reference's (pixel, exit depth) sort
// produces, so no partial buffer or sort pass is needed.
#include <algorithm>
#include <cfloat>

#include "gvr_hex_device.cuh"

namespace gvr {
namespace {

constexpr int kTile = kMarchTile;  // CTA tile edge in pixels
constexpr int kThreads = 256; // 8 warps, each a 32-ray packet
// Per-ray compositing state kept in shared memory while a domain is marched
// (rgb, front depth, last entry distance, covered exit, last domain, ray
// end, pixel): parked there rather than in registers, the unrolled march
// loop fits 64 registers (4 CTAs per SM) with little or no spilling.
constexpr int kStateSlots = 11;   // the last one: render_ray_unified's sequence position

struct Ray {
  float o[3];
  float d[3];
};

__device__ __forceinline__ bool slab(const DomainDev &dm, const Ray &r, float &t0,
                                     float &t1)
{
  float tmin = 0.f, tmax = FLT_MAX;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (r.d[a] != 0.f) {
      const float inv = 1.f / r.d[a];
      float ta = (dm.lo[a] - r.o[a]) * inv;
      float tb = (dm.hi[a] - r.o[a]) * inv;
      if (ta > tb) { const float t = ta; ta = tb; tb = t; }
      tmin = fmaxf(tmin, ta);
      tmax = fminf(tmax, tb);
    } else if (r.o[a] < dm.lo[a] || r.o[a] > dm.hi[a]) {
      return false;
    }
  }
  t0 = tmin;
  t1 = tmax;
  return tmax > tmin;
}

__device__ __forceinline__ float lerpf(float a, float b, float w)
{
  return fmaf(w, b - a, a);
}

// Nearest LUT entry of a saturated scalar s in [0, 1]: s * (n - 1) <= n - 1
// in float, so (int)(s * nm1) is an index of the table without a clamp
// (the value a clamp to n - 1 would give).
__device__ __forceinline__ float4 lut_nearest(const float4 *lut, float nm1, float s)
{
  return lut[(int)(s * nm1)];
}

__device__ __forceinline__ float4 lut_fetch(const float4 *lut, int n, int filter, float s)
{
  if (filter == GVR_LUT_LINEAR) {
    const float x = s * (float)(n - 1);
    int i0 = min((int)x, n - 2);
    const float w = x - (float)i0;
    const float4 a = lut[i0], b = lut[i0 + 1];
    return make_float4(lerpf(a.x, b.x, w), lerpf(a.y, b.y, w), lerpf(a.z, b.z, w),
                       lerpf(a.w, b.w, w));
  }
  const int i = min((int)(s * (float)(n - 1)), n - 1);
  return lut[i];
}

// Rectilinear axis search: move the cell index until x[i] <= p <= x[i+1].
__device__ __forceinline__ int rect_cell(const float *__restrict__ x, int n, float p, int i)
{
  while (i < n - 2 && p > __ldg(x + i + 1)) ++i;
  while (i > 0 && p < __ldg(x + i)) --i;
  return i;
}

struct Partial {
  float4 acc;   // premultiplied colour and opacity of the domain's partial
  int count;    // samples the stepping rule took
};

// March one structured domain over [t0, t1) from zero opacity: the domain's
// partial and its sample count. Not inlined (the general path: rectilinear
// coordinates, element fields), so that its registers do not weigh on the
// kernels' uniform-grid loop; the ray comes by value and the result goes
// back by value, so nothing is kept in local memory for the call.
__device__ __noinline__ Partial march_domain(const DomainDev &dm, const Ray r, float t0, float t1,
                                             const MarchParams &mp, const float4 *lut, float thr)
{
  const float dt = mp.sample_dist;
  int count = 0;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  const int nx = dm.dims[0], ny = dm.dims[1], nz = dm.dims[2];
  const float gmax[3] = {(float)(nx - 1), (float)(ny - 1), (float)(nz - 1)};
  // grid coordinates g = A + t B (uniform)
  float A[3], B[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
    B[a] = r.d[a] * dm.inv_spacing[a];
  }
  int rc[3] = {0, 0, 0};  // rectilinear cell indices carried along the ray
  if (dm.kind == GVR_DOMAIN_RECTILINEAR) {
    // first-sample binary search per axis
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float p = fmaf(t0, r.d[a], r.o[a]);
      int lo = 0, hi = dm.dims[a] - 1;
      while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(dm.coord[a] + mid) <= p) lo = mid; else hi = mid;
      }
      rc[a] = min(lo, dm.dims[a] - 2);
    }
  }
  const int nbx = dm.nbrick[0], nby = dm.nbrick[1];
  const int bsh = dm.bshift, bc = brick_cells(bsh), bn = brick_nodes(bsh), bf = brick_floats(bsh);
  const float inv_dt = 1.f / dt;
  for (int k = 0;; ++k) {
    const float t = fmaf((float)k, dt, t0);
    if (!(t < t1)) break;
    ++count;
    int c[3];
    float w[3];
    if (dm.kind == GVR_DOMAIN_UNIFORM) {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float g = fminf(fmaxf(fmaf(t, B[a], A[a]), 0.f), gmax[a]);
        c[a] = min((int)g, dm.dims[a] - 2);
        w[a] = g - (float)c[a];
      }
    } else {
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        const float p = fmaf(t, r.d[a], r.o[a]);
        rc[a] = rect_cell(dm.coord[a], dm.dims[a], p, rc[a]);
        const float x0 = __ldg(dm.coord[a] + rc[a]);
        const float x1 = __ldg(dm.coord[a] + rc[a] + 1);
        c[a] = rc[a];
        w[a] = __saturatef((p - x0) / (x1 - x0));
      }
    }
    float v;
    if (dm.assoc == GVR_ASSOC_ELEMENT) {
      v = __ldg(dm.cells + ((int64_t)c[2] * (ny - 1) + c[1]) * (nx - 1) + c[0]);
    } else {
      const int bx = c[0] >> bsh, by = c[1] >> bsh, bz = c[2] >> bsh;
      const int64_t brick = ((int64_t)bz * nby + by) * nbx + bx;
      if (mp.skip_empty && dm.brick_empty[brick]) {
        // Empty brick: every sample inside it has zero opacity. Jump to the
        // last sample before the brick's exit; those samples still count.
        float texit = t1;
        const int b3[3] = {bx, by, bz};
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          if (dm.kind == GVR_DOMAIN_UNIFORM && B[a] != 0.f) {
            const float edge = B[a] > 0.f ? (float)min((b3[a] + 1) * bc, dm.dims[a] - 1)
                                          : (float)(b3[a] * bc);
            texit = fminf(texit, (edge - A[a]) / B[a]);
          }
        }
        if (dm.kind == GVR_DOMAIN_UNIFORM) {
          const int knew = (int)floorf((texit - t0) * inv_dt);
          if (knew > k + 1) {
            // samples k+1 .. knew-1 are skipped; they satisfy t < texit <= t1
            int skipped = knew - 1 - k;
            count += skipped;
            k = knew - 1;
          }
        }
        continue;
      }
      const int m = bc - 1;
      const float *p = dm.bricks + brick * bf + ((c[2] & m) * bn + (c[1] & m)) * bn + (c[0] & m);
      const float v000 = __ldg(p), v100 = __ldg(p + 1);
      const float v010 = __ldg(p + bn), v110 = __ldg(p + bn + 1);
      const float v001 = __ldg(p + bn * bn);
      const float v101 = __ldg(p + bn * bn + 1);
      const float v011 = __ldg(p + bn * bn + bn);
      const float v111 = __ldg(p + bn * bn + bn + 1);
      const float c00 = lerpf(v000, v100, w[0]);
      const float c10 = lerpf(v010, v110, w[0]);
      const float c01 = lerpf(v001, v101, w[0]);
      const float c11 = lerpf(v011, v111, w[0]);
      const float c0 = lerpf(c00, c10, w[1]);
      const float c1 = lerpf(c01, c11, w[1]);
      v = lerpf(c0, c1, w[2]);
    }
    const float s = __saturatef((v - mp.scalar_min) * mp.inv_range);
    const float4 col = lut_fetch(lut, mp.lut_size, mp.lut_filter, s);
    const float wa = (1.f - acc.w) * col.w;
    acc.x = fmaf(wa, col.x, acc.x);
    acc.y = fmaf(wa, col.y, acc.y);
    acc.z = fmaf(wa, col.z, acc.z);
    acc.w += wa;
    if (acc.w >= thr) break;
  }
  return Partial{acc, count};
}


// Samples k .. k + UNROLL - 1 of a ray in a uniform vertex domain, whose
// grid-space position at distance t is A + t B: each is located, its cell's
// 8 corners are loaded from the bricks unless the sample before was in the
// same cell (lc, last_off hold that cell's), and v[u] is the trilinear
// value. ok[u]: the sample lies before t1 (and, with LIMIT, its index
// before kend); a sample that does not is placed at t0 so that its loads
// stay inside the domain. Shared by the per-domain loops and the one-loop
// domain walk, so all of them take the same samples with the same
// arithmetic.
template <int UNROLL, int SH, bool LIMIT>
__device__ __forceinline__ void sample_cells(const float *__restrict__ bricks, const float A[3],
                                             const float B[3], const int cmax[3], int sy, int sz,
                                             int k, int kend, float dt, float t0, float t1,
                                             int &last_off, float lc[8], float v[UNROLL],
                                             bool ok[UNROLL])
{
  constexpr int BC = brick_cells(SH), BN = brick_nodes(SH), BF = brick_floats(SH);
#pragma unroll
  for (int u = 0; u < UNROLL; ++u) {
    float t = fmaf((float)(k + u), dt, t0);
    ok[u] = LIMIT ? (k + u < kend && t < t1) : t < t1;
    t = ok[u] ? t : t0;
    int off = 0;
    float w[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      const float g = fmaf(t, B[a], A[a]);
      const int c = max(0, min((int)g, cmax[a]));
      w[a] = g - (float)c;
      const int hi = c >> SH, lo = c & (BC - 1);
      off += a == 0 ? hi * BF + lo
                    : (a == 1 ? hi * sy + lo * BN : hi * sz + lo * BN * BN);
    }
    if (off != last_off) {
      const float *p = bricks + off;
      lc[0] = __ldg(p);
      lc[1] = __ldg(p + 1);
      lc[2] = __ldg(p + BN);
      lc[3] = __ldg(p + BN + 1);
      lc[4] = __ldg(p + BN * BN);
      lc[5] = __ldg(p + BN * BN + 1);
      lc[6] = __ldg(p + BN * BN + BN);
      lc[7] = __ldg(p + BN * BN + BN + 1);
      last_off = off;
    }
    const float c00 = lerpf(lc[0], lc[1], w[0]);
    const float c10 = lerpf(lc[2], lc[3], w[0]);
    const float c01 = lerpf(lc[4], lc[5], w[0]);
    const float c11 = lerpf(lc[6], lc[7], w[0]);
    v[u] = lerpf(lerpf(c00, c10, w[1]), lerpf(c01, c11, w[1]), w[2]);
  }
}

// Uniform grid, vertex field, no empty bricks: the hot path. UNROLL samples
// are located and their 8 corners loaded before any of them is blended, so
// a warp keeps UNROLL x 8 loads in flight. A sample in the cell of the one
// before it reuses that cell's corners from registers (the same values, so
// the result does not change). Blending stays sequential and stops exactly
// where the one-sample loop stops.
template <int UNROLL, int SH>
__device__ __forceinline__ int march_uniform(const DomainDev &dm, const Ray &r, float t0,
                                             float t1, const MarchParams &mp,
                                             const float4 *lut, float thr, float4 &acc)
{
  const float dt = mp.sample_dist;
  float A[3], B[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
    B[a] = r.d[a] * dm.inv_spacing[a];
  }
  const int cmax[3] = {dm.dims[0] - 2, dm.dims[1] - 2, dm.dims[2] - 2};
  constexpr int BC = brick_cells(SH), BN = brick_nodes(SH), BF = brick_floats(SH);
  const int sy = dm.nbrick[0] * BF;
  const int sz = dm.nbrick[1] * sy;
  const float *__restrict__ bricks = dm.bricks;
  const float nm1 = (float)(mp.lut_size - 1);
  // corners of the last cell loaded (at half-cell spacing about half of the
  // samples fall in the cell of the sample before)
  int last_off = -1;
  float lc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  // samples taken: k + u when sample k + u lies past t1, k + u + 1 when it
  // reached the threshold (no counter in the loop)
  for (int k = 0;; k += UNROLL) {
    float v[UNROLL];
    bool ok[UNROLL];
    sample_cells<UNROLL, SH, false>(bricks, A, B, cmax, sy, sz, k, 0, dt, t0, t1, last_off, lc, v, ok);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      if (!ok[u]) return k + u;
      const float s = __saturatef((v[u] - mp.scalar_min) * mp.inv_range);
      float4 col;
      if (mp.lut_filter == GVR_LUT_LINEAR) {
        col = lut_fetch(lut, mp.lut_size, GVR_LUT_LINEAR, s);
      } else {
        col = lut_nearest(lut, nm1, s);
      }
      const float wa = (1.f - acc.w) * col.w;
      acc.x = fmaf(wa, col.x, acc.x);
      acc.y = fmaf(wa, col.y, acc.y);
      acc.z = fmaf(wa, col.z, acc.z);
      acc.w += wa;
      if (acc.w >= thr) return k + u + 1;
    }
  }
}

// Uniform grid, vertex field, with empty bricks: the march walks the ray
// brick by brick. Entering a brick it computes the last sample before the
// brick's exit (a whole step inside it); an empty brick's samples up to
// there are counted and jumped over (they would blend with zero opacity),
// and a non-empty brick's samples up to its exit run through the same
// unrolled, corner-reusing loop as march_uniform. Compared with a test per
// sample, the emptiness test and the exit distance are paid once per brick.
template <int UNROLL, int SH>
__device__ __forceinline__ int march_bricks(const DomainDev &dm, const Ray &r, float t0,
                                         float t1, const MarchParams &mp,
                                         const float4 *lut, float thr, float4 &acc)
{
  const float dt = mp.sample_dist;
  float A[3], B[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
    B[a] = r.d[a] * dm.inv_spacing[a];
  }
  const int cmax[3] = {dm.dims[0] - 2, dm.dims[1] - 2, dm.dims[2] - 2};
  constexpr int BC = brick_cells(SH), BN = brick_nodes(SH), BF = brick_floats(SH);
  const int sy = dm.nbrick[0] * BF;
  const int sz = dm.nbrick[1] * sy;
  const float *__restrict__ bricks = dm.bricks;
  const float nm1 = (float)(mp.lut_size - 1);
  int count = 0;
  int last_off = -1;
  float lc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  int k = 0;
  for (;;) {
    const float t = fmaf((float)k, dt, t0);
    if (!(t < t1)) return count;
    int b[3];
    float texit = t1;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      b[a] = max(0, min((int)fmaf(t, B[a], A[a]), cmax[a])) >> SH;
      if (B[a] != 0.f) {
        const float edge = B[a] > 0.f ? (float)min((b[a] + 1) * BC, cmax[a] + 1)
                                      : (float)(b[a] * BC);
        texit = fminf(texit, (edge - A[a]) / B[a]);
      }
    }
    // samples k .. kx - 1 lie at least one step before the exit
    const int kx = (int)floorf((texit - t0) / dt);
    if (dm.brick_empty[(b[2] * dm.nbrick[1] + b[1]) * dm.nbrick[0] + b[0]]) {
      const int kn = max(kx, k + 1);  // sample k itself is in the empty brick
      count += kn - k;
      k = kn;
      continue;
    }
    const int kend = max(kx + 1, k + 1);
    for (; k < kend; k += UNROLL) {
      float v[UNROLL];
      bool ok[UNROLL];
      sample_cells<UNROLL, SH, true>(bricks, A, B, cmax, sy, sz, k, kend, dt, t0, t1, last_off, lc, v, ok);
#pragma unroll
      for (int u = 0; u < UNROLL; ++u) {
        if (!ok[u]) break;
        ++count;
        const float sc = __saturatef((v[u] - mp.scalar_min) * mp.inv_range);
        float4 col;
        if (mp.lut_filter == GVR_LUT_LINEAR) {
          col = lut_fetch(lut, mp.lut_size, GVR_LUT_LINEAR, sc);
        } else {
          col = lut_nearest(lut, nm1, sc);
        }
        const float wa = (1.f - acc.w) * col.w;
        acc.x = fmaf(wa, col.x, acc.x);
        acc.y = fmaf(wa, col.y, acc.y);
        acc.z = fmaf(wa, col.z, acc.z);
        acc.w += wa;
        if (acc.w >= thr) return count;
      }
    }
    k = kend;
  }
}

// Hexahedral domain: each sample is located by Newton's method in the cell
// of the previous sample (starting from its reference coordinates moved by
// the last Jacobian's image of the ray step); when the
// solution lies outside that cell, the march steps to the face neighbour it
// left through (up to kHexHops cells), and only when that fails walks the
// LBVH. The eight corner records of the current cell stay in registers
// between samples. Samples outside every
// cell contribute nothing but are counted, like the structured stepping rule.
__device__ int march_hex(const DomainDev &dm, const Ray &r, float t0, float t1,
                         const MarchParams &mp, const float4 *lut, float thr, float4 &acc)
{
  HexGeom v;
  int cur = -1;
  float rst[3] = {0.5f, 0.5f, 0.5f};
  // change of rst from one sample to the next (J^-1 times the ray step,
  // from the last Newton solve): the next sample's guess
  float drst[3] = {0.f, 0.f, 0.f};
  const float step[3] = {r.d[0] * mp.sample_dist, r.d[1] * mp.sample_dist, r.d[2] * mp.sample_dist};
  int count = 0;
  for (int k = 0;; ++k) {
    const float t = fmaf((float)k, mp.sample_dist, t0);
    if (!(t < t1)) break;
    ++count;
    const float p[3] = {fmaf(t, r.d[0], r.o[0]), fmaf(t, r.d[1], r.o[1]), fmaf(t, r.d[2], r.o[2])};
    bool found = false;
    if (cur >= 0) {
      float g[3] = {rst[0] + drst[0], rst[1] + drst[1], rst[2] + drst[2]};
      // Predicted exit: the extrapolated guess is clearly outside the cell,
      // so step to the face neighbour before solving (a cheap divergent
      // branch: eight loads) and let every lane do its one solve together;
      // solving in the old cell first and then in the neighbour costs the
      // warp two solves per step (19.5 vs 14.1 Gsamples/s on a jittered
      // 200^3 mesh). Mispredictions fall through to the stepping below.
      if (dm.hex_nbr && !(g[0] > -kHexPredictMargin && g[0] < 1.f + kHexPredictMargin &&
                          g[1] > -kHexPredictMargin && g[1] < 1.f + kHexPredictMargin &&
                          g[2] > -kHexPredictMargin && g[2] < 1.f + kHexPredictMargin)) {
        const int face = hex_exit_face(g);
        const int nb = __ldg(dm.hex_nbr + 6 * (int64_t)cur + face);
        if (nb >= 0) {
          cur = nb;
          hex_load(dm, cur, v);
          g[face >> 1] += (face & 1) ? -1.f : 1.f;
        }
      }
      int st = hex_newton_status(v, p, g, step, drst, true);
      // left the cell: step to the neighbour across the face it left
      // through (Newton's outside solution names it), a few times at most
      for (int hop = 0; st == 0 && hop < kHexHops && dm.hex_nbr; ++hop) {
        const int face = hex_exit_face(g);
        const int nb = __ldg(dm.hex_nbr + 6 * (int64_t)cur + face);
        if (nb < 0) break;
        cur = nb;
        hex_load(dm, cur, v);
        // guess: the point's coordinates across a like-oriented face
        g[face >> 1] += (face & 1) ? -1.f : 1.f;
        g[0] = __saturatef(g[0]);
        g[1] = __saturatef(g[1]);
        g[2] = __saturatef(g[2]);
        st = hex_newton_status(v, p, g, step, drst, true);
      }
      if (st == 1) {
        found = true;
        rst[0] = g[0]; rst[1] = g[1]; rst[2] = g[2];
      }
    }
    if (!found) {
      cur = hex_locate(dm, p, rst, v);
      found = cur >= 0;
      drst[0] = drst[1] = drst[2] = 0.f;
    }
    if (!found) continue;
    float val;
    if (dm.assoc == GVR_ASSOC_ELEMENT) {
      val = __ldg(dm.cells + cur);
    } else {
      val = hex_value(dm, cur, __saturatef(rst[0]), __saturatef(rst[1]), __saturatef(rst[2]));
    }
    const float s = __saturatef((val - mp.scalar_min) * mp.inv_range);
    const float4 col = lut_fetch(lut, mp.lut_size, mp.lut_filter, s);
    const float wa = (1.f - acc.w) * col.w;
    acc.x = fmaf(wa, col.x, acc.x);
    acc.y = fmaf(wa, col.y, acc.y);
    acc.z = fmaf(wa, col.z, acc.z);
    acc.w += wa;
    if (acc.w >= thr) break;
  }
  return count;
}

// Everything one ray does: march the candidate domains (bits of `mask`) in
// increasing exit distance, blend their partials, and finish the pixel
// (image depth, uint8 round trip, background). Returns the samples taken.
// g_state: the CTA's shared-memory slots for the state that must survive
// the march of a domain (kStateSlots words per thread, slot k of thread i
// at g_state[k * kThreads + i]).
// The ray of pixel (px, py): the pinhole model partials_to_canvas inverts
// (VolumeRenderer.cpp:335-344).
__device__ __forceinline__ Ray pixel_ray(const ViewDev &view, const MarchParams &mp, int px, int py)
{
  Ray r;
  const float fx = view.dx_scale * ((float)px - 0.5f * (float)mp.width - view.xoff);
  const float fy = view.dy_scale * ((float)py - 0.5f * (float)mp.height - view.yoff);
  float d[3], dn = 0.f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    d[a] = view.look[a] + view.ru[a] * fx + view.rv[a] * fy;
    dn = fmaf(d[a], d[a], dn);
  }
  const float inv = rsqrtf(dn);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r.o[a] = view.origin[a];
    r.d[a] = d[a] * inv;
  }
  return r;
}

// Opaque canvas: the ray ends at the world point of the canvas depth
// (MapCanvasToRays: pixel (i, j) at depth d unprojected from NDC
// (2i/W - 1, 2j/H - 1, 2d - 1); FP64, as in the oracle). FLT_MAX without a
// canvas.
__device__ __forceinline__ float canvas_ray_end(const ViewDev &view, const MarchParams &mp, int px,
                                                int py)
{
  float t_max = FLT_MAX;
  if (mp.canvas_depth) {
    const int64_t pix = (int64_t)py * mp.width + px;
    const float din = mp.canvas_depth[pix];
    const double xn = 2.0 * px / mp.width - 1.0, yn = 2.0 * py / mp.height - 1.0;
    const double zn = 2.0 * (double)din - 1.0;
    const double *I = view.inv_projview;
    double P[4];
#pragma unroll
    for (int q = 0; q < 4; ++q) P[q] = I[4 * q] * xn + I[4 * q + 1] * yn + I[4 * q + 2] * zn + I[4 * q + 3];
    if (P[3] != 0.0) {
      const double ex = P[0] / P[3] - view.origin[0], ey = P[1] / P[3] - view.origin[1],
                   ez = P[2] / P[3] - view.origin[2];
      t_max = (float)sqrt(ex * ex + ey * ey + ez * ez);
    }
  }
  return t_max;
}

// The pixel's final value from its composited partial (have = whether any
// partial survived the cull): partials_to_canvas over the cleared or opaque
// canvas with the image depth, then the uint8 round trip and background.
__device__ __forceinline__ void finish_pixel(const ViewDev &view, const MarchParams &mp, int px, int py,
                                             bool have, const float crgb[3], float ca, float cdepth,
                                             float4 &out, float &dep)
{
  float4 cin = make_float4(0.f, 0.f, 0.f, 0.f);
  float din = mp.clear_depth;
  if (mp.canvas_depth) {
    const int64_t pix = (int64_t)py * mp.width + px;
    cin = mp.canvas_rgba[pix];
    din = mp.canvas_depth[pix];
  }
  out = cin;
  dep = din;
  if (have) {
    const float om = 1.f - ca;
    out = make_float4(crgb[0] + cin.x * om, crgb[1] + cin.y * om, crgb[2] + cin.z * om,
                      cin.w * om + ca);
    // partials_to_canvas ray rebuild: delta_y runs along ru there
    const float ex = view.dx_scale * (float)(2 * px - mp.width) * 0.5f;
    const float ey = view.dy_scale * (float)(2 * py - mp.height) * 0.5f;
    float q[3], qn = 0.f;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      q[a] = view.look[a] + view.ru[a] * ex + view.ru[a] * ey;
      qn = fmaf(q[a], q[a], qn);
    }
    const float qi = rsqrtf(qn);
    float pos[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) pos[a] = fmaf(cdepth, q[a] * qi, view.origin[a]);
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
}

// render_ray for scenes whose domains (at most kUnifiedDomains) are all
// uniform vertex fields with no empty bricks to jump, bricked alike: one
// loop walks the samples of every domain the ray crosses. A lane that
// reaches the end of a domain (or its opacity threshold) blends that
// domain's partial and sets up the next domain inside the same loop, while
// the other lanes of its warp go on sampling; in the per-domain form a
// lane that left its domain first waits at the end of the domain's loop
// until the last lane of the warp leaves it. The domain order, the sample
// positions, the per-domain accumulation and the blend are render_ray's
// and march_uniform's, operation for operation, so images are identical.
constexpr int kUnifiedDomains = 16;

template <int UNROLL, int SH>
__device__ __forceinline__ int render_ray_unified(const DomainDev *doms, uint64_t mask, const ViewDev &view,
                                                  const MarchParams &mp, const float4 *lut, int px, int py,
                                                  float4 &out, float &dep, float *g_state)
{
  int count = 0;
  const Ray r = pixel_ray(view, mp, px, py);
  float *st = g_state + threadIdx.x;
  st[7 * kThreads] = canvas_ray_end(view, mp, px, py);
  st[8 * kThreads] = __int_as_float(px);
  st[9 * kThreads] = __int_as_float(py);
  st[0 * kThreads] = 0.f;          // composited rgb
  st[1 * kThreads] = 0.f;
  st[2 * kThreads] = 0.f;
  st[3 * kThreads] = 0.f;          // depth of the front partial
  st[5 * kThreads] = -FLT_MAX;     // furthest exit covered
  // the ray's domains in render_ray's order, (entry distance, index)
  // ascending, 4 bits each; kept in two state slots with the next position
  {
    uint64_t seq = 0;
    int nseq = 0;
    float last_t0 = -FLT_MAX;
    int last_d = -1;
    for (;;) {
      int best = -1;
      float bt0 = FLT_MAX;
      for (uint64_t m = mask; m; m &= m - 1) {
        const int dd = __ffsll((long long)m) - 1;
        float t0, t1;
        if (!slab(doms[dd], r, t0, t1)) continue;
        const bool after = t0 > last_t0 || (t0 == last_t0 && dd > last_d);
        const bool before = best < 0 || t0 < bt0;
        if (after && before) { best = dd; bt0 = t0; }
      }
      if (best < 0) break;
      seq |= (uint64_t)best << (4 * nseq);
      ++nseq;
      last_t0 = bt0;
      last_d = best;
    }
    st[4 * kThreads] = __int_as_float((int)(uint32_t)seq);
    st[6 * kThreads] = __int_as_float((int)(uint32_t)(seq >> 32));
    st[5 * kThreads] = -FLT_MAX;
    // next position in the sequence (low 8 bits) and its length (next 8)
    st[10 * kThreads] = __int_as_float(nseq << 8);
  }
  float ca = 0.f;
  bool have = false;
  bool fresh = true;      // the next iteration starts a domain
  bool started = false;   // a domain has been marched (its partial is pending)
  const float dt = mp.sample_dist;
  const float nm1 = (float)(mp.lut_size - 1);
  constexpr int BC = brick_cells(SH), BN = brick_nodes(SH), BF = brick_floats(SH);
  float A[3] = {0.f, 0.f, 0.f}, B[3] = {0.f, 0.f, 0.f};
  int cmax[3] = {0, 0, 0};
  int sy = 0, sz = 0;
  const float *__restrict__ bricks = nullptr;
  float bt0 = 0.f, bt1 = 0.f, thr = 2.f;
  float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
  int k = 0;
  int last_off = -1;
  float lc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  for (;;) {
    if (fresh) {
      if (started && !(acc.w < mp.alpha_cull)) {
        if (!have) {
          st[0 * kThreads] = acc.x; st[1 * kThreads] = acc.y; st[2 * kThreads] = acc.z;
          ca = acc.w;
          st[3 * kThreads] = bt1;
          have = true;
        } else if (ca < 1.f && acc.w != 0.f) {
          const float op = 1.f - ca;
          st[0 * kThreads] = fmaf(op, acc.x, st[0 * kThreads]);
          st[1 * kThreads] = fmaf(op, acc.y, st[1 * kThreads]);
          st[2 * kThreads] = fmaf(op, acc.z, st[2 * kThreads]);
          ca = fminf(fmaf(op, acc.w, ca), 1.f);
        }
      }
      if (ca >= mp.early_term) break;
      const int pos = __float_as_int(st[10 * kThreads]);
      const int next = pos & 255, nseq = pos >> 8;
      if (next >= nseq) break;
      st[10 * kThreads] = __int_as_float(pos + 1);
      const uint32_t word = (uint32_t)__float_as_int(st[(next < 8 ? 4 : 6) * kThreads]);
      const int d = (int)((word >> (4 * (next & 7))) & 15u);
      const DomainDev &dm = doms[d];
      float t0, t1;
      slab(dm, r, t0, t1);
      const float covered = st[5 * kThreads];
      bt0 = fmaxf(t0, covered);
      bt1 = fminf(t1, st[7 * kThreads]);
      st[5 * kThreads] = fmaxf(covered, bt1);
      thr = mp.early_term < 1.f ? (mp.early_term - ca) / (1.f - ca) : 2.f;
      acc = make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
        B[a] = r.d[a] * dm.inv_spacing[a];
        cmax[a] = dm.dims[a] - 2;
      }
      sy = dm.nbrick[0] * BF;
      sz = dm.nbrick[1] * sy;
      bricks = dm.bricks;
      k = 0;
      last_off = -1;
      started = true;
      fresh = false;
    }
    float v[UNROLL];
    bool ok[UNROLL];
    sample_cells<UNROLL, SH, false>(bricks, A, B, cmax, sy, sz, k, 0, dt, bt0, bt1, last_off, lc, v, ok);
#pragma unroll
    for (int u = 0; u < UNROLL; ++u) {
      if (!ok[u]) { count += k + u; fresh = true; break; }
      const float sc = __saturatef((v[u] - mp.scalar_min) * mp.inv_range);
      float4 col;
      if (mp.lut_filter == GVR_LUT_LINEAR) {
        col = lut_fetch(lut, mp.lut_size, GVR_LUT_LINEAR, sc);
      } else {
        col = lut_nearest(lut, nm1, sc);
      }
      const float wa = (1.f - acc.w) * col.w;
      acc.x = fmaf(wa, col.x, acc.x);
      acc.y = fmaf(wa, col.y, acc.y);
      acc.z = fmaf(wa, col.z, acc.z);
      acc.w += wa;
      if (acc.w >= thr) { count += k + u + 1; fresh = true; break; }
    }
    k += UNROLL;
  }
  const float crgb[3] = {st[0], st[kThreads], st[2 * kThreads]};
  const float cdepth = st[3 * kThreads];
  px = __float_as_int(st[8 * kThreads]);
  py = __float_as_int(st[9 * kThreads]);
  finish_pixel(view, mp, px, py, have, crgb, ca, cdepth, out, dep);
  return count;
}

template <int UNROLL, bool HEX>
__device__ __forceinline__ int render_ray(const DomainDev *doms, uint64_t mask, const ViewDev &view,
                                          const MarchParams &mp, const float4 *lut, int px, int py,
                                          float4 &out, float &dep, float *g_state)
{
  if (!HEX && (mask & (mask - 1)) != 0 && mp.n_domains <= kUnifiedDomains) {
    // two or more domains, every one a uniform vertex field in 8^3-cell
    // bricks with no empty bricks to jump: the one-loop walk (a single
    // domain has no crossing to wait at, and its own loop keeps fewer
    // values live: 1.39 against 1.49 ms on the 513^3 field as one domain)
    bool uni = true;
    for (uint64_t m = mask; m; m &= m - 1) {
      const DomainDev &dm = doms[__ffsll((long long)m) - 1];
      uni = uni && dm.kind == GVR_DOMAIN_UNIFORM && dm.assoc == GVR_ASSOC_VERTEX && dm.bshift == 3 &&
            !(mp.skip_empty && *dm.any_empty);
    }
    if (uni) return render_ray_unified<UNROLL, 3>(doms, mask, view, mp, lut, px, py, out, dep, g_state);
  }
  int count = 0;
  const Ray r = pixel_ray(view, mp, px, py);
  const float t_max = canvas_ray_end(view, mp, px, py);

  // Compositing state that lives across the march of a domain is parked in
  // shared memory (one word per thread per slot, st[k * kThreads]), so the
  // march loop gets the registers.
  float *st = g_state + threadIdx.x;
  st[7 * kThreads] = t_max;
  st[8 * kThreads] = __int_as_float(px);
  st[9 * kThreads] = __int_as_float(py);
  st[0 * kThreads] = 0.f;          // composited rgb
  st[1 * kThreads] = 0.f;
  st[2 * kThreads] = 0.f;
  st[3 * kThreads] = 0.f;          // depth of the front partial
  st[4 * kThreads] = -FLT_MAX;     // entry distance of the last domain
  st[5 * kThreads] = -FLT_MAX;     // furthest exit covered
  st[6 * kThreads] = __int_as_float(-1);  // last domain
  float ca = 0.f;
  bool have = false;
  for (;;) {
    if (ca >= mp.early_term) break;
    // Next domain along the ray by (entry distance, index). Domains tile
    // space without overlapping, so each is marched from the furthest exit
    // reached so far: every point of the ray is covered once, also where
    // rounding makes neighbouring intervals overlap (rays lying in a shared
    // face). For disjoint boxes this is the order of the reference's
    // (pixel, depth = exit distance) sort.
    int best = -1;
    float bt0 = FLT_MAX, bt1 = 0.f;
    {
      const float last_t0 = st[4 * kThreads];
      const int last_d = __float_as_int(st[6 * kThreads]);
      for (uint64_t m = mask; m; m &= m - 1) {
        const int dd = __ffsll((long long)m) - 1;
        float t0, t1;
        if (!slab(doms[dd], r, t0, t1)) continue;
        const bool after = t0 > last_t0 || (t0 == last_t0 && dd > last_d);
        const bool before = best < 0 || t0 < bt0;
        if (after && before) { best = dd; bt0 = t0; bt1 = t1; }
      }
    }
    if (best < 0) break;
    st[4 * kThreads] = bt0;
    st[6 * kThreads] = __int_as_float(best);
    {
      const float covered = st[5 * kThreads];
      bt0 = fmaxf(bt0, covered);
      bt1 = fminf(bt1, st[7 * kThreads]);
      st[5 * kThreads] = fmaxf(covered, bt1);
    }
    const float thr = mp.early_term < 1.f ? (mp.early_term - ca) / (1.f - ca) : 2.f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    const DomainDev &dm = doms[best];
    if (HEX && dm.kind == GVR_DOMAIN_HEX)
      count += march_hex(dm, r, bt0, bt1, mp, lut, thr, acc);
    else if (dm.kind == GVR_DOMAIN_UNIFORM && dm.assoc == GVR_ASSOC_VERTEX &&
             !(mp.skip_empty && *dm.any_empty))
      count += dm.bshift == 3 ? march_uniform<UNROLL, 3>(dm, r, bt0, bt1, mp, lut, thr, acc)
             : dm.bshift == 2 ? march_uniform<UNROLL, 2>(dm, r, bt0, bt1, mp, lut, thr, acc)
                              : march_uniform<UNROLL, 4>(dm, r, bt0, bt1, mp, lut, thr, acc);
    else if (dm.kind == GVR_DOMAIN_UNIFORM && dm.assoc == GVR_ASSOC_VERTEX)
      count += dm.bshift == 3 ? march_bricks<UNROLL, 3>(dm, r, bt0, bt1, mp, lut, thr, acc)
             : dm.bshift == 2 ? march_bricks<UNROLL, 2>(dm, r, bt0, bt1, mp, lut, thr, acc)
                              : march_bricks<UNROLL, 4>(dm, r, bt0, bt1, mp, lut, thr, acc);
    else {
      const Partial part = march_domain(dm, r, bt0, bt1, mp, lut, thr);
      acc = part.acc;
      count += part.count;
    }
    if (acc.w < mp.alpha_cull) continue;
    if (!have) {
      st[0 * kThreads] = acc.x; st[1 * kThreads] = acc.y; st[2 * kThreads] = acc.z;
      ca = acc.w;
      st[3 * kThreads] = bt1;
      have = true;
    } else if (ca < 1.f && acc.w != 0.f) {
      const float op = 1.f - ca;
      st[0 * kThreads] = fmaf(op, acc.x, st[0 * kThreads]);
      st[1 * kThreads] = fmaf(op, acc.y, st[1 * kThreads]);
      st[2 * kThreads] = fmaf(op, acc.z, st[2 * kThreads]);
      ca = fminf(fmaf(op, acc.w, ca), 1.f);
    }
  }
  const float crgb[3] = {st[0], st[kThreads], st[2 * kThreads]};
  const float cdepth = st[3 * kThreads];
  px = __float_as_int(st[8 * kThreads]);
  py = __float_as_int(st[9 * kThreads]);

  finish_pixel(view, mp, px, py, have, crgb, ca, cdepth, out, dep);
  return count;
}

// PW x (32 / PW) pixel packet per warp, 16 x 16 pixels per CTA.
template <int PW, int UNROLL, int MINB, bool HEX = false>
__global__ void __launch_bounds__(kThreads, MINB)
march_kernel(const DomainDev *__restrict__ g_domains, const __grid_constant__ ViewDev view,
             const __grid_constant__ MarchParams mp, const float4 *__restrict__ g_lut,
             float4 *__restrict__ rgba, float *__restrict__ depth,
             unsigned long long *__restrict__ samples, const int *__restrict__ order)
{
  constexpr int PH = 32 / PW;
  constexpr int PX = kTile / PW;  // packets per tile row
  const int tiles_x = (mp.width + kTile - 1) / kTile;
  const int tile = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  const int tile_x = tile % tiles_x, tile_y = tile / tiles_x;
  extern __shared__ float4 smem[];
  __shared__ float s_state[kStateSlots * kThreads];
  float4 *lut = smem;
  DomainDev *doms = reinterpret_cast<DomainDev *>(smem + mp.lut_size);
  for (int i = threadIdx.x; i < mp.lut_size; i += kThreads) lut[i] = g_lut[i];
  {
    const int words = mp.n_domains * (int)(sizeof(DomainDev) / 4);
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g_domains);
    uint32_t *dst = reinterpret_cast<uint32_t *>(doms);
    for (int i = threadIdx.x; i < words; i += kThreads) dst[i] = src[i];
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = tile_x * kTile + (warp % PX) * PW + (lane % PW);
  const int py = tile_y * kTile + (warp / PX) * PH + (lane / PW);
  const bool valid = px < mp.width && py < mp.height;
  int count = 0;
  if (valid) {
    const uint64_t all = mp.n_domains >= 64 ? ~0ull : ((1ull << mp.n_domains) - 1ull);
    float4 out;
    float dep;
    count = render_ray<UNROLL, HEX>(doms, all, view, mp, lut, px, py, out, dep, s_state);
    const int64_t pix = (int64_t)py * mp.width + px;
    rgba[pix] = out;
    depth[pix] = dep;
  }
  if (samples) {
    unsigned long long c = (unsigned long long)count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(samples, c);
  }
}


// ---------------------------------------------------------------------------
// Shared-memory staged march (uniform grids, vertex fields).
//
// The CTA's 256 rays form a thin frustum (its 16 x 16 tile). The kernel walks
// the frustum in slabs of ray distance [T, T + dT): for each slab it lists
// the bricks of the current domain that the frustum crosses there (a plane
// test of every brick in the slab's bounding box against the frustum's four
// side planes and its near and far planes), copies them into shared memory
// with one bulk copy each (cp.async.bulk, 2944 contiguous bytes, completing
// on an mbarrier with a bounded wait), and then every ray takes its samples
// of the slab from shared memory. dT is the deepest of {8, 4, 2, 1, 1/2, 1/4}
// brick edges whose box of candidate bricks fits the map and whose frustum
// bricks fit the kStageSlots slots. Bricks whose LUT opacity is zero over
// their range are not copied: their samples are counted and skipped, as the
// brick-walking march does. A brick the plan did not stage (frustum test
// rounding, slots full) is read from global memory, so the plan never
// changes a pixel.
//
// Domains are taken in one front-to-back order for the whole CTA (computed on
// the host per view from the planes that separate the domains' boxes, see
// staged_order in gvr_api.cpp). For boxes that do not overlap, every ray that
// crosses two of them crosses them in that order, so each ray composites its
// partials in the order the per-ray walk of render_ray would choose, with the
// same per-sample arithmetic: the images are bit-identical to march_kernel's.
// ---------------------------------------------------------------------------
constexpr int kStageSlots = 24;           // staged bricks per slab (24 x 2944 B = 69 KB)
constexpr int kStageMap = 1024;           // bricks in a slab's candidate box
constexpr long long kStagePolls = 1ll << 20;  // bounded mbarrier wait (polls)

__device__ __forceinline__ unsigned smem_addr(const void *p)
{
  return static_cast<unsigned>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool stage_wait(const uint64_t *bar, unsigned phase, long long polls)
{
  for (long long i = 0; i < polls; ++i) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_addr(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
    if (i > 32) __nanosleep(32);
  }
  return false;
}

// Frustum of a tile: ray origin, unit centre direction, the cosine of the
// widest corner ray against it, and four inward side-plane normals through
// the origin (corner rays at the tile's outer pixel edges).
struct Frustum {
  float o[3];
  float c[3];
  float cos_min;
  float n[4][3];
  float dn[4][3];   // unit corner directions
};

__device__ void tile_frustum(const ViewDev &view, const MarchParams &mp, int x0, int y0, Frustum &f)
{
  auto dir = [&](float x, float y, float d[3]) {
    const float fx = view.dx_scale * (x - 0.5f * (float)mp.width - view.xoff);
    const float fy = view.dy_scale * (y - 0.5f * (float)mp.height - view.yoff);
    float n2 = 0.f;
    for (int a = 0; a < 3; ++a) {
      d[a] = view.look[a] + view.ru[a] * fx + view.rv[a] * fy;
      n2 += d[a] * d[a];
    }
    const float inv = rsqrtf(n2);
    for (int a = 0; a < 3; ++a) d[a] *= inv;
  };
  const float xa = (float)x0 - 0.5f, xb = (float)(x0 + kTile - 1) + 0.5f;
  const float ya = (float)y0 - 0.5f, yb = (float)(y0 + kTile - 1) + 0.5f;
  dir(xa, ya, f.dn[0]);
  dir(xb, ya, f.dn[1]);
  dir(xb, yb, f.dn[2]);
  dir(xa, yb, f.dn[3]);
  dir(0.5f * (xa + xb), 0.5f * (ya + yb), f.c);
  for (int a = 0; a < 3; ++a) f.o[a] = view.origin[a];
  f.cos_min = 1.f;
  for (int i = 0; i < 4; ++i) {
    const float *u = f.dn[i], *v = f.dn[(i + 1) & 3];
    float nn[3] = {u[1] * v[2] - u[2] * v[1], u[2] * v[0] - u[0] * v[2], u[0] * v[1] - u[1] * v[0]};
    const float side = nn[0] * f.c[0] + nn[1] * f.c[1] + nn[2] * f.c[2];
    for (int a = 0; a < 3; ++a) f.n[i][a] = side < 0.f ? -nn[a] : nn[a];
    f.cos_min = fminf(f.cos_min, u[0] * f.c[0] + u[1] * f.c[1] + u[2] * f.c[2]);
  }
  f.cos_min -= 1e-6f;
}

// Could the frustum's points at ray distance [t0, t1] lie in the box? (No
// false negatives beyond float rounding; a brick wrongly rejected is read
// from global memory.)
__device__ __forceinline__ bool frustum_box(const Frustum &f, float t0, float t1, const float lo[3],
                                            const float hi[3])
{
  for (int i = 0; i < 4; ++i) {
    float m = 0.f;
    for (int a = 0; a < 3; ++a) m += f.n[i][a] * ((f.n[i][a] > 0.f ? hi[a] : lo[a]) - f.o[a]);
    if (m < 0.f) return false;
  }
  float zmax = 0.f, zmin = 0.f;
  for (int a = 0; a < 3; ++a) {
    zmax += f.c[a] * ((f.c[a] > 0.f ? hi[a] : lo[a]) - f.o[a]);
    zmin += f.c[a] * ((f.c[a] > 0.f ? lo[a] : hi[a]) - f.o[a]);
  }
  return zmax >= t0 * f.cos_min && zmin <= t1;
}

template <int PW>
__global__ void __launch_bounds__(kThreads, 2)
staged_kernel(const DomainDev *__restrict__ g_domains, const __grid_constant__ ViewDev view,
              const __grid_constant__ MarchParams mp,
              const float4 *__restrict__ g_lut, float4 *__restrict__ rgba, float *__restrict__ depth,
              unsigned long long *__restrict__ samples, const int *__restrict__ order,
              const StageOrder dorder, unsigned long long *__restrict__ stage_fail)
{
  constexpr int PH = 32 / PW;
  constexpr int PX = kTile / PW;
  const int tiles_x = (mp.width + kTile - 1) / kTile;
  const int tile = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  const int tile_x = tile % tiles_x, tile_y = tile / tiles_x;
  extern __shared__ float4 smem[];
  float4 *lut = smem;
  DomainDev *doms = reinterpret_cast<DomainDev *>(smem + mp.lut_size);
  const size_t head = ((sizeof(float4) * mp.lut_size + sizeof(DomainDev) * mp.n_domains) + 127) & ~(size_t)127;
  float *slots = reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + head);
  __shared__ short s_map[kStageMap];
  __shared__ int s_list[kStageSlots];
  __shared__ __align__(8) uint64_t s_bar;
  __shared__ Frustum s_fr;
  __shared__ int s_box[6];      // first brick and extent of the slab's candidate box
  __shared__ int s_count;       // frustum bricks found (may exceed the slots)
  __shared__ int s_level;       // slab depth level of the plan
  __shared__ float s_t1;        // slab end
  __shared__ unsigned s_tmin;   // next sample distance of the CTA's live rays (bits)

  for (int i = threadIdx.x; i < mp.lut_size; i += kThreads) lut[i] = g_lut[i];
  {
    const int words = mp.n_domains * (int)(sizeof(DomainDev) / 4);
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g_domains);
    uint32_t *dst = reinterpret_cast<uint32_t *>(doms);
    for (int i = threadIdx.x; i < words; i += kThreads) dst[i] = src[i];
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&s_bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    tile_frustum(view, mp, tile_x * kTile, tile_y * kTile, s_fr);
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = tile_x * kTile + (warp % PX) * PW + (lane % PW);
  const int py = tile_y * kTile + (warp / PX) * PH + (lane / PW);
  const bool valid = px < mp.width && py < mp.height;
  const Ray r = pixel_ray(view, mp, valid ? px : 0, valid ? py : 0);
  const float t_max = valid ? canvas_ray_end(view, mp, px, py) : FLT_MAX;
  const float dt = mp.sample_dist;
  const float nm1 = (float)(mp.lut_size - 1);

  float crgb[3] = {0.f, 0.f, 0.f}, ca = 0.f, cdepth = 0.f, covered = -FLT_MAX;
  bool have = false;
  int count = 0;
  unsigned phase = 0;
  bool staging = true;          // CTA-uniform: off after a wait gave up

  for (int oi = 0; oi < dorder.n; ++oi) {
    const DomainDev &dm = doms[dorder.d[oi]];
    // this ray's interval in the domain, as render_ray clamps it
    float bt0 = 0.f, bt1 = 0.f;
    bool act = false;
    if (valid && ca < mp.early_term) {
      float t0, t1;
      if (slab(dm, r, t0, t1)) {
        bt0 = fmaxf(t0, covered);
        bt1 = fminf(t1, t_max);
        covered = fmaxf(covered, bt1);
        act = true;
      }
    }
    if (!__syncthreads_or(act)) continue;
    const float thr = mp.early_term < 1.f ? (mp.early_term - ca) / (1.f - ca) : 2.f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float A[3], B[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
      B[a] = r.d[a] * dm.inv_spacing[a];
    }
    const int cmax[3] = {dm.dims[0] - 2, dm.dims[1] - 2, dm.dims[2] - 2};
    const int nbx = dm.nbrick[0], nby = dm.nbrick[1];
    const bool skip = mp.skip_empty && *dm.any_empty;
    int k = 0;
    bool live = act;
    int last_off = -1;
    float lc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    if (threadIdx.x == 0) s_level = 2;
    for (;;) {
      // the CTA's next sample distance
      float tn = FLT_MAX;
      if (live) {
        tn = fmaf((float)k, dt, bt0);
        if (!(tn < bt1)) {
          live = false;
          tn = FLT_MAX;
        }
      }
      if (threadIdx.x == 0) s_tmin = __float_as_uint(FLT_MAX);
      __syncthreads();
      if (live) atomicMin(&s_tmin, __float_as_uint(fmaxf(tn, 0.f)));
      __syncthreads();
      const float T = __uint_as_float(s_tmin);
      if (!(T < FLT_MAX)) break;

      // plan the slab: depth level, candidate box, frustum bricks -> slots
      const float brick_w = 8.f * fminf(fminf(1.f / dm.inv_spacing[0], 1.f / dm.inv_spacing[1]),
                                        1.f / dm.inv_spacing[2]);
      for (;;) {
        if (threadIdx.x == 0) {
          int lvl = s_level;
          for (;; ++lvl) {
            const float dT = brick_w * (float)(8 >> min(lvl, 3)) / (float)(1 << max(lvl - 3, 0));
            // (a slab that would not advance past T in float covers the rest)
            const float t1 = T + dT > T ? T + dT : FLT_MAX;
            float gmin[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, gmax[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
            for (int q = 0; q < 9; ++q) {
              const float *dd = q < 8 ? s_fr.dn[q & 3] : s_fr.c;
              const float tq = q < 4 ? T : t1;
              for (int a = 0; a < 3; ++a) {
                const float g = (fmaf(tq, dd[a], s_fr.o[a]) - dm.origin[a]) * dm.inv_spacing[a];
                gmin[a] = fminf(gmin[a], g);
                gmax[a] = fmaxf(gmax[a], g);
              }
            }
            int nb = 1;
            for (int a = 0; a < 3; ++a) {
              const int c0 = max(0, min((int)floorf(fmaxf(gmin[a], -1.f)) - 1, cmax[a]));
              const int c1 = max(0, min((int)floorf(fminf(gmax[a], (float)cmax[a] + 2.f)) + 1, cmax[a]));
              s_box[a] = c0 >> 3;
              s_box[3 + a] = (c1 >> 3) - (c0 >> 3) + 1;
              nb *= s_box[3 + a];
            }
            s_t1 = t1;
            if (nb <= kStageMap || lvl >= 5) {
              if (nb > kStageMap) s_box[3] = s_box[4] = s_box[5] = 0;  // no map: global reads
              s_level = lvl;
              break;
            }
          }
          s_count = 0;
        }
        __syncthreads();
        const int nb = s_box[3] * s_box[4] * s_box[5];
        for (int i = threadIdx.x; i < nb; i += kThreads) {
          const int bx = s_box[0] + i % s_box[3];
          const int by = s_box[1] + (i / s_box[3]) % s_box[4];
          const int bz = s_box[2] + i / (s_box[3] * s_box[4]);
          const int64_t gi = ((int64_t)bz * nby + by) * nbx + bx;
          short m = -1;
          if (skip && dm.brick_empty[gi]) {
            m = -2;
          } else {
            const int b3[3] = {bx, by, bz};
            float lo[3], hi[3];
            for (int a = 0; a < 3; ++a) {
              const float sp = 1.f / dm.inv_spacing[a];
              lo[a] = dm.origin[a] + sp * (float)(b3[a] * kBrickCells);
              hi[a] = dm.origin[a] + sp * (float)min((b3[a] + 1) * kBrickCells, cmax[a] + 1);
            }
            if (staging && frustum_box(s_fr, T, s_t1, lo, hi)) {
              const int slot = atomicAdd(&s_count, 1);
              if (slot < kStageSlots) {
                m = (short)slot;
                s_list[slot] = (int)gi;
              }
            }
          }
          s_map[i] = m;
        }
        __syncthreads();
        // too many frustum bricks for the slots: a shallower slab
        if (s_count <= kStageSlots || s_level >= 5) break;
        __syncthreads();
        if (threadIdx.x == 0) s_level = s_level + 1;
      }
      const float t1s = s_t1;
      const int staged = min(s_count, kStageSlots);

      // stage the slab's bricks
      if (staging && staged > 0) {
        if (threadIdx.x == 0)
          asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(&s_bar)),
                       "r"((unsigned)(staged * kBrickFloats * 4))
                       : "memory");
        __syncthreads();
        if (threadIdx.x < staged) {
          const float *src = dm.bricks + (int64_t)s_list[threadIdx.x] * kBrickFloats;
          asm volatile(
              "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                  smem_addr(slots + threadIdx.x * kBrickFloats)),
              "l"(src), "r"((unsigned)(kBrickFloats * 4)), "r"(smem_addr(&s_bar))
              : "memory");
        }
        const bool ok = __syncthreads_and(stage_wait(&s_bar, phase, kStagePolls));
        if (!ok) {
          // give the copies a second, long bound to land, then stop staging:
          // the rest of this CTA reads global memory (same values)
          stage_wait(&s_bar, phase, kStagePolls * 8);
          if (threadIdx.x == 0) atomicAdd(stage_fail, 1ull);
          staging = false;
        }
        phase ^= 1u;
      }
      const bool use_map = staging;

      // this slab's samples: t < min(bt1, slab end)
      while (live) {
        const float t = fmaf((float)k, dt, bt0);
        if (!(t < bt1)) { live = false; break; }
        if (!(t < t1s)) break;
        ++k;
        ++count;
        int c[3];
        float w[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float g = fmaf(t, B[a], A[a]);
          c[a] = max(0, min((int)g, cmax[a]));
          w[a] = g - (float)c[a];
        }
        const int bx = c[0] >> 3, by = c[1] >> 3, bz = c[2] >> 3;
        const int loff = ((c[2] & 7) * kBrickNodes + (c[1] & 7)) * kBrickNodes + (c[0] & 7);
        const int64_t gi = ((int64_t)bz * nby + by) * nbx + bx;
        const int off = (int)(gi * kBrickFloats) + loff;
        if (off != last_off) {
          int m = -1;
          if (use_map) {
            const unsigned rx = (unsigned)(bx - s_box[0]), ry = (unsigned)(by - s_box[1]),
                           rz = (unsigned)(bz - s_box[2]);
            if (rx < (unsigned)s_box[3] && ry < (unsigned)s_box[4] && rz < (unsigned)s_box[5])
              m = s_map[(rz * s_box[4] + ry) * s_box[3] + rx];
          }
          if (m == -2) continue;   // empty brick: zero opacity, counted
          if (m >= 0) {
            const float *q = slots + m * kBrickFloats + loff;
            lc[0] = q[0];
            lc[1] = q[1];
            lc[2] = q[kBrickNodes];
            lc[3] = q[kBrickNodes + 1];
            lc[4] = q[kBrickNodes * kBrickNodes];
            lc[5] = q[kBrickNodes * kBrickNodes + 1];
            lc[6] = q[kBrickNodes * kBrickNodes + kBrickNodes];
            lc[7] = q[kBrickNodes * kBrickNodes + kBrickNodes + 1];
          } else {
            const float *q = dm.bricks + off;
            lc[0] = __ldg(q);
            lc[1] = __ldg(q + 1);
            lc[2] = __ldg(q + kBrickNodes);
            lc[3] = __ldg(q + kBrickNodes + 1);
            lc[4] = __ldg(q + kBrickNodes * kBrickNodes);
            lc[5] = __ldg(q + kBrickNodes * kBrickNodes + 1);
            lc[6] = __ldg(q + kBrickNodes * kBrickNodes + kBrickNodes);
            lc[7] = __ldg(q + kBrickNodes * kBrickNodes + kBrickNodes + 1);
          }
          last_off = off;
        }
        const float c00 = lerpf(lc[0], lc[1], w[0]);
        const float c10 = lerpf(lc[2], lc[3], w[0]);
        const float c01 = lerpf(lc[4], lc[5], w[0]);
        const float c11 = lerpf(lc[6], lc[7], w[0]);
        const float v = lerpf(lerpf(c00, c10, w[1]), lerpf(c01, c11, w[1]), w[2]);
        const float sc = __saturatef((v - mp.scalar_min) * mp.inv_range);
        float4 col;
        if (mp.lut_filter == GVR_LUT_LINEAR) {
          col = lut_fetch(lut, mp.lut_size, GVR_LUT_LINEAR, sc);
        } else {
          col = lut_nearest(lut, nm1, sc);
        }
        const float wa = (1.f - acc.w) * col.w;
        acc.x = fmaf(wa, col.x, acc.x);
        acc.y = fmaf(wa, col.y, acc.y);
        acc.z = fmaf(wa, col.z, acc.z);
        acc.w += wa;
        if (acc.w >= thr) { live = false; break; }
      }
      __syncthreads();   // the slots and the map are rewritten by the next slab
      if (threadIdx.x == 0) s_level = max(s_level - 1, 0);
    }
    // the domain's partial, as render_ray blends it
    if (act && !(acc.w < mp.alpha_cull)) {
      if (!have) {
        crgb[0] = acc.x; crgb[1] = acc.y; crgb[2] = acc.z; ca = acc.w;
        cdepth = bt1;
        have = true;
      } else if (ca < 1.f && acc.w != 0.f) {
        const float op = 1.f - ca;
        crgb[0] = fmaf(op, acc.x, crgb[0]);
        crgb[1] = fmaf(op, acc.y, crgb[1]);
        crgb[2] = fmaf(op, acc.z, crgb[2]);
        ca = fminf(fmaf(op, acc.w, ca), 1.f);
      }
    }
  }
  if (valid) {
    float4 out;
    float dep;
    finish_pixel(view, mp, px, py, have, crgb, ca, cdepth, out, dep);
    const int64_t pix = (int64_t)py * mp.width + px;
    rgba[pix] = out;
    depth[pix] = dep;
  }
  if (samples) {
    unsigned long long cnt = (unsigned long long)count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0 && cnt) atomicAdd(samples, cnt);
  }
}


// ---------------------------------------------------------------------------
// Layer-staged march (staging mode 2): uniform vertex domains in 8^3-cell
// bricks, walked by brick layers along the axis the tile's rays advance
// fastest on. For each layer the tile's four corner rays, crossing the
// layer's two bounding planes, give a window of bricks that holds every
// sample the tile's rays take in that layer (the rays of the tile lie in the
// cone of its corner rays); the window's bricks are bulk-copied
// (cp.async.bulk, 2944 contiguous bytes each) into one of two shared-memory
// buffers, the next layer's copies in flight while the rays sample the
// current one. A window larger than SLOTS bricks, a layer that contains the
// camera, a sample outside the window (rounding) and a CTA whose bounded
// wait gave up read global memory instead: the same values, so images
// equal the gather march's. Domains are taken in one front-to-back order per
// CTA, as in staged_kernel. A scene with empty bricks to jump, or any domain
// this walk does not cover, is rendered by render_ray for every pixel.
// ---------------------------------------------------------------------------
constexpr long long kLayerPolls = 1 << 20;

// Thread 0: the window of layer L into win[0..3] = {first u brick, first v
// brick, width, height} (win[0] = -1: not staged) and its bulk copies into
// buf, completing on bar.
template <int SLOTS>
__device__ void layer_issue(const DomainDev &dm, const float (*cA)[3], const float (*cB)[3], int ax, int L,
                           float *buf, uint64_t *bar, int *win)
{
  const int u = ax == 0 ? 1 : 0, v = ax == 2 ? 1 : 2;
  float lo_u = FLT_MAX, hi_u = -FLT_MAX, lo_v = FLT_MAX, hi_v = -FLT_MAX;
  bool ok = true;
  for (int c = 0; c < 4; ++c) {
    if (!(cB[c][ax] != 0.f)) { ok = false; break; }
    for (int q = 0; q < 2; ++q) {
      const float t = ((float)((L + q) * kBrickCells) - cA[c][ax]) / cB[c][ax];
      if (!(t >= 0.f)) ok = false;   // the layer holds the camera (or NaN)
      const float gu = fmaf(t, cB[c][u], cA[c][u]), gv = fmaf(t, cB[c][v], cA[c][v]);
      lo_u = fminf(lo_u, gu); hi_u = fmaxf(hi_u, gu);
      lo_v = fminf(lo_v, gv); hi_v = fmaxf(hi_v, gv);
    }
  }
  int bu0 = 0, bu1 = -1, bv0 = 0, bv1 = -1;
  if (ok && lo_u > -1e9f && hi_u < 1e9f && lo_v > -1e9f && hi_v < 1e9f) {
    const int cu = dm.dims[u] - 2, cv = dm.dims[v] - 2;
    bu0 = max(0, min((int)floorf(lo_u), cu)) >> 3;
    bu1 = max(0, min((int)floorf(hi_u), cu)) >> 3;
    bv0 = max(0, min((int)floorf(lo_v), cv)) >> 3;
    bv1 = max(0, min((int)floorf(hi_v), cv)) >> 3;
  }
  const int wu = bu1 - bu0 + 1, wv = bv1 - bv0 + 1;
  const bool staged = ok && wu >= 1 && wv >= 1 && wu * wv <= SLOTS;
  win[0] = staged ? bu0 : -1;
  win[1] = bv0;
  win[2] = wu;
  win[3] = wv;
  const unsigned bytes = staged ? (unsigned)(wu * wv) * (unsigned)(sizeof(float) * kBrickFloats) : 0u;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)), "r"(bytes)
               : "memory");
  if (!staged) return;
  for (int j = 0; j < wv; ++j)
    for (int i = 0; i < wu; ++i) {
      int b[3];
      b[ax] = L;
      b[u] = bu0 + i;
      b[v] = bv0 + j;
      const int64_t lin = ((int64_t)b[2] * dm.nbrick[1] + b[1]) * dm.nbrick[0] + b[0];
      const float *src = dm.bricks + lin * kBrickFloats;
      float *dst = buf + (j * wu + i) * kBrickFloats;
      asm volatile(
          "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
              smem_addr(dst)),
          "l"(src), "r"((unsigned)(sizeof(float) * kBrickFloats)), "r"(smem_addr(bar))
          : "memory");
    }
}

template <int PW, int SLOTS, int MINB>
__global__ void __launch_bounds__(kThreads, MINB)
layer_kernel(const DomainDev *__restrict__ g_domains, const __grid_constant__ ViewDev view,
             const __grid_constant__ MarchParams mp, const float4 *__restrict__ g_lut,
             float4 *__restrict__ rgba, float *__restrict__ depth, unsigned long long *__restrict__ samples,
             const int *__restrict__ order, const StageOrder dorder, unsigned long long *__restrict__ stage_fail)
{
  constexpr int PH = 32 / PW;
  constexpr int PX = kTile / PW;
  const int tiles_x = (mp.width + kTile - 1) / kTile;
  const int tile = order ? __ldg(order + blockIdx.x) : (int)blockIdx.x;
  const int tile_x = tile % tiles_x, tile_y = tile / tiles_x;
  extern __shared__ float4 smem[];
  float4 *lut = smem;
  DomainDev *doms = reinterpret_cast<DomainDev *>(smem + mp.lut_size);
  const size_t head = ((sizeof(float4) * mp.lut_size + sizeof(DomainDev) * mp.n_domains) + 127) & ~(size_t)127;
  float *bufs = reinterpret_cast<float *>(reinterpret_cast<char *>(smem) + head);
  __shared__ __align__(8) uint64_t s_bar[2];
  __shared__ int s_win[2][4];
  __shared__ float s_cA[4][3], s_cB[4][3];
  __shared__ int s_ax, s_lmin, s_lmax;

  for (int i = threadIdx.x; i < mp.lut_size; i += kThreads) lut[i] = g_lut[i];
  {
    const int words = mp.n_domains * (int)(sizeof(DomainDev) / 4);
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g_domains);
    uint32_t *dst = reinterpret_cast<uint32_t *>(doms);
    for (int i = threadIdx.x; i < words; i += kThreads) dst[i] = src[i];
  }
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&s_bar[0])) : "memory");
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&s_bar[1])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  __syncthreads();

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int px = tile_x * kTile + (warp % PX) * PW + (lane % PW);
  const int py = tile_y * kTile + (warp / PX) * PH + (lane / PW);
  const bool valid = px < mp.width && py < mp.height;

  // every domain a uniform vertex field in 8^3-cell bricks with nothing to
  // jump (the same for all threads): else the per-ray march
  bool covered_all = true;
  for (int d = 0; d < mp.n_domains; ++d) {
    const DomainDev &dm = doms[d];
    covered_all = covered_all && dm.kind == GVR_DOMAIN_UNIFORM && dm.assoc == GVR_ASSOC_VERTEX &&
                  dm.bshift == 3 && !(mp.skip_empty && *dm.any_empty);
  }
  if (!covered_all) {
    // the buffers are not used on this path: render_ray's per-ray state
    // lives there
    static_assert(2 * SLOTS * kBrickFloats >= kStateSlots * kThreads, "state fits the buffers");
    float *s_state = bufs;
    int count = 0;
    if (valid) {
      const uint64_t all = mp.n_domains >= 64 ? ~0ull : ((1ull << mp.n_domains) - 1ull);
      float4 out;
      float dep;
      count = render_ray<1, false>(doms, all, view, mp, lut, px, py, out, dep, s_state);
      const int64_t pix = (int64_t)py * mp.width + px;
      rgba[pix] = out;
      depth[pix] = dep;
    }
    if (samples) {
      unsigned long long c = (unsigned long long)count;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
      if (lane == 0 && c) atomicAdd(samples, c);
    }
    return;
  }

  const Ray r = pixel_ray(view, mp, valid ? px : 0, valid ? py : 0);
  const float t_max = valid ? canvas_ray_end(view, mp, px, py) : FLT_MAX;
  const float dt = mp.sample_dist;
  const float nm1 = (float)(mp.lut_size - 1);
  float crgb[3] = {0.f, 0.f, 0.f}, ca = 0.f, cdepth = 0.f, covered = -FLT_MAX;
  bool have = false;
  int count = 0;
  unsigned ph0 = 0, ph1 = 0;   // barrier phases (CTA-uniform)
  bool staging = true;         // CTA-uniform: off after a wait gave up

  for (int oi = 0; oi < dorder.n; ++oi) {
    const DomainDev &dm = doms[dorder.d[oi]];
    float bt0 = 0.f, bt1 = 0.f;
    bool act = false;
    if (valid && ca < mp.early_term) {
      float t0, t1;
      if (slab(dm, r, t0, t1)) {
        bt0 = fmaxf(t0, covered);
        bt1 = fminf(t1, t_max);
        covered = fmaxf(covered, bt1);
        act = true;
      }
    }
    if (threadIdx.x == 0) {
      s_lmin = INT_MAX;
      s_lmax = -1;
      // the tile's corner rays in this domain's grid space, and the axis
      // its centre ray advances fastest on
      const int x0 = tile_x * kTile, y0 = tile_y * kTile;
      const int cx[4] = {x0, x0 + kTile - 1, x0, x0 + kTile - 1};
      const int cy[4] = {y0, y0, y0 + kTile - 1, y0 + kTile - 1};
      for (int c = 0; c < 4; ++c) {
        const Ray rc = pixel_ray(view, mp, cx[c], cy[c]);
        for (int a = 0; a < 3; ++a) {
          s_cA[c][a] = (rc.o[a] - dm.origin[a]) * dm.inv_spacing[a];
          s_cB[c][a] = rc.d[a] * dm.inv_spacing[a];
        }
      }
      const Ray rm = pixel_ray(view, mp, x0 + kTile / 2, y0 + kTile / 2);
      float best = -1.f;
      int ax = 2;
      for (int a = 0; a < 3; ++a) {
        const float m = fabsf(rm.d[a] * dm.inv_spacing[a]);
        if (m > best) { best = m; ax = a; }
      }
      s_ax = ax;
    }
    __syncthreads();
    if (!__syncthreads_or(act)) continue;
    const int ax = s_ax;
    const float thr = mp.early_term < 1.f ? (mp.early_term - ca) / (1.f - ca) : 2.f;
    float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
    float A[3], B[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      A[a] = (r.o[a] - dm.origin[a]) * dm.inv_spacing[a];
      B[a] = r.d[a] * dm.inv_spacing[a];
    }
    const int cmax[3] = {dm.dims[0] - 2, dm.dims[1] - 2, dm.dims[2] - 2};
    const int nbx = dm.nbrick[0], nby = dm.nbrick[1];
    // this ray's layers: those of its first sample and of its interval's end
    if (act) {
      const float aa = ax == 0 ? A[0] : (ax == 1 ? A[1] : A[2]);
      const float ba = ax == 0 ? B[0] : (ax == 1 ? B[1] : B[2]);
      const int ca_max = ax == 0 ? cmax[0] : (ax == 1 ? cmax[1] : cmax[2]);
      const int c0 = max(0, min((int)fmaf(bt0, ba, aa), ca_max)) >> 3;
      const int c1 = max(0, min((int)fmaf(bt1, ba, aa), ca_max)) >> 3;
      atomicMin(&s_lmin, min(c0, c1));
      atomicMax(&s_lmax, max(c0, c1));
    }
    __syncthreads();
    const bool up = s_cB[0][ax] + s_cB[1][ax] + s_cB[2][ax] + s_cB[3][ax] > 0.f;
    const int lmin = s_lmin, lmax = s_lmax;
    const int n_layers = lmax - lmin + 1;
    const int Lb = up ? lmin : lmax, step = up ? 1 : -1;
    // a ray that does not advance along the axis the tile's corner rays do
    // (none in practice: the axis is its centre ray's dominant one) takes
    // all its samples in the first layer, from global memory outside the
    // window
    const float bax = ax == 0 ? B[0] : (ax == 1 ? B[1] : B[2]);
    const bool ordered = up ? bax > 0.f : bax < 0.f;
    if (threadIdx.x == 0 && staging) {
      layer_issue<SLOTS>(dm, s_cA, s_cB, ax, Lb, bufs, &s_bar[0], s_win[0]);
      if (n_layers > 1) layer_issue<SLOTS>(dm, s_cA, s_cB, ax, Lb + step, bufs + SLOTS * kBrickFloats,
                                           &s_bar[1], s_win[1]);
    }
    bool pend0 = staging, pend1 = staging && n_layers > 1;   // copies issued, not yet waited for
    int k = 0;
    bool live = act;
    int last_off = -1;
    float lc[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
    for (int li = 0; li < n_layers; ++li) {
      const int L = Lb + step * li;
      const int b = li & 1;
      bool use = false;
      if (b == 0 ? pend0 : pend1) {
        uint64_t *bar = &s_bar[b];
        const unsigned ph = b == 0 ? ph0 : ph1;
        bool ok = __syncthreads_and(stage_wait(bar, ph, kLayerPolls));
        if (!ok) {
          // the copies may still land: wait once more, longer, then read
          // global memory for the rest of the tile
          if (threadIdx.x == 0) atomicAdd(stage_fail, 1ull);
          __syncthreads_and(stage_wait(bar, ph, 8 * kLayerPolls));
          staging = false;
        }
        if (b == 0) { ph0 ^= 1u; pend0 = false; } else { ph1 ^= 1u; pend1 = false; }
        use = ok && s_win[b][0] >= 0;
      }
      const float *buf = bufs + b * SLOTS * kBrickFloats;
      const int wu0 = s_win[b][0], wv0 = s_win[b][1], wu = s_win[b][2], wv = s_win[b][3];
      const int u = ax == 0 ? 1 : 0, v = ax == 2 ? 1 : 2;
      while (live) {
        const float t = fmaf((float)k, dt, bt0);
        if (!(t < bt1)) { live = false; break; }
        int c[3];
        float w[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          const float g = fmaf(t, B[a], A[a]);
          c[a] = max(0, min((int)g, cmax[a]));
          w[a] = g - (float)c[a];
        }
        // (selects, not c[ax]: a runtime index would put c in local memory)
        const int lay = (ax == 0 ? c[0] : (ax == 1 ? c[1] : c[2])) >> 3;
        if (ordered && (up ? lay > L : lay < L)) break;   // a later layer's sample
        ++k;
        ++count;
        const int loff = ((c[2] & 7) * kBrickNodes + (c[1] & 7)) * kBrickNodes + (c[0] & 7);
        const int64_t gi = ((int64_t)(c[2] >> 3) * nby + (c[1] >> 3)) * nbx + (c[0] >> 3);
        const int off = (int)(gi * kBrickFloats) + loff;
        if (off != last_off) {
          const int cu = u == 0 ? c[0] : c[1], cv = v == 1 ? c[1] : c[2];
          const unsigned iu = (unsigned)((cu >> 3) - wu0), iv = (unsigned)((cv >> 3) - wv0);
          if (use && iu < (unsigned)wu && iv < (unsigned)wv) {
            const float *q = buf + (iv * wu + iu) * kBrickFloats + loff;
            lc[0] = q[0];
            lc[1] = q[1];
            lc[2] = q[kBrickNodes];
            lc[3] = q[kBrickNodes + 1];
            lc[4] = q[kBrickNodes * kBrickNodes];
            lc[5] = q[kBrickNodes * kBrickNodes + 1];
            lc[6] = q[kBrickNodes * kBrickNodes + kBrickNodes];
            lc[7] = q[kBrickNodes * kBrickNodes + kBrickNodes + 1];
          } else {
            const float *q = dm.bricks + off;
            lc[0] = __ldg(q);
            lc[1] = __ldg(q + 1);
            lc[2] = __ldg(q + kBrickNodes);
            lc[3] = __ldg(q + kBrickNodes + 1);
            lc[4] = __ldg(q + kBrickNodes * kBrickNodes);
            lc[5] = __ldg(q + kBrickNodes * kBrickNodes + 1);
            lc[6] = __ldg(q + kBrickNodes * kBrickNodes + kBrickNodes);
            lc[7] = __ldg(q + kBrickNodes * kBrickNodes + kBrickNodes + 1);
          }
          last_off = off;
        }
        const float c00 = lerpf(lc[0], lc[1], w[0]);
        const float c10 = lerpf(lc[2], lc[3], w[0]);
        const float c01 = lerpf(lc[4], lc[5], w[0]);
        const float c11 = lerpf(lc[6], lc[7], w[0]);
        const float val = lerpf(lerpf(c00, c10, w[1]), lerpf(c01, c11, w[1]), w[2]);
        const float sc = __saturatef((val - mp.scalar_min) * mp.inv_range);
        float4 col;
        if (mp.lut_filter == GVR_LUT_LINEAR) {
          col = lut_fetch(lut, mp.lut_size, GVR_LUT_LINEAR, sc);
        } else {
          col = lut_nearest(lut, nm1, sc);
        }
        const float wa = (1.f - acc.w) * col.w;
        acc.x = fmaf(wa, col.x, acc.x);
        acc.y = fmaf(wa, col.y, acc.y);
        acc.z = fmaf(wa, col.z, acc.z);
        acc.w += wa;
        if (acc.w >= thr) { live = false; break; }
      }
      // the buffer is free again: the layer two ahead goes into it, unless
      // no ray is left (then only the copies already issued are waited for)
      const bool any = __syncthreads_or(live);
      if (any && staging && li + 2 < n_layers) {
        if (threadIdx.x == 0)
          layer_issue<SLOTS>(dm, s_cA, s_cB, ax, L + 2 * step, bufs + b * SLOTS * kBrickFloats, &s_bar[b],
                             s_win[b]);
        if (b == 0) pend0 = true; else pend1 = true;
      }
      if (!any) break;
    }
    // drain copies still in flight before the buffers are reused
    for (int b = 0; b < 2; ++b) {
      if (!(b == 0 ? pend0 : pend1)) continue;
      const unsigned ph = b == 0 ? ph0 : ph1;
      if (!__syncthreads_and(stage_wait(&s_bar[b], ph, 8 * kLayerPolls))) {
        if (threadIdx.x == 0) atomicAdd(stage_fail, 1ull);
        staging = false;
      }
      if (b == 0) { ph0 ^= 1u; pend0 = false; } else { ph1 ^= 1u; pend1 = false; }
    }
    __syncthreads();
    // the domain's partial, as render_ray blends it
    if (act && !(acc.w < mp.alpha_cull)) {
      if (!have) {
        crgb[0] = acc.x; crgb[1] = acc.y; crgb[2] = acc.z; ca = acc.w;
        cdepth = bt1;
        have = true;
      } else if (ca < 1.f && acc.w != 0.f) {
        const float op = 1.f - ca;
        crgb[0] = fmaf(op, acc.x, crgb[0]);
        crgb[1] = fmaf(op, acc.y, crgb[1]);
        crgb[2] = fmaf(op, acc.z, crgb[2]);
        ca = fminf(fmaf(op, acc.w, ca), 1.f);
      }
    }
  }
  if (valid) {
    float4 out;
    float dep;
    finish_pixel(view, mp, px, py, have, crgb, ca, cdepth, out, dep);
    const int64_t pix = (int64_t)py * mp.width + px;
    rgba[pix] = out;
    depth[pix] = dep;
  }
  if (samples) {
    unsigned long long cnt = (unsigned long long)count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    if (lane == 0 && cnt) atomicAdd(samples, cnt);
  }
}

// Many views in one persistent launch. A device counter hands out work items
// of `tiles_per_item` consecutive 16x16 tiles; items run through every tile
// of view 0, then view 1, ... so neighbouring CTAs share bricks in L2. Each
// tile first builds the bitmask of domains whose projected screen rectangle
// (rects[view * n_domains + d], inclusive pixel bounds, computed on the host)
// touches it, and its rays march only those. The counter only grows: no CTA
// ever waits for another.
template <int PW, int UNROLL, int MINB, bool HEX>
__global__ void __launch_bounds__(kThreads, MINB)
batch_kernel(const DomainDev *__restrict__ g_domains, const ViewDev *__restrict__ views,
             const int4 *__restrict__ rects, const __grid_constant__ MarchParams mp, int n_views,
             int tiles_x,
             int tiles_y, int tiles_per_item, const float4 *__restrict__ g_lut,
             float4 *__restrict__ rgba, float *__restrict__ depth,
             unsigned long long *__restrict__ samples, unsigned int *__restrict__ queue)
{
  constexpr int PH = 32 / PW;
  constexpr int PX = kTile / PW;
  extern __shared__ float4 smem[];
  float4 *lut = smem;
  DomainDev *doms = reinterpret_cast<DomainDev *>(smem + mp.lut_size);
  __shared__ unsigned int s_item;
  __shared__ unsigned int s_mask[2];
  __shared__ float s_state[kStateSlots * kThreads];
  for (int i = threadIdx.x; i < mp.lut_size; i += kThreads) lut[i] = g_lut[i];
  {
    const int words = mp.n_domains * (int)(sizeof(DomainDev) / 4);
    const uint32_t *src = reinterpret_cast<const uint32_t *>(g_domains);
    uint32_t *dst = reinterpret_cast<uint32_t *>(doms);
    for (int i = threadIdx.x; i < words; i += kThreads) dst[i] = src[i];
  }
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int tiles_per_view = tiles_x * tiles_y;
  const long long total_tiles = (long long)tiles_per_view * n_views;
  const long long n_items = (total_tiles + tiles_per_item - 1) / tiles_per_item;
  const int64_t pixels = (int64_t)mp.width * mp.height;
  int count = 0;
  for (;;) {
    __syncthreads();
    if (threadIdx.x == 0) s_item = atomicAdd(queue, 1u);
    __syncthreads();
    const long long item = s_item;
    if (item >= n_items) break;
    for (int sub = 0; sub < tiles_per_item; ++sub) {
      const long long tile = item * tiles_per_item + sub;
      if (tile >= total_tiles) break;
      const int v = (int)(tile / tiles_per_view);
      const int t = (int)(tile % tiles_per_view);
      const int tx = t % tiles_x, ty = t / tiles_x;
      const int x0 = tx * kTile, y0 = ty * kTile;
      if (warp < 2) {
        const int d = warp * 32 + lane;
        bool hit = false;
        if (d < mp.n_domains) {
          const int4 r = __ldg(rects + (int64_t)v * mp.n_domains + d);
          hit = !(r.z < x0 || r.x > x0 + kTile - 1 || r.w < y0 || r.y > y0 + kTile - 1);
        }
        const unsigned b = __ballot_sync(0xffffffffu, hit);
        if (lane == 0) s_mask[warp] = b;
      }
      __syncthreads();
      const uint64_t mask = ((uint64_t)s_mask[1] << 32) | s_mask[0];
      const int px = x0 + (warp % PX) * PW + (lane % PW);
      const int py = y0 + (warp / PX) * PH + (lane / PW);
      if (px < mp.width && py < mp.height) {
        float4 out;
        float dep;
        count += render_ray<UNROLL, HEX>(doms, mask, views[v], mp, lut, px, py, out, dep, s_state);
        const int64_t pix = (int64_t)v * pixels + (int64_t)py * mp.width + px;
        rgba[pix] = out;
        depth[pix] = dep;
      }
      __syncthreads();
    }
  }
  if (samples) {
    unsigned long long c = (unsigned long long)count;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0 && c) atomicAdd(samples, c);
  }
}

}  // namespace

namespace {

using MarchFn = void (*)(const DomainDev *, const ViewDev, const MarchParams, const float4 *,
                         float4 *, float *, unsigned long long *, const int *);

template <int PW, int UNROLL, int MINB>
MarchFn pick() { return march_kernel<PW, UNROLL, MINB>; }

MarchFn select(const Tuning &t, bool has_hex)
{
  // the hex path keeps a cell's eight coefficient records in registers: 2 or
  // 3 CTAs per SM (3 spills some 400 bytes and measured 1.5% faster)
  if (has_hex) {
    const bool m3 = t.min_blocks >= 4;
    if (t.packet_w == 4) return m3 ? march_kernel<4, 1, 3, true> : march_kernel<4, 1, 2, true>;
    return m3 ? march_kernel<8, 1, 3, true> : march_kernel<8, 1, 2, true>;
  }
  // three samples per iteration exists only at 4 CTAs per SM (at 3 it
  // measured slower than two)
  if (t.unroll >= 4)
    return t.min_blocks >= 4 ? (t.packet_w == 4 ? pick<4, 4, 4>() : pick<8, 4, 4>())
                             : (t.packet_w == 4 ? pick<4, 4, 3>() : pick<8, 4, 3>());
  if (t.unroll >= 3) {
    if (t.min_blocks < 4) return t.packet_w == 4 ? pick<4, 3, 3>() : pick<8, 3, 3>();
    return t.packet_w == 4 ? pick<4, 3, 4>() : (t.packet_w == 16 ? pick<16, 3, 4>() : pick<8, 3, 4>());
  }
  const int u = t.unroll >= 2 ? 2 : 1;
  const int m = t.min_blocks >= 4 ? 4 : 3;
  switch (t.packet_w) {
    case 4:
      return u == 2 ? (m == 4 ? pick<4, 2, 4>() : pick<4, 2, 3>()) : (m == 4 ? pick<4, 1, 4>() : pick<4, 1, 3>());
    case 16:
      return u == 2 ? (m == 4 ? pick<16, 2, 4>() : pick<16, 2, 3>()) : (m == 4 ? pick<16, 1, 4>() : pick<16, 1, 3>());
    default:
      return u == 2 ? (m == 4 ? pick<8, 2, 4>() : pick<8, 2, 3>()) : (m == 4 ? pick<8, 1, 4>() : pick<8, 1, 3>());
  }
}

}  // namespace

cudaError_t launch_march(const DomainDev *d_domains, const ViewDev &view,
                         const MarchParams &mp, const float4 *d_lut, float4 *d_rgba,
                         float *d_depth, unsigned long long *d_samples, const Tuning &tuning,
                         bool has_hex, const int *d_order, cudaStream_t stream)
{
  const size_t smem = sizeof(float4) * mp.lut_size + sizeof(DomainDev) * mp.n_domains;
  MarchFn fn = select(tuning, has_hex);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(float4) * kMaxLut + sizeof(DomainDev) * kMaxDomains));
  if (e != cudaSuccess) return e;
  const int64_t tiles = (int64_t)((mp.width + kTile - 1) / kTile) * ((mp.height + kTile - 1) / kTile);
  fn<<<(unsigned)tiles, kThreads, smem, stream>>>(d_domains, view, mp, d_lut, d_rgba, d_depth,
                                                  d_samples, d_order);
  count_launch();
  return cudaGetLastError();
}


// Longest-first launch order of the march tiles for one view: the cost of a
// tile is the summed length, through every domain box, of five of its rays
// (its centre and corner pixels); tiles are counting-sorted into 1024 cost
// bins, longest first, so that the last tiles the GPU takes are the short
// ones (longest-processing-time-first list scheduling). Two launches: the
// costs with one thread per tile (keys[t] = the cost's bits, *top = their
// maximum), then one CTA bins, scans and scatters them and clears *top for
// the next view. The order of tiles within a bin is whatever the
// shared-memory atomics give, and no order changes a pixel.
__global__ void __launch_bounds__(256)
tile_cost_kernel(const DomainDev *__restrict__ g_domains, const __grid_constant__ ViewDev view,
                 const __grid_constant__ MarchParams mp, unsigned *__restrict__ keys,
                 unsigned *__restrict__ top)
{
  const int tiles_x = (mp.width + kTile - 1) / kTile;
  const int n = tiles_x * ((mp.height + kTile - 1) / kTile);
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned bits = 0u;
  if (t < n) {
    const int x0 = (t % tiles_x) * kTile, y0 = (t / tiles_x) * kTile;
    const int x1 = min(x0 + kTile - 1, mp.width - 1), y1 = min(y0 + kTile - 1, mp.height - 1);
    const int rx[5] = {(x0 + x1) >> 1, x0, x1, x0, x1};
    const int ry[5] = {(y0 + y1) >> 1, y0, y0, y1, y1};
    float cost = 0.f;
    for (int k = 0; k < 5; ++k) {
      const Ray r = pixel_ray(view, mp, rx[k], ry[k]);
      for (int d = 0; d < mp.n_domains; ++d) {
        float t0, t1;
        if (slab(g_domains[d], r, t0, t1)) cost += t1 - t0;
      }
    }
    cost = cost > 0.f && cost < FLT_MAX ? cost : 0.f;   // NaN and inf cost nothing
    bits = __float_as_uint(cost);
    keys[t] = bits;
  }
  bits = __reduce_max_sync(0xffffffffu, bits);
  if ((threadIdx.x & 31) == 0 && bits) atomicMax(top, bits);
}

__global__ void __launch_bounds__(1024)
tile_order_sort_kernel(const __grid_constant__ MarchParams mp, const unsigned *__restrict__ keys,
                       unsigned *__restrict__ top, int *__restrict__ order)
{
  __shared__ int s_hist[1024];
  __shared__ int s_warp[32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int tiles_x = (mp.width + kTile - 1) / kTile;
  const int n = tiles_x * ((mp.height + kTile - 1) / kTile);
  s_hist[tid] = 0;
  const float high = __uint_as_float(*top);
  const float scale = high > 0.f ? 1023.f / high : 0.f;
  __syncthreads();
  for (int t = tid; t < n; t += 1024)
    atomicAdd(&s_hist[1023 - min(1023, (int)(__uint_as_float(keys[t]) * scale))], 1);
  __syncthreads();
  // exclusive scan of the 1024 bins, one per thread
  const int v = s_hist[tid];
  int x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_warp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = s_warp[lane];
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    s_warp[lane] = w;
  }
  __syncthreads();
  s_hist[tid] = x - v + (warp ? s_warp[warp - 1] : 0);
  __syncthreads();
  for (int t = tid; t < n; t += 1024) {
    const int bin = 1023 - min(1023, (int)(__uint_as_float(keys[t]) * scale));
    order[atomicAdd(&s_hist[bin], 1)] = t;
  }
  if (tid == 0) *top = 0u;
}

cudaError_t launch_tile_cost_order(const DomainDev *d_domains, const ViewDev &view, const MarchParams &mp,
                                   int *d_order, unsigned *d_keys, unsigned *d_top, cudaStream_t stream)
{
  const int64_t tiles = (int64_t)((mp.width + kTile - 1) / kTile) * ((mp.height + kTile - 1) / kTile);
  if (tiles > kCostOrderTiles) return cudaErrorInvalidValue;
  tile_cost_kernel<<<(unsigned)((tiles + 255) / 256), 256, 0, stream>>>(d_domains, view, mp, d_keys, d_top);
  tile_order_sort_kernel<<<1, 1024, 0, stream>>>(mp, d_keys, d_top, d_order);
  count_launch(2);
  return cudaGetLastError();
}

namespace {

using StagedFn = void (*)(const DomainDev *, const ViewDev, const MarchParams, const float4 *, float4 *,
                          float *, unsigned long long *, const int *, const StageOrder,
                          unsigned long long *);

StagedFn select_staged(const Tuning &t)
{
  return t.packet_w == 4 ? staged_kernel<4> : (t.packet_w == 16 ? staged_kernel<16> : staged_kernel<8>);
}

size_t staged_smem(int lut_size, int n_domains)
{
  const size_t head = (sizeof(float4) * lut_size + sizeof(DomainDev) * n_domains + 127) & ~(size_t)127;
  return head + sizeof(float) * kBrickFloats * kStageSlots;
}

}  // namespace

cudaError_t launch_staged(const DomainDev *d_domains, const ViewDev &view, const MarchParams &mp,
                          const float4 *d_lut, float4 *d_rgba, float *d_depth,
                          unsigned long long *d_samples, const Tuning &tuning, const int *d_order,
                          const StageOrder &order, unsigned long long *d_stage_fail,
                          cudaStream_t stream)
{
  if (tuning.staged == 2) {
    // the layer walk, two buffers: 9 bricks per window (3 x 3) at 3 CTAs per
    // SM, or 12 at 2 (min_blocks 4)
    const bool wide = tuning.min_blocks >= 4;
    const int slots = wide ? 12 : 9;
    StagedFn lfn = wide ? (tuning.packet_w == 4 ? layer_kernel<4, 12, 2> : layer_kernel<8, 12, 2>)
                        : (tuning.packet_w == 4 ? layer_kernel<4, 9, 3> : layer_kernel<8, 9, 3>);
    auto lsmem = [slots](int lut_size, int n_domains) {
      const size_t head = (sizeof(float4) * lut_size + sizeof(DomainDev) * n_domains + 127) & ~(size_t)127;
      return head + 2 * sizeof(float) * kBrickFloats * slots;
    };
    cudaError_t e = cudaFuncSetAttribute(lfn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)lsmem(kMaxLut, kMaxDomains));
    if (e != cudaSuccess) return e;
    const int64_t tiles = (int64_t)((mp.width + kTile - 1) / kTile) * ((mp.height + kTile - 1) / kTile);
    lfn<<<(unsigned)tiles, kThreads, lsmem(mp.lut_size, mp.n_domains), stream>>>(
        d_domains, view, mp, d_lut, d_rgba, d_depth, d_samples, d_order, order, d_stage_fail);
    count_launch();
    return cudaGetLastError();
  }
  StagedFn fn = select_staged(tuning);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)staged_smem(kMaxLut, kMaxDomains));
  if (e != cudaSuccess) return e;
  const int64_t tiles = (int64_t)((mp.width + kTile - 1) / kTile) * ((mp.height + kTile - 1) / kTile);
  fn<<<(unsigned)tiles, kThreads, staged_smem(mp.lut_size, mp.n_domains), stream>>>(
      d_domains, view, mp, d_lut, d_rgba, d_depth, d_samples, d_order, order, d_stage_fail);
  count_launch();
  return cudaGetLastError();
}

namespace {

using BatchFn = void (*)(const DomainDev *, const ViewDev *, const int4 *, const MarchParams, int,
                         int, int, int, const float4 *, float4 *, float *, unsigned long long *,
                         unsigned int *);

BatchFn select_batch(const Tuning &t, bool has_hex)
{
  if (has_hex) return t.packet_w == 4 ? batch_kernel<4, 1, 2, true> : batch_kernel<8, 1, 2, true>;
  const int u = t.unroll >= 2 ? 2 : 1;
  const int m = t.min_blocks >= 4 ? 4 : 3;
  switch (t.packet_w) {
    case 4:
      return u == 2 ? (m == 4 ? batch_kernel<4, 2, 4, false> : batch_kernel<4, 2, 3, false>)
                    : (m == 4 ? batch_kernel<4, 1, 4, false> : batch_kernel<4, 1, 3, false>);
    case 16:
      return u == 2 ? (m == 4 ? batch_kernel<16, 2, 4, false> : batch_kernel<16, 2, 3, false>)
                    : (m == 4 ? batch_kernel<16, 1, 4, false> : batch_kernel<16, 1, 3, false>);
    default:
      return u == 2 ? (m == 4 ? batch_kernel<8, 2, 4, false> : batch_kernel<8, 2, 3, false>)
                    : (m == 4 ? batch_kernel<8, 1, 4, false> : batch_kernel<8, 1, 3, false>);
  }
}

}  // namespace

// Resident CTAs of the batch kernel for this launch shape (SMs x CTAs per SM
// from the occupancy calculator), capped by the number of work items. Also
// sets the kernel's dynamic shared-memory limit; call it outside any capture.
cudaError_t batch_grid(const MarchParams &mp, int n_views, const Tuning &tuning, bool has_hex,
                       int *grid)
{
  const size_t smem = sizeof(float4) * mp.lut_size + sizeof(DomainDev) * mp.n_domains;
  BatchFn fn = select_batch(tuning, has_hex);
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)(sizeof(float4) * kMaxLut + sizeof(DomainDev) * kMaxDomains));
  if (e != cudaSuccess) return e;
  int dev = 0, sms = 0, per_sm = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kThreads, smem);
  if (e != cudaSuccess) return e;
  const int tiles_x = (mp.width + kTile - 1) / kTile, tiles_y = (mp.height + kTile - 1) / kTile;
  const int tpi = tuning.tiles_per_item > 0 ? tuning.tiles_per_item : 1;
  const long long items = ((long long)tiles_x * tiles_y * n_views + tpi - 1) / tpi;
  *grid = (int)std::max(1ll, std::min<long long>(items, (long long)sms * std::max(per_sm, 1)));
  return cudaSuccess;
}

// Clear the work counter and launch the persistent batch kernel (both stream
// operations, so the pair can be captured into a CUDA graph).
cudaError_t launch_batch(const DomainDev *d_domains, const ViewDev *d_views, const int4 *d_rects,
                         const MarchParams &mp, int n_views, const float4 *d_lut, float4 *d_rgba,
                         float *d_depth, unsigned long long *d_samples, unsigned int *d_queue,
                         const Tuning &tuning, bool has_hex, int grid, cudaStream_t stream)
{
  const size_t smem = sizeof(float4) * mp.lut_size + sizeof(DomainDev) * mp.n_domains;
  BatchFn fn = select_batch(tuning, has_hex);
  const int tiles_x = (mp.width + kTile - 1) / kTile, tiles_y = (mp.height + kTile - 1) / kTile;
  const int tpi = tuning.tiles_per_item > 0 ? tuning.tiles_per_item : 1;
  cudaError_t e = cudaMemsetAsync(d_queue, 0, sizeof(unsigned int), stream);
  if (e != cudaSuccess) return e;
  fn<<<(unsigned)grid, kThreads, smem, stream>>>(d_domains, d_views, d_rects, mp, n_views, tiles_x,
                                                 tiles_y, tpi, d_lut, d_rgba, d_depth, d_samples,
                                                 d_queue);
  return cudaGetLastError();
}

}  // namespace gvr
