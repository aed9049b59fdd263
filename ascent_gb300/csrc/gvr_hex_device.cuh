// gvr_hex_device.cuh — point location in hexahedral meshes (device code).
//
// A point is located by walking the mesh's LBVH (flat layout written by
// gvr_hex.cu) and, at each candidate leaf, solving the inverse trilinear
// map x(r,s,t) = p by Newton's method. This is the algorithm of Devil Ray's
// DeviceMesh::locate (src/libs/dray/data_model/device_mesh.hpp:250-360: a
// stack walk that enters the left child first, pushes the right one when the
// point is inside both boxes, and stops at the first leaf whose element
// contains the point) with its NewtonSolve (src/libs/dray/newton_solver.hpp:
// 33-110, at most 10 steps). Arithmetic is FP32.
//
// Flat BVH node (4 float4 per inner node):
//   [0] = left.lo.x, left.lo.y, left.lo.z, left.hi.x
//   [1] = left.hi.y, left.hi.z, right.lo.x, right.lo.y
//   [2] = right.lo.z, right.hi.x, right.hi.y, right.hi.z
//   [3] = bits of int left child, bits of int right child, 0, 0
// A child >= 0 is an inner node index; a child < 0 is leaf k = -child - 1
// (k indexes the Morton-sorted leaves; hex_ids[k] is its cell id).
#pragma once

#include "gvr_internal.h"

namespace gvr {

constexpr int kHexNewtonSteps = 10;        // NewtonSolve default_max_steps
// Newton's method converges quadratically on the trilinear map: after a
// step of size d the remaining error is about c d^2, c well below 1 for
// cells that are not folded (jittered 200^3 mesh: ~1e-6 after a 2e-3 step),
// so a solve is accepted once its step is below 2e-3 — one iteration from
// the extrapolated guess instead of two, 12% faster on that mesh with the
// same image error against the FP64 oracle. FP32 positions resolve a cell
// of a 200^3 unit-cube mesh to ~1e-5 in reference units, and the inside
// test allows 2e-4: tighter bounds leave samples near faces unlocated in
// every neighbouring cell.
constexpr float kHexNewtonTol = 2e-3f;     // |step|_inf in reference space
// The march's solves start from the guess extrapolated along the ray, whose
// first step is ~0.02 and already leaves ~1e-4 (a CPU emulation on a
// jittered mesh: 4.9e-5 median, 6.4e-4 p99 after a step below 0.05), and
// the field is continuous across faces, so there a step below
// kHexLooseTol ends the solve. Swept on the jittered 200^3 mesh at 1024^2
// (Gsamples/s, full-frame error against the FP64 oracle): 2e-3 20.9;
// 0.05 accepted only 0.01 or more inside every face 21.1; 0.1 24.3;
// 0.15 25.3; 0.2 26.0; 0.3 26.1 — every one with 100% of pixels within
// 2/255 and the same maximum error (3.8e-3), mean error 2.6e-7 at 0.2
// against 2.9e-8 at 2e-3. Point location from a cell's centre keeps
// kHexNewtonTol.
#ifndef GVR_HEX_LOOSE_TOL
#define GVR_HEX_LOOSE_TOL 0.2f
#endif
constexpr float kHexLooseTol = GVR_HEX_LOOSE_TOL;
constexpr float kHexInsideTol = 2e-4f;     // r, s, t in [-tol, 1 + tol]
constexpr int kHexStack = 64;
constexpr int kHexHops = 4;                // face-neighbour steps before the LBVH walk
constexpr float kHexPredictMargin = 0.02f; // guess this far outside: step before solving

// A cell's trilinear map x(r,s,t) = sum_k c_k m_k(r,s,t) over the monomials
// m = (1, r, s, t, rs, rt, st, rst); c_k are position coefficients and w_k
// those of the vertex field. From the VTK corners v0..v7:
//   c0 = v0, c1 = v1 - v0, c2 = v3 - v0, c3 = v4 - v0,
//   c4 = v2 - v1 - v3 + v0, c5 = v5 - v1 - v4 + v0, c6 = v7 - v3 - v4 + v0,
//   c7 = v6 - v2 - v5 - v7 + v1 + v3 + v4 - v0.
// Evaluating the map and its Jacobian this way takes ~50 multiply-adds per
// Newton step instead of ~140 through the corner weights. A cell's record
// is 32 contiguous floats (8 float4, 128 bytes): the 24 position
// coefficients c0.xyz .. c7.xyz, then w0 .. w7. The march keeps the 24
// position coefficients in registers while it stays in a cell and reads the
// field's 8 (two float4, usually L1 hits) only to interpolate a sample, so
// the Newton solve has 8 more registers than with whole float4 corners.
struct HexGeom {
  float c[8][3];
};

__device__ __forceinline__ void hex_load(const DomainDev &dm, int cell, HexGeom &g)
{
  const float4 *q = dm.hex_coef + 8 * (int64_t)cell;
  float f[24];
#pragma unroll
  for (int k = 0; k < 6; ++k) {
    const float4 a = __ldg(q + k);
    f[4 * k] = a.x;
    f[4 * k + 1] = a.y;
    f[4 * k + 2] = a.z;
    f[4 * k + 3] = a.w;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    g.c[k][0] = f[3 * k];
    g.c[k][1] = f[3 * k + 1];
    g.c[k][2] = f[3 * k + 2];
  }
}

// Value of the vertex field of cell `cell` at (r, s, t).
__device__ __forceinline__ float hex_value(const DomainDev &dm, int cell, float r, float s, float t)
{
  const float4 *q = dm.hex_coef + 8 * (int64_t)cell + 6;
  const float4 a = __ldg(q), b = __ldg(q + 1);   // w0..w3, w4..w7
  const float rs = r * s;
  return fmaf(fmaf(b.w, t, b.x), rs,
              fmaf(b.z, s * t, fmaf(b.y, r * t, fmaf(a.w, t, fmaf(a.z, s, fmaf(a.y, r, a.x))))));
}

// Newton's method on x(r,s,t) - p = 0 from the guess in rst: 1 when it
// converged inside the element, 0 when it converged outside (rst then holds
// the reference coordinates of p, outside [0,1]^3), -1 when it failed.
// When it converged and `step` is given, drst receives J^-1 step with the
// last Jacobian: the change of rst over a world-space displacement `step`
// (the next sample's guess along a ray). `loose` selects the kHexLooseTol
// acceptance (the march's solves from an extrapolated guess; point location
// from the cell centre keeps kHexNewtonTol).
__device__ __forceinline__ int hex_newton_status(const HexGeom &geo, const float p[3],
                                                 float rst[3], const float *step = nullptr,
                                                 float *drst = nullptr, bool loose = false)
{
  float r = rst[0], s = rst[1], t = rst[2];
  bool conv = false;
  const float (&cx)[8][3] = geo.c;
  for (int it = 0; it < kHexNewtonSteps; ++it) {
    const float rs = r * s, rt = r * t, st = s * t, rst_ = rs * t;
    float F[3], J[3][3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
      F[a] = fmaf(cx[7][a], rst_, fmaf(cx[6][a], st, fmaf(cx[5][a], rt, fmaf(cx[4][a], rs,
             fmaf(cx[3][a], t, fmaf(cx[2][a], s, fmaf(cx[1][a], r, cx[0][a] - p[a])))))));
      J[a][0] = fmaf(cx[7][a], st, fmaf(cx[5][a], t, fmaf(cx[4][a], s, cx[1][a])));
      J[a][1] = fmaf(cx[7][a], rt, fmaf(cx[6][a], t, fmaf(cx[4][a], r, cx[2][a])));
      J[a][2] = fmaf(cx[7][a], rs, fmaf(cx[6][a], s, fmaf(cx[5][a], r, cx[3][a])));
    }
    // solve J d = F by the adjugate
    const float c00 = J[1][1] * J[2][2] - J[1][2] * J[2][1];
    const float c01 = J[1][2] * J[2][0] - J[1][0] * J[2][2];
    const float c02 = J[1][0] * J[2][1] - J[1][1] * J[2][0];
    const float det = J[0][0] * c00 + J[0][1] * c01 + J[0][2] * c02;
    if (!(fabsf(det) > 0.f)) return -1;
    const float id = 1.f / det;
    const float c10 = J[0][2] * J[2][1] - J[0][1] * J[2][2];
    const float c11 = J[0][0] * J[2][2] - J[0][2] * J[2][0];
    const float c12 = J[0][1] * J[2][0] - J[0][0] * J[2][1];
    const float c20 = J[0][1] * J[1][2] - J[0][2] * J[1][1];
    const float c21 = J[0][2] * J[1][0] - J[0][0] * J[1][2];
    const float c22 = J[0][0] * J[1][1] - J[0][1] * J[1][0];
    const float d0 = (c00 * F[0] + c10 * F[1] + c20 * F[2]) * id;
    const float d1 = (c01 * F[0] + c11 * F[1] + c21 * F[2]) * id;
    const float d2 = (c02 * F[0] + c12 * F[1] + c22 * F[2]) * id;
    r -= d0;
    s -= d1;
    t -= d2;
    if (!(fabsf(r) < 1e3f && fabsf(s) < 1e3f && fabsf(t) < 1e3f)) return -1;
    const float dmax = fmaxf(fabsf(d0), fmaxf(fabsf(d1), fabsf(d2)));
    if (dmax < (loose ? kHexLooseTol : kHexNewtonTol)) {
      conv = true;
      if (step) {
        drst[0] = (c00 * step[0] + c10 * step[1] + c20 * step[2]) * id;
        drst[1] = (c01 * step[0] + c11 * step[1] + c21 * step[2]) * id;
        drst[2] = (c02 * step[0] + c12 * step[1] + c22 * step[2]) * id;
      }
      break;
    }
  }
  rst[0] = r;
  rst[1] = s;
  rst[2] = t;
  if (!conv) return -1;
  return r >= -kHexInsideTol && r <= 1.f + kHexInsideTol && s >= -kHexInsideTol &&
         s <= 1.f + kHexInsideTol && t >= -kHexInsideTol && t <= 1.f + kHexInsideTol;
}

__device__ __forceinline__ bool hex_newton(const HexGeom &geo, const float p[3], float rst[3])
{
  return hex_newton_status(geo, p, rst) == 1;
}

// Face through which reference coordinates rst (outside the element) leave
// it: the most violated bound, numbered r=0, r=1, s=0, s=1, t=0, t=1.
__device__ __forceinline__ int hex_exit_face(const float rst[3])
{
  int face = 0;
  float worst = -rst[0];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    if (-rst[a] > worst) { worst = -rst[a]; face = 2 * a; }
    if (rst[a] - 1.f > worst) { worst = rst[a] - 1.f; face = 2 * a + 1; }
  }
  return face;
}

__device__ __forceinline__ bool in_box(const float p[3], float lx, float ly, float lz, float hx,
                                       float hy, float hz)
{
  return !(p[0] < lx || p[1] < ly || p[2] < lz || p[0] > hx || p[1] > hy || p[2] > hz);
}

// Locate p: returns the cell id (or -1) and fills rst and the cell's
// position coefficients.
__device__ __forceinline__ int hex_locate(const DomainDev &dm, const float p[3], float rst[3],
                                          HexGeom &v)
{
  if (dm.n_cells == 1) {
    hex_load(dm, 0, v);
    rst[0] = rst[1] = rst[2] = 0.5f;
    return hex_newton(v, p, rst) ? 0 : -1;
  }
  int stack[kHexStack];
  int sp = 0;
  int node = 0;
  for (;;) {
    if (node >= 0) {
      const float4 *q = dm.hex_bvh + 4 * (int64_t)node;
      const float4 a = __ldg(q), b = __ldg(q + 1), c = __ldg(q + 2), ch = __ldg(q + 3);
      const bool inl = in_box(p, a.x, a.y, a.z, a.w, b.x, b.y);
      const bool inr = in_box(p, b.z, b.w, c.x, c.y, c.z, c.w);
      if (!inl && !inr) {
        if (sp == 0) return -1;
        node = stack[--sp];
        continue;
      }
      const int lc = __float_as_int(ch.x), rc = __float_as_int(ch.y);
      if (inl && inr) {
        if (sp < kHexStack) stack[sp++] = rc;
        node = lc;
      } else {
        node = inl ? lc : rc;
      }
    } else {
      const int k = -node - 1;
      const int cell = __ldg(dm.hex_ids + k);
      hex_load(dm, cell, v);
      rst[0] = rst[1] = rst[2] = 0.5f;
      if (hex_newton(v, p, rst)) return cell;
      if (sp == 0) return -1;
      node = stack[--sp];
    }
  }
}

}  // namespace gvr
