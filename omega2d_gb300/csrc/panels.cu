// panels.cu -- constant-strength panel influence: panels -> points, points -> panels, the
// panel-on-panel influence matrix and the BEM right-hand side.
//
// Reference: kernelu_1v_0p / kernelu_1vs_0p / kernelu_1vos_0p (src/Kernels.h:311-458),
// panels_affect_points (src/Influence.h:422-614), points_affect_panels (:633-771),
// panels_on_panels_coeff (src/Coefficients.h:155-427), vels_to_rhs_panels (src/RHS.h:54-115).
//
// Pair arithmetic is FP32 like the reference, with accuracy changes that leave the mathematics
// unchanged: the subtended angle is one atan2 of (cross, dot) instead of the difference of two
// atan2 values, with the cross product taken against the panel vector, and
// 0.5*log(r0^2/r1^2) is formed from the exactly computed difference r0^2 - r1^2 (log1p, or
// atanh of (rho-1)/(rho+1)).  These remove cancellations the reference suffers at distant
// targets.
#include <algorithm>
#include <cstring>

#include "obs_context.h"
#include "obs_device.cuh"
#include "panels.h"

namespace obs {

namespace {

constexpr int PAN_THREADS = 128;
constexpr int PAN_TILE = 128;           // panels (or particles) per shared-memory tile
constexpr int PAN_COMP_BLOCK = 32;
constexpr int PAN_TPB = 2 * PAN_THREADS;   // targets per block: two per thread

// Per panel: P = (x0, y0, x1, y1), Q = (ux, uy, vortex strength, source strength), where
// (ux, uy) is the unit tangent node0 -> node1 formed as the reference does (px * rsqrt(panl),
// src/Kernels.h:380-384).  Padded panels are far away with zero strength.
__global__ void pack_panels_kernel(const float* __restrict__ nx, const float* __restrict__ ny,
                                   const unsigned* __restrict__ idx, int nnodes,
                                   const float* __restrict__ vs, const float* __restrict__ ss,
                                   int np, int np_pad, float4* __restrict__ P, float4* __restrict__ Q,
                                   float* __restrict__ len, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np_pad) return;
  if (i >= np) {
    P[i] = make_float4(1.0e6f, 1.0e6f, 1.0e6f + 1.0f, 1.0e6f);
    Q[i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    if (len) len[i] = 1.0f;
    return;
  }
  unsigned j0 = idx[2 * i], j1 = idx[2 * i + 1];
  if (j0 >= (unsigned)nnodes || j1 >= (unsigned)nnodes) {
    record_failure(status, DEV_ERR_BOUNDS, 301, i, (int)max(j0, j1));
    P[i] = make_float4(1.0e6f, 1.0e6f, 1.0e6f + 1.0f, 1.0e6f);
    Q[i] = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
    if (len) len[i] = 1.0f;
    return;
  }
  const float x0 = nx[j0], y0 = ny[j0], x1 = nx[j1], y1 = ny[j1];
  const float px = x1 - x0, py = y1 - y0;
  const float panl = px * px + py * py;
  const float m = 1.0f / sqrtf(panl);
  P[i] = make_float4(x0, y0, x1, y1);
  Q[i] = make_float4(px * m, py * m, vs ? vs[i] : 0.0f, ss ? ss[i] : 0.0f);
  if (len) len[i] = sqrtf(panl);
}

// ---- the subtended angle u* and log ratio v* of a panel seen from a target (get_ustar and
// my_halflog(rij2/rij12) of src/Kernels.h:256-268, 330-338), in forms that need few
// instructions: a polynomial arctangent of (cross, dot) with the cross product taken against
// the panel vector, and the half-log as atanh of s = (rho-1)/(rho+1), rho = r0^2/r1^2, from its
// odd series where |s| <= 0.2 (every target more than a few panel lengths from the panel),
// else log1p of the exactly formed (r0^2 - r1^2)/r1^2 or the ratio itself near node 0.  Both
// keep full relative accuracy at small angles and logs.

__device__ __forceinline__ float rcp_approx(float x) {
  float y;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

// u* and v* of a panel seen from a target, for two (panel, target) pairs at once in f32x2
// register pairs (FADD2 / FMUL2 / FFMA2 for the arithmetic; per-lane reciprocals, selects and
// the rare near-panel fix-up).  atan on [0, 1] is r * P(r^2) with P of degree 8 fitted to
// atan(r)/r for minimum maximum relative error (omega2d_gb300/poly_fit.py; 1.5e-7 relative in
// FP32), reflected into the octant of (cross, dot).
__device__ __forceinline__ float2 sub2(float2 a, float2 b) { return __ffma2_rn(b, f2(-1.0f, -1.0f), a); }

__device__ __forceinline__ float atan2_fix(float p, float y, float x, float ay, float ax) {
  p = (ay > ax) ? 1.57079632679f - p : p;
  p = (x < 0.0f) ? 3.14159265359f - p : p;
  return copysignf(p, y);
}

__device__ __forceinline__ float half_log_near(float dx0, float dy0, float r1, float diff) {
  const float q = diff / r1;
  return (q > -0.5f) ? 0.5f * log1pf(q) : 0.5f * logf((dx0 * dx0 + dy0 * dy0) / r1);
}

__device__ __forceinline__ void panel_uv_star_fast2(float2 x0, float2 y0, float2 x1, float2 y1, float2 px, float2 py,
                                                    float2 tx, float2 ty, float2& us, float2& vs) {
  const float2 dx0 = sub2(tx, x0), dy0 = sub2(ty, y0);
  const float2 dx1 = sub2(tx, x1), dy1 = sub2(ty, y1);
  const float2 cr = sub2(__fmul2_rn(dx0, py), __fmul2_rn(dy0, px));     // (t - p0) x (p1 - p0)
  const float2 dt = __ffma2_rn(dx0, dx1, __fmul2_rn(dy0, dy1));
  // the half-log's operands: r1^2, r0^2 - r1^2 formed exactly, and r0^2 + r1^2
  const float2 r1 = __ffma2_rn(dx1, dx1, __fmul2_rn(dy1, dy1));
  const float2 diff = __ffma2_rn(px, __fadd2_rn(dx0, dx1), __fmul2_rn(py, __fadd2_rn(dy0, dy1)));
  const float2 den = __ffma2_rn(f2(2.0f, 2.0f), r1, diff);
  if (fabsf(cr.x) < 0.05f * dt.x && fabsf(cr.y) < 0.05f * dt.y && fabsf(diff.x) < 0.05f * den.x &&
      fabsf(diff.y) < 0.05f * den.y) {
    // both targets more than about twenty panel lengths away: the arctangent ratio and the
    // atanh argument are below 0.05, where both odd series end at the 5th power (the next
    // term is below 2.3e-9 relative)
    const float2 r = __fmul2_rn(cr, f2(rcp_approx(dt.x), rcp_approx(dt.y)));
    const float2 sv = __fmul2_rn(diff, f2(rcp_approx(den.x), rcp_approx(den.y)));
    const float2 t = __fmul2_rn(r, r), ts = __fmul2_rn(sv, sv);
    us = __ffma2_rn(__fmul2_rn(r, t), __ffma2_rn(t, f2(0.2f, 0.2f), f2(-1.0f / 3.0f, -1.0f / 3.0f)), r);
    vs = __ffma2_rn(__fmul2_rn(sv, ts), __ffma2_rn(ts, f2(0.2f, 0.2f), f2(1.0f / 3.0f, 1.0f / 3.0f)), sv);
    return;
  }
  if (fabsf(cr.x) < 0.2f * dt.x && fabsf(cr.y) < 0.2f * dt.y) {
    // both targets see the panel under less than atan(0.2) from in front (every target more
    // than a few panel lengths away): atan of the signed ratio by its odd Taylor series to
    // r^9 (truncation below 1e-8 relative), no octant reflection
    const float2 r = __fmul2_rn(cr, f2(rcp_approx(dt.x), rcp_approx(dt.y)));
    const float2 t = __fmul2_rn(r, r);
    float2 p = __ffma2_rn(t, f2(1.0f / 9.0f, 1.0f / 9.0f), f2(-1.0f / 7.0f, -1.0f / 7.0f));
    p = __ffma2_rn(p, t, f2(1.0f / 5.0f, 1.0f / 5.0f));
    p = __ffma2_rn(p, t, f2(-1.0f / 3.0f, -1.0f / 3.0f));
    us = __ffma2_rn(__fmul2_rn(r, t), p, r);
  } else {
    // arctangent: |min|/|max| per lane, the polynomial packed
    const float ax0 = fabsf(dt.x), ay0 = fabsf(cr.x), ax1 = fabsf(dt.y), ay1 = fabsf(cr.y);
    const float mx0 = fmaxf(ax0, ay0), mx1 = fmaxf(ax1, ay1);
    const float2 r = f2((mx0 > 0.0f) ? fminf(ax0, ay0) * rcp_approx(mx0) : 0.0f,
                        (mx1 > 0.0f) ? fminf(ax1, ay1) * rcp_approx(mx1) : 0.0f);
    const float2 t = __fmul2_rn(r, r);
    float2 p = __ffma2_rn(f2(2.849889686e-03f, 2.849889686e-03f), t, f2(-1.606862992e-02f, -1.606862992e-02f));
    p = __ffma2_rn(p, t, f2(4.269152135e-02f, 4.269152135e-02f));
    p = __ffma2_rn(p, t, f2(-7.504294813e-02f, -7.504294813e-02f));
    p = __ffma2_rn(p, t, f2(1.064093411e-01f, 1.064093411e-01f));
    p = __ffma2_rn(p, t, f2(-1.420364380e-01f, -1.420364380e-01f));
    p = __ffma2_rn(p, t, f2(1.999261975e-01f, 1.999261975e-01f));
    p = __ffma2_rn(p, t, f2(-3.333307207e-01f, -3.333307207e-01f));
    p = __ffma2_rn(p, t, f2(1.0f, 1.0f));
    p = __fmul2_rn(r, p);
    us = f2(atan2_fix(p.x, cr.x, dt.x, ay0, ax0), atan2_fix(p.y, cr.y, dt.y, ay1, ax1));
  }
  // half-log: atanh series of (rho - 1)/(rho + 1)
  const float2 sv = __fmul2_rn(diff, f2(rcp_approx(den.x), rcp_approx(den.y)));
  const float2 ts = __fmul2_rn(sv, sv);
  float2 q = __ffma2_rn(ts, f2(1.0f / 9.0f, 1.0f / 9.0f), f2(1.0f / 7.0f, 1.0f / 7.0f));
  q = __ffma2_rn(q, ts, f2(1.0f / 5.0f, 1.0f / 5.0f));
  q = __ffma2_rn(q, ts, f2(1.0f / 3.0f, 1.0f / 3.0f));
  vs = __ffma2_rn(__fmul2_rn(sv, ts), q, sv);
  if (!(fabsf(sv.x) <= 0.2f)) vs.x = half_log_near(dx0.x, dy0.x, r1.x, diff.x);
  if (!(fabsf(sv.y) <= 0.2f)) vs.y = half_log_near(dx0.y, dy0.y, r1.y, diff.y);
}

struct PanArgs {
  const float* gx;      // the panel set: node coordinates, node-index pairs (mode 0: the
  const float* gy;      //   sources, padded to nsrc with far panels of zero strength; modes 1
  const unsigned* gidx; //   and 2: the targets)
  int nnodes;
  int npan;
  const float* gvs;     // vortex and source strengths (mode 0; either may be null)
  const float* gss;
  int* status;
  const float4* pts;    // packed cotangent points (x, y, lu, lv) for mode 2
  const float* sx;      // the particles of mode 1, read directly (nreal of them; the padding
  const float* sy;      //   up to nsrc is far away with zero strength)
  const float* ss;
  int nreal;
  int nsrc;             // panels (pan->pt) or particles (pt->pan), padded count
  int nblk;             // 32-source blocks (nsrc / 32)
  const float* tx;
  const float* ty;
  int nt;               // targets (points or panels)
  int nsplit;
  int blks_per_split;
  float* out_u;
  float* out_v;
  void* part;
  int finalize;
  double fsx, fsy;
  int mode;             // 0: panels -> points, 1: points -> panels, 2: VJP of mode 0 w.r.t. the
                        //    panel strengths (sources = points with their cotangents)
};

// Panel j of the set as pack_panels_kernel forms it: P = (x0, y0, x1, y1), Q = (unit tangent,
// strengths), len; an index past npan is a far panel of zero strength, a node index out of
// range records DEV_ERR_BOUNDS (code 301) and gives the same far panel
__device__ __forceinline__ void panel_geom(const PanArgs& a, int j, float4& P, float4& Q, float& len) {
  P = make_float4(1.0e6f, 1.0e6f, 1.0e6f + 1.0f, 1.0e6f);
  Q = make_float4(1.0f, 0.0f, 0.0f, 0.0f);
  len = 1.0f;
  if (j >= a.npan) return;
  const unsigned j0 = a.gidx[2 * j], j1 = a.gidx[2 * j + 1];
  if (j0 >= (unsigned)a.nnodes || j1 >= (unsigned)a.nnodes) {
    record_failure(a.status, DEV_ERR_BOUNDS, 301, j, (int)max(j0, j1));
    return;
  }
  const float x0 = a.gx[j0], y0 = a.gy[j0], x1 = a.gx[j1], y1 = a.gy[j1];
  const float px = x1 - x0, py = y1 - y0;
  const float panl = px * px + py * py;
  const float m = 1.0f / sqrtf(panl);
  P = make_float4(x0, y0, x1, y1);
  Q = make_float4(px * m, py * m, a.gvs ? a.gvs[j] : 0.0f, a.gss ? a.gss[j] : 0.0f);
  len = sqrtf(panl);
}

__device__ __forceinline__ void pan_store(const PanArgs& a, int i, double su, double sv) {
  const double f = a.finalize ? 0.15915494309189535 : 1.0;
  const double fx = a.finalize ? a.fsx : 0.0, fy = a.finalize ? a.fsy : 0.0;
  a.out_u[i] = (float)(((double)a.out_u[i] + su) * f + fx);
  a.out_v[i] = (float)(((double)a.out_v[i] + sv) * f + fy);
}

// The per-target steps after the sum over sources, then the store: (ux, uy) is the target
// panel's unit tangent and tinv its inverse length (modes 1 and 2)
__device__ __forceinline__ void pan_finish(const PanArgs& a, int i, double su, double sv, float tux, float tuy,
                                           float tinv) {
  if (a.mode == 1) {
    // (sum w u*, sum w v*) -> velocity along the fixed tangent, times -1/len
    const double ux = tux, uy = tuy;
    const double vu = su * ux - sv * uy, vv = su * uy + sv * ux;
    su = -vu * (double)tinv;
    sv = -vv * (double)tinv;
  } else if (a.mode == 2) {
    // A = g tx + s ty, B = s tx - g ty: dL/dg = tx P + ty Q, dL/ds = ty P - tx Q, times the
    // finalize factor 1/(2 pi) (the gradients are of the finalized velocities)
    const double ux = tux, uy = tuy;
    const double gg = (ux * su + uy * sv) * 0.15915494309189535, gs = (uy * su - ux * sv) * 0.15915494309189535;
    su = gg;
    sv = gs;
  }
  pan_store(a, i, su, sv);
}

// Two targets per thread (h = 0, 1: targets blockIdx.x PAN_TPB + h PAN_THREADS + tid) in
// f32x2 register pairs; sources (panels or particles) staged through shared memory; grid =
// (target blocks, source splits).  Compensated: FP32 partials over 32 sources folded into
// two-sum pairs, FP64 out; plain: FP32 throughout.
//   panels -> points: with the panel's unit tangent (tx, ty) and strengths (g, s), the sheet
//     velocity (kernelu_1vs_0p) is u = u* A + v* B, v = v* A - u* B with A = g tx + s ty,
//     B = s tx - g ty, formed once per panel when the tile is staged;
//   points -> panels: the target panel's tangent is fixed per thread, so the particle sums
//     are of w u* and w v* and the tangent is applied once at the end.
template <bool COMP>
__global__ void __launch_bounds__(PAN_THREADS) pan_kernel(const PanArgs a) {
  // sources pre-duplicated for the packed operands: panels (x0,x0,y0,y0) (x1,x1,y1,y1)
  // (px,px,py,py) (A,A,B,B); particles (x,x,y,y) (w,w,0,0)
  __shared__ float4 sE[PAN_TILE][4];
  const int sp = blockIdx.y;
  int ti[2];
  float tx[2] = {0.0f, 0.0f}, ty[2] = {0.0f, 0.0f}, tinv[2] = {0.0f, 0.0f};
  float4 TP[2], TQ[2];
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    ti[h] = blockIdx.x * PAN_TPB + h * PAN_THREADS + threadIdx.x;
    const int ic = ti[h] < a.nt ? ti[h] : a.nt - 1;
    TP[h] = TQ[h] = make_float4(0, 0, 0, 0);
    if (a.mode == 0) {
      tx[h] = a.tx[ic];
      ty[h] = a.ty[ic];
    } else {
      float len;
      panel_geom(a, ic, TP[h], TQ[h], len);
      tinv[h] = 1.0f / len;
    }
  }
  const float2 T2x = f2(tx[0], tx[1]), T2y = f2(ty[0], ty[1]);
  const float2 X0 = f2(TP[0].x, TP[1].x), Y0 = f2(TP[0].y, TP[1].y);
  const float2 X1 = f2(TP[0].z, TP[1].z), Y1 = f2(TP[0].w, TP[1].w);
  const float2 PX = sub2(X1, X0), PY = sub2(Y1, Y0);
  const float2 z2 = f2(0.0f, 0.0f);
  float2 au = z2, av = z2, hu = z2, lu = z2, hv = z2, lv = z2;
  // this split's 32-source blocks [b0, b1), staged PAN_TILE sources at a time
  const int b0 = sp * a.blks_per_split;
  const int b1 = min(b0 + a.blks_per_split, a.nblk);
  for (int base = b0; base < b1; base += PAN_TILE / PAN_COMP_BLOCK) {
    const int ns = min(PAN_TILE, (b1 - base) * PAN_COMP_BLOCK);
    __syncthreads();
    for (int k = threadIdx.x; k < ns; k += PAN_THREADS) {
      const int j = base * PAN_COMP_BLOCK + k;
      if (a.mode == 0) {
        float4 P, Q;
        float len;
        panel_geom(a, j, P, Q, len);
        const float px = P.z - P.x, py = P.w - P.y;
        const float A = Q.z * Q.x + Q.w * Q.y, B = Q.w * Q.x - Q.z * Q.y;
        sE[k][0] = make_float4(P.x, P.x, P.y, P.y);
        sE[k][1] = make_float4(P.z, P.z, P.w, P.w);
        sE[k][2] = make_float4(px, px, py, py);
        sE[k][3] = make_float4(A, A, B, B);
      } else {
        // (x, y, 0, strength) or, mode 2, (x, y, lu, lv)
        const float4 q = (a.mode == 2) ? a.pts[j]
                         : (j < a.nreal) ? make_float4(a.sx[j], a.sy[j], 0.0f, a.ss[j])
                                         : make_float4(1.0e6f, 1.0e6f, 0.0f, 0.0f);
        sE[k][0] = make_float4(q.x, q.x, q.y, q.y);
        sE[k][1] = (a.mode == 1) ? make_float4(q.w, q.w, 0.0f, 0.0f) : make_float4(q.z, q.z, q.w, q.w);
      }
    }
    __syncthreads();
    for (int b = 0; b < ns; b += PAN_COMP_BLOCK) {
      if (a.mode == 0) {
#pragma unroll 2
        for (int k = 0; k < PAN_COMP_BLOCK; ++k) {
          const float4 E0 = sE[b + k][0], E1 = sE[b + k][1], E2 = sE[b + k][2], E3 = sE[b + k][3];
          float2 us, vs;
          panel_uv_star_fast2(f2(E0.x, E0.y), f2(E0.z, E0.w), f2(E1.x, E1.y), f2(E1.z, E1.w), f2(E2.x, E2.y),
                              f2(E2.z, E2.w), T2x, T2y, us, vs);
          const float2 A = f2(E3.x, E3.y), B = f2(E3.z, E3.w);
          au = __ffma2_rn(us, A, __ffma2_rn(vs, B, au));
          av = __ffma2_rn(vs, A, sub2(av, __fmul2_rn(us, B)));
        }
      } else if (a.mode == 1) {
        // the panel is the "source" of kernelu_1v_0p with the particle strength, the particle
        // the "target"; the sum is used with a minus sign (src/Influence.h:737-759)
#pragma unroll 2
        for (int k = 0; k < PAN_COMP_BLOCK; ++k) {
          const float4 E0 = sE[b + k][0], E1 = sE[b + k][1];
          float2 us, vs;
          panel_uv_star_fast2(X0, Y0, X1, Y1, PX, PY, f2(E0.x, E0.y), f2(E0.z, E0.w), us, vs);
          const float2 w = f2(E1.x, E1.y);
          au = __ffma2_rn(w, us, au);
          av = __ffma2_rn(w, vs, av);
        }
      } else {
        // VJP of the sheet velocity u = u* A + v* B, v = v* A - u* B at a point with cotangent
        // (lu, lv): P = sum lu u* + lv v*, Q = sum lv u* - lu v*; dL/dA = P, dL/dB = -Q
#pragma unroll 2
        for (int k = 0; k < PAN_COMP_BLOCK; ++k) {
          const float4 E0 = sE[b + k][0], E1 = sE[b + k][1];
          float2 us, vs;
          panel_uv_star_fast2(X0, Y0, X1, Y1, PX, PY, f2(E0.x, E0.y), f2(E0.z, E0.w), us, vs);
          const float2 lu = f2(E1.x, E1.y), lv = f2(E1.z, E1.w);
          au = __ffma2_rn(lu, us, __ffma2_rn(lv, vs, au));
          av = __ffma2_rn(lv, us, sub2(av, __fmul2_rn(lu, vs)));
        }
      }
      if (COMP) {
        two_sum2(hu, lu, au);
        two_sum2(hv, lv, av);
        au = z2;
        av = z2;
      }
    }
  }
#pragma unroll
  for (int h = 0; h < 2; ++h) {
    const int i = ti[h];
    if (i >= a.nt) continue;
    if (a.nsplit > 1) {
      // this split's raw sums (double-float when compensated); the reduction applies the
      // per-target steps below once to their total
      if (COMP) {
        float2* p = static_cast<float2*>(a.part);
        p[(size_t)sp * a.nt + i] = make_float2(h ? hu.y : hu.x, h ? lu.y : lu.x);
        p[((size_t)a.nsplit + sp) * a.nt + i] = make_float2(h ? hv.y : hv.x, h ? lv.y : lv.x);
      } else {
        float* p = static_cast<float*>(a.part);
        p[(size_t)sp * a.nt + i] = h ? au.y : au.x;
        p[((size_t)a.nsplit + sp) * a.nt + i] = h ? av.y : av.x;
      }
      continue;
    }
    const double su = COMP ? (double)(h ? hu.y : hu.x) + (double)(h ? lu.y : lu.x) : (double)(h ? au.y : au.x);
    const double sv = COMP ? (double)(h ? hv.y : hv.x) + (double)(h ? lv.y : lv.x) : (double)(h ? av.y : av.x);
    pan_finish(a, i, su, sv, TQ[h].x, TQ[h].y, tinv[h]);
  }
}

// (hi, lo) += (bh, bl) in double-float
__device__ __forceinline__ void pan_df_add(float& hi, float& lo, float bh, float bl) {
  two_sum_acc(hi, lo, bh);
  lo += bl;
}

// the per-target steps of pan_finish for the target panel of modes 1 and 2 (mode 0: none)
__device__ __forceinline__ void pan_finish_sum(const PanArgs& a, int i, float4 t) {
  const double su = (double)t.x + (double)t.y, sv = (double)t.z + (double)t.w;
  float tux = 0.0f, tuy = 0.0f, tinv = 0.0f;
  if (a.mode != 0) {
    float4 P, Q;
    float len;
    panel_geom(a, i, P, Q, len);
    tux = Q.x;
    tuy = Q.y;
    if (a.mode == 1) tinv = 1.0f / len;
  }
  pan_finish(a, i, su, sv, tux, tuy, tinv);
}

// Sum of the split partials in split order, one thread per target (consecutive threads read
// consecutive targets): double-float sums when compensated; for a few splits
template <bool COMP>
__global__ void pan_reduce_kernel(const PanArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nt) return;
  float4 t = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  if (COMP) {
    const float2* p = static_cast<const float2*>(a.part);
    for (int k = 0; k < a.nsplit; ++k) {
      const float2 u = p[(size_t)k * a.nt + i], v = p[((size_t)a.nsplit + k) * a.nt + i];
      pan_df_add(t.x, t.y, u.x, u.y);
      pan_df_add(t.z, t.w, v.x, v.y);
    }
  } else {
    const float* p = static_cast<const float*>(a.part);
    for (int k = 0; k < a.nsplit; ++k) {
      t.x += p[(size_t)k * a.nt + i];
      t.z += p[((size_t)a.nsplit + k) * a.nt + i];
    }
  }
  pan_finish_sum(a, i, t);
}

// The same for many splits (few targets): a block takes 32 consecutive targets (lane = target,
// so every load of a warp is 256 contiguous bytes) and its PAN_RED_WARPS warps take every
// PAN_RED_WARPS-th split; the warps' sums are added in warp order, so the result does not
// depend on timing
constexpr int PAN_RED_WARPS = 32;
template <bool COMP>
__global__ void __launch_bounds__(32 * PAN_RED_WARPS) pan_reduce_wide_kernel(const PanArgs a) {
  __shared__ float4 red[PAN_RED_WARPS][32];
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int i = blockIdx.x * 32 + lane;
  const int ic = i < a.nt ? i : a.nt - 1;
  float hu = 0.0f, lu = 0.0f, hv = 0.0f, lv = 0.0f;
  if (COMP) {
    const float2* p = static_cast<const float2*>(a.part);
#pragma unroll 4
    for (int k = wp; k < a.nsplit; k += PAN_RED_WARPS) {
      const float2 u = p[(size_t)k * a.nt + ic], v = p[((size_t)a.nsplit + k) * a.nt + ic];
      pan_df_add(hu, lu, u.x, u.y);
      pan_df_add(hv, lv, v.x, v.y);
    }
  } else {
    const float* p = static_cast<const float*>(a.part);
#pragma unroll 4
    for (int k = wp; k < a.nsplit; k += PAN_RED_WARPS) {
      hu += p[(size_t)k * a.nt + ic];
      hv += p[((size_t)a.nsplit + k) * a.nt + ic];
    }
  }
  red[wp][lane] = make_float4(hu, lu, hv, lv);
  __syncthreads();
  if (wp != 0 || i >= a.nt) return;
  float4 t = red[0][lane];
  for (int w = 1; w < PAN_RED_WARPS; ++w) {
    const float4 q = red[w][lane];
    if (COMP) {
      pan_df_add(t.x, t.y, q.x, q.y);
      pan_df_add(t.z, t.w, q.z, q.w);
    } else {
      t.x += q.x;
      t.z += q.z;
    }
  }
  pan_finish_sum(a, i, t);
}

__global__ void pack_cotangents_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                       const float* __restrict__ lu, const float* __restrict__ lv, int n, int n_pad,
                                       float4* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n_pad) return;
  out[i] = i < n ? make_float4(x[i], y[i], lu[i], lv[i]) : make_float4(1.0e6f, 1.0e6f, 0.0f, 0.0f);
}

// Particles -> float4 (x, y, 0, strength), padded with zero-strength particles far away.
// float -> double from the bits (exact): float->double conversions run on the slow FP64 path of
// this GPU; zero and normal values are rebiased with integer operations, anything else (a
// subnormal, infinity or NaN) takes the hardware conversion
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned b = __float_as_uint(f);
  const unsigned e = (b >> 23) & 0xff;
  const unsigned long long sign = (unsigned long long)(b >> 31) << 63;
  if ((b & 0x7fffffffu) == 0) return __longlong_as_double((long long)sign);
  if (e == 0 || e == 0xff) return (double)f;
  const unsigned long long d = sign | ((unsigned long long)(e - 127 + 1023) << 52) |
                               ((unsigned long long)(b & 0x7fffffu) << 29);
  return __longlong_as_double((long long)d);
}

// panels_on_panels_coeff: one thread per (target panel i, source panel j); column-major output
// with targets as rows (src/Coefficients.h:155-427).  Unit-strength influence of source j at
// the midpoint of target i, dotted with target i's tangent and normal, averaged with the
// reversed evaluation weighted by len_j/len_i, the self block set to pi, all times 1/(2 pi).
__global__ void coeff_kernel(const float4* __restrict__ SP, const float4* __restrict__ SQ,
                             const float* __restrict__ SL, int nsrc,
                             const float4* __restrict__ TP, const float4* __restrict__ TQ,
                             const float* __restrict__ TL, int ntarg, int nunk, int self,
                             float* __restrict__ A32, double* __restrict__ A64) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int j = blockIdx.y;
  if (i >= ntarg || j >= nsrc) return;
  const float4 sp = SP[j], sq = SQ[j];
  const float4 tp = TP[i], tq = TQ[i];
  const float ttx = tq.x, tty = tq.y;        // target tangent
  const float tnx = -tq.y, tny = tq.x;       // target normal (left of node0 -> node1)
  const float xi = 0.5f * (tp.z + tp.x), yi = 0.5f * (tp.w + tp.y);
  const float xj = 0.5f * (sp.x + sp.z), yj = 0.5f * (sp.y + sp.w);
  // both evaluations in one packed call: lane x = source panel j at the midpoint of i, lane y =
  // target panel i at the midpoint of j (the reversed roles below)
  float2 us2, vs2;
  panel_uv_star_fast2(f2(sp.x, tp.x), f2(sp.y, tp.y), f2(sp.z, tp.z), f2(sp.w, tp.w), f2(sp.z - sp.x, tp.z - tp.x),
                      f2(sp.w - sp.y, tp.w - tp.y), f2(xi, xj), f2(yi, yj), us2, vs2);
  float us = us2.x, vs = vs2.x;
  float vu = us * sq.x - vs * sq.y, vv = us * sq.y + vs * sq.x;
  float c11 = vu * ttx + vv * tty, c12 = vu * tnx + vv * tny;
  float c21 = 0.0f, c22 = 0.0f;
  if (nunk == 2) {
    const float su = us * sq.y + vs * sq.x, sv = vs * sq.y - us * sq.x;
    c21 = su * ttx + sv * tty;
    c22 = su * tnx + sv * tny;
  }
  // reversed roles: target panel as source, evaluated at the source midpoint
  us = us2.y;
  vs = vs2.y;
  const float fact = SL[j] / TL[i];
  vu = us * tq.x - vs * tq.y;
  vv = us * tq.y + vs * tq.x;
  c11 = 0.5f * (c11 - fact * (vu * ttx + vv * tty));
  c12 = 0.5f * (c12 - fact * (vu * tnx + vv * tny));
  if (nunk == 2) {
    const float su = us * tq.y + vs * tq.x, sv = vs * tq.y - us * tq.x;
    c21 = 0.5f * (c21 - fact * (su * ttx + sv * tty));
    c22 = 0.5f * (c22 - fact * (su * tnx + sv * tny));
  }
  if (self && i == j) {
    c11 = (float)M_PI;
    c12 = 0.0f;
    c21 = 0.0f;
    c22 = (float)M_PI;
  }
  const float fac = (float)(1.0 / (2.0 * M_PI));
  c11 *= fac; c12 *= fac; c21 *= fac; c22 *= fac;
  const size_t nrows = (size_t)ntarg * nunk;
  if (nunk == 2) {
    const size_t c0 = (size_t)(2 * j) * nrows + 2 * i, c1 = (size_t)(2 * j + 1) * nrows + 2 * i;
    if (A32) { A32[c0] = c11; A32[c0 + 1] = c12; A32[c1] = c21; A32[c1 + 1] = c22; }
    if (A64) {
      A64[c0] = f2d_bits(c11);
      A64[c0 + 1] = f2d_bits(c12);
      A64[c1] = f2d_bits(c21);
      A64[c1 + 1] = f2d_bits(c22);
    }
  } else {
    const size_t c0 = (size_t)j * nrows + i;
    if (A32) A32[c0] = c11;
    if (A64) A64[c0] = f2d_bits(c11);
  }
}

// vels_to_rhs_panels (src/RHS.h:54-115): rhs = -u.t (and -u.n + bc_n for two unknowns), into
// rhs32 and / or rhs64; the unit tangent formed from the panel's nodes as pack_panels_kernel
// forms it
__global__ void rhs_kernel(const float* __restrict__ nx, const float* __restrict__ ny,
                           const unsigned* __restrict__ idx, int nnodes, const float* __restrict__ pu,
                           const float* __restrict__ pv, const float* __restrict__ bcn, int np, int nunk,
                           float* __restrict__ rhs32, double* __restrict__ rhs64, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= np) return;
  const unsigned j0 = idx[2 * i], j1 = idx[2 * i + 1];
  float qx = 1.0f, qy = 0.0f;
  if (j0 >= (unsigned)nnodes || j1 >= (unsigned)nnodes) {
    record_failure(status, DEV_ERR_BOUNDS, 301, i, (int)max(j0, j1));
  } else {
    const float px = nx[j1] - nx[j0], py = ny[j1] - ny[j0];
    const float panl = px * px + py * py;
    const float m = 1.0f / sqrtf(panl);
    qx = px * m;
    qy = py * m;
  }
  const float t = -(pu[i] * qx + pv[i] * qy);
  if (nunk == 1) {
    if (rhs32) rhs32[i] = t;
    if (rhs64) rhs64[i] = (double)t;
  } else {
    const float n = -(pu[i] * (-qy) + pv[i] * qx) + (bcn ? bcn[i] : 0.0f);
    if (rhs32) { rhs32[2 * i] = t; rhs32[2 * i + 1] = n; }
    if (rhs64) { rhs64[2 * i] = (double)t; rhs64[2 * i + 1] = (double)n; }
  }
}

}  // namespace

// ------------------------------------------------------------------------------------- host

int pack_panels(obs_context* ctx, const PanelSet& ps, const float* vs, const float* ss, float4* P, float4* Q,
                float* len, int np_pad) {
  const int threads = 256;
  pack_panels_kernel<<<(np_pad + threads - 1) / threads, threads, 0, ctx->stream>>>(
      ps.nx, ps.ny, ps.idx, ps.nnodes, vs, ss, ps.npan, np_pad, P, Q, len, ctx->d_status);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

namespace {

// source splits: enough (target block, split) blocks for ~32 per SM, each split at least one
// 32-source block (small problems -- a few thousand panels -- need the fine splits to fill the
// GPU at all)
int plan_splits(obs_context* ctx, int nblk, int tblocks) {
  const int want = 8 * 4 * ctx->num_sms;
  const int nsplit = std::max(1, (want + tblocks - 1) / tblocks);
  return std::min(nsplit, std::max(1, nblk));
}

void set_panels(PanArgs& a, const PanelSet& ps, const float* vs, const float* ss, obs_context* ctx) {
  a.gx = ps.nx; a.gy = ps.ny; a.gidx = ps.idx; a.nnodes = ps.nnodes; a.npan = ps.npan;
  a.gvs = vs; a.gss = ss;
  a.status = ctx->d_status;
}

int run_pan(obs_context* ctx, PanArgs& a, bool comp, size_t scratch_off) {
  const int tblocks = (a.nt + PAN_TPB - 1) / PAN_TPB;
  int nsplit = plan_splits(ctx, a.nblk, tblocks);
  const int bps = (a.nblk + nsplit - 1) / nsplit;
  nsplit = (a.nblk + bps - 1) / bps;
  a.nsplit = nsplit;
  a.blks_per_split = bps;
  if (nsplit > 1) {
    const size_t bytes = (size_t)2 * nsplit * a.nt * (comp ? sizeof(double) : sizeof(float));
    int s = ctx->work.ensure(scratch_off + bytes, ctx->stream);
    if (s) return s;
    a.part = ctx->work.as<char>(scratch_off);
  }
  // the work buffer may have moved: the caller re-derives packed pointers after ensure
  return OBS_OK;
}

}  // namespace

int launch_pan(obs_context* ctx, PanArgs& a, bool comp) {
  const int tblocks = (a.nt + PAN_TPB - 1) / PAN_TPB;
  dim3 grid(tblocks, a.nsplit);
  timing_main_begin(ctx);
  if (comp) pan_kernel<true><<<grid, PAN_THREADS, 0, ctx->stream>>>(a);
  else pan_kernel<false><<<grid, PAN_THREADS, 0, ctx->stream>>>(a);
  ctx->launches++;
  timing_main_end(ctx);
  cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess && a.nsplit > 16) {
    const unsigned blocks = (unsigned)((a.nt + 31) / 32);
    if (comp) pan_reduce_wide_kernel<true><<<blocks, 32 * PAN_RED_WARPS, 0, ctx->stream>>>(a);
    else pan_reduce_wide_kernel<false><<<blocks, 32 * PAN_RED_WARPS, 0, ctx->stream>>>(a);
    ctx->launches++;
    e = cudaGetLastError();
  } else if (e == cudaSuccess && a.nsplit > 1) {
    if (comp) pan_reduce_kernel<true><<<(a.nt + 255) / 256, 256, 0, ctx->stream>>>(a);
    else pan_reduce_kernel<false><<<(a.nt + 255) / 256, 256, 0, ctx->stream>>>(a);
    ctx->launches++;
    e = cudaGetLastError();
  }
  return cuda_status(e);
}

// panels -> points (panels_affect_points)
int run_panels_affect_points(obs_context* ctx, const PanelSet& ps, const float* vs, const float* ss,
                             int accum, int flags, double fsx, double fsy,
                             int nt, const float* tx, const float* ty, float* tu, float* tv) {
  if (ps.npan == 0 || nt == 0) return OBS_OK;
  const bool comp = accum == OBS_COMPENSATED;
  const int ntiles = (ps.npan + PAN_TILE - 1) / PAN_TILE;
  const int np_pad = ntiles * PAN_TILE;
  const size_t off_part = 256;
  PanArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nsrc = np_pad; a.nblk = np_pad / PAN_COMP_BLOCK;
  a.tx = tx; a.ty = ty; a.nt = nt;
  a.out_u = tu; a.out_v = tv;
  a.finalize = (flags & OBS_FLAG_FINALIZE) ? 1 : 0;
  a.fsx = fsx; a.fsy = fsy;
  a.mode = 0;
  set_panels(a, ps, vs, ss, ctx);
  int s = ctx->work.ensure(off_part, ctx->stream);
  if (!s) s = run_pan(ctx, a, comp, off_part);
  if (s) return s;
  if (a.nsplit > 1) a.part = ctx->work.as<char>(off_part);
  timing_begin(ctx);
  s = launch_pan(ctx, a, comp);
  timing_end(ctx);
  return s;
}

// points -> panels (points_affect_panels): mean velocity on each panel due to the particles
int run_points_affect_panels(obs_context* ctx, int ns, const float* sx, const float* sy, const float* ss,
                             const PanelSet& ps, int accum, int flags, double fsx, double fsy,
                             float* pu, float* pv) {
  if (ps.npan == 0 || ns == 0) return OBS_OK;
  const bool comp = accum == OBS_COMPENSATED;
  const int ntiles = (ns + PAN_TILE - 1) / PAN_TILE;
  const int ns_pad = ntiles * PAN_TILE;
  const size_t off_part = 256;
  PanArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nsrc = ns_pad; a.nblk = ns_pad / PAN_COMP_BLOCK;
  a.nt = ps.npan;
  a.out_u = pu; a.out_v = pv;
  a.finalize = (flags & OBS_FLAG_FINALIZE) ? 1 : 0;
  a.fsx = fsx; a.fsy = fsy;
  a.mode = 1;
  set_panels(a, ps, nullptr, nullptr, ctx);
  a.sx = sx; a.sy = sy; a.ss = ss; a.nreal = ns;
  int s = ctx->work.ensure(off_part, ctx->stream);
  if (!s) s = run_pan(ctx, a, comp, off_part);
  if (s) return s;
  if (a.nsplit > 1) a.part = ctx->work.as<char>(off_part);
  timing_begin(ctx);
  s = launch_pan(ctx, a, comp);
  timing_end(ctx);
  return s;
}

// Reverse mode of panels_affect_points with respect to the panel strengths: for cotangents
// (lu, lv) of the finalized point velocities, gvs[p] += dL/dgamma_p and gss[p] += dL/dsigma_p
// (gss may be null).  The panels are the targets of the sum, the points its sources.
int run_panels_affect_points_vjp(obs_context* ctx, const PanelSet& ps, int nt, const float* tx, const float* ty,
                                 const float* lu, const float* lv, int accum, float* gvs, float* gss) {
  if (ps.npan == 0 || nt == 0) return OBS_OK;
  const bool comp = accum == OBS_COMPENSATED;
  const int ntiles = (nt + PAN_TILE - 1) / PAN_TILE;
  const int nt_pad = ntiles * PAN_TILE;
  const int np = ps.npan;
  const size_t hdr = 256;
  const size_t lbytes = ((size_t)np * sizeof(float) + 255) & ~(size_t)255;
  const size_t off_pts = hdr + lbytes;
  const size_t off_part = off_pts + (size_t)nt_pad * sizeof(float4);
  PanArgs a;
  std::memset(&a, 0, sizeof(a));
  a.nsrc = nt_pad; a.nblk = nt_pad / PAN_COMP_BLOCK;
  a.nt = np;
  a.finalize = 0;
  a.mode = 2;
  set_panels(a, ps, nullptr, nullptr, ctx);
  int s = ctx->work.ensure(off_part, ctx->stream);
  if (!s) s = run_pan(ctx, a, comp, off_part);
  if (s) return s;
  float* sink = ctx->work.as<float>(hdr);   // dL/dsigma when not wanted
  float4* pts = ctx->work.as<float4>(off_pts);
  a.pts = pts;
  a.out_u = gvs;
  a.out_v = gss ? gss : sink;
  if (a.nsplit > 1) a.part = ctx->work.as<char>(off_part);
  timing_begin(ctx);
  s = OBS_OK;
  if (!gss) s = cuda_status(cudaMemsetAsync(sink, 0, (size_t)np * sizeof(float), ctx->stream));
  if (!s) {
    pack_cotangents_kernel<<<(nt_pad + 255) / 256, 256, 0, ctx->stream>>>(tx, ty, lu, lv, nt, nt_pad, pts);
    ctx->launches++;
    s = cuda_status(cudaGetLastError());
  }
  if (!s) s = launch_pan(ctx, a, comp);
  timing_end(ctx);
  return s;
}

// panels_on_panels_coeff into caller buffers (either may be null)
int run_panels_on_panels_coeff(obs_context* ctx, const PanelSet& src, const PanelSet& targ, int nunk, int self,
                               float* A32, double* A64) {
  if (src.npan == 0 || targ.npan == 0) return OBS_OK;
  if (src.npan > 65535) return OBS_ERR_UNSUPPORTED;   // one grid row per source panel
  const size_t hdr = 256;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t sp = al((size_t)src.npan * sizeof(float4)), sl = al((size_t)src.npan * sizeof(float));
  const size_t tp = al((size_t)targ.npan * sizeof(float4)), tl = al((size_t)targ.npan * sizeof(float));
  int s = ctx->work.ensure(hdr + 2 * sp + sl + 2 * tp + tl, ctx->stream);
  if (s) return s;
  size_t off = hdr;
  float4* SP = ctx->work.as<float4>(off); off += sp;
  float4* SQ = ctx->work.as<float4>(off); off += sp;
  float* SL = ctx->work.as<float>(off); off += sl;
  float4* TP = ctx->work.as<float4>(off); off += tp;
  float4* TQ = ctx->work.as<float4>(off); off += tp;
  float* TL = ctx->work.as<float>(off);
  // a self block packs its one panel set once
  const bool same = src.nx == targ.nx && src.ny == targ.ny && src.idx == targ.idx && src.npan == targ.npan &&
                    src.nnodes == targ.nnodes;
  if (same) {
    TP = SP;
    TQ = SQ;
    TL = SL;
  }
  timing_begin(ctx);
  s = pack_panels(ctx, src, nullptr, nullptr, SP, SQ, SL, src.npan);
  if (!s && !same) s = pack_panels(ctx, targ, nullptr, nullptr, TP, TQ, TL, targ.npan);
  if (s) return s;
  dim3 grid((targ.npan + 127) / 128, src.npan);
  timing_main_begin(ctx);
  coeff_kernel<<<grid, 128, 0, ctx->stream>>>(SP, SQ, SL, src.npan, TP, TQ, TL, targ.npan, nunk, self, A32, A64);
  ctx->launches++;
  timing_main_end(ctx);
  timing_end(ctx);
  return cuda_status(cudaGetLastError());
}

int run_vels_to_rhs(obs_context* ctx, const PanelSet& ps, int nunk, const float* pu, const float* pv,
                    const float* bcn, float* rhs32, double* rhs64) {
  if (ps.npan == 0 || (!rhs32 && !rhs64)) return OBS_OK;
  const int blocks = (ps.npan + 255) / 256;
  rhs_kernel<<<blocks, 256, 0, ctx->stream>>>(ps.nx, ps.ny, ps.idx, ps.nnodes, pu, pv, bcn, ps.npan, nunk, rhs32, rhs64,
                                              ctx->d_status);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

}  // namespace obs
