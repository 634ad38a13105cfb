/* oracle.c -- CPU restatement of the reference's direct Biot-Savart path (TEST INFRASTRUCTURE).
 *
 * This library is the checker for the CUDA engine and the "port" CPU baseline.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU arms load it; the engine never does.
 *
 * Two instantiations of oracle_impl.h:
 *   *_f : float pair arithmetic, double accumulators -- the reference's default non-Vc build
 *         (STORE=float, ACCUM=double, src/Simulation.h:44-50);
 *   *_d : double everywhere -- the FP64 oracle ("reference semantics in FP64").
 * Plus FP64-only adjoint references (no counterpart in the reference, which has no adjoint).
 *
 * Parity pin: the *_f functions are checked against the reference's own compiled code
 * (oracle/_ref, built by oracle/build_ref.py) and against the golden vectors committed under
 * tests/golden/ that were generated from it.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* float instantiation */
#define R float
#define A double
#define SFX(n) n##_f
#define EXP expf
#define LOG logf
#define SQRT sqrtf
#define CBRT cbrtf
#define ATAN2 atan2f
#define FMA fmaf
#define NEXTAFTER nextafterf
#include "oracle_impl.h"
#undef NEXTAFTER
#undef R
#undef A
#undef SFX
#undef EXP
#undef LOG
#undef SQRT
#undef CBRT
#undef ATAN2
#undef FMA

/* double instantiation */
#define R double
#define A double
#define SFX(n) n##_d
#define EXP exp
#define LOG log
#define SQRT sqrt
#define CBRT cbrt
#define ATAN2 atan2
#define FMA fma
#define NEXTAFTER nextafter
#include "oracle_impl.h"
#undef NEXTAFTER
#undef R
#undef A
#undef SFX
#undef EXP
#undef LOG
#undef SQRT
#undef CBRT
#undef ATAN2
#undef FMA

/* ------------------------------------------------------------------ FP64 adjoint references */

static const double INV2PI = 0.5 / M_PI;

/* Probe-velocity VJP.  Forward (0p field-point targets, src/Influence.h:196-211 + finalize):
 *   u_p = fs + (1/2pi) sum_j s_j K(|p - x_j|^2; r_j) J(p - x_j),  J(d) = (-dy, dx).
 * Given cotangents (lu, lv) on the finalized u_p, accumulate dL/dx_j, dL/dy_j, dL/ds_j.
 * With M(d) = d(K J)/dd = [[-b dx dy, -K - b dy^2], [K + b dx^2, b dx dy]] (b = 2 dK/d(d^2)):
 *   dL/ds_j += c sum_p lam_p . K J(d);   dL/dx_j -= c s_j sum_p M(d)^T lam_p. */
void o_probe_vjp_d(int core, int ns, const double* sx, const double* sy, const double* sr,
                   const double* ss, int np, const double* px, const double* py,
                   const double* lu, const double* lv, double* gx, double* gy, double* gs) {
  #pragma omp parallel for schedule(static)
  for (int j = 0; j < ns; ++j) {
    double ax = 0, ay = 0, as = 0;
    for (int p = 0; p < np; ++p) {
      const double dx = px[p] - sx[j], dy = py[p] - sy[j];
      const double d2 = dx*dx + dy*dy;
      double K, b;
      core_grad_d(core, d2, sr[j], 0.0, 0, &K, &b);
      as += (lu[p] * (-dy) + lv[p] * dx) * K;
      const double q = dx * lv[p] - dy * lu[p];
      ax += K * lv[p] + b * dx * q;
      ay += -K * lu[p] + b * dy * q;
    }
    gs[j] += INV2PI * as;
    gx[j] -= INV2PI * ss[j] * ax;
    gy[j] -= INV2PI * ss[j] * ay;
  }
}

/* Self-interaction VJP (thick targets == sources, src/Influence.h:347-363 + finalize):
 *   u_k = fs + c sum_j s_j K_kj J(x_k - x_j).
 * Gather form for particle k over all j (M is even in d, K symmetric in the two radii):
 *   dL/dx_k += c sum_j M(d_kj)^T (s_j lam_k - s_k lam_j)
 *   dL/ds_k -= c sum_j lam_j . K_kj J(d_kj) */
void o_self_vjp_d(int core, int n, const double* x, const double* y, const double* r,
                  const double* s, const double* lu, const double* lv,
                  double* gx, double* gy, double* gs) {
  #pragma omp parallel for schedule(static)
  for (int k = 0; k < n; ++k) {
    double ax = 0, ay = 0, as = 0;
    for (int j = 0; j < n; ++j) {
      const double dx = x[k] - x[j], dy = y[k] - y[j];
      const double d2 = dx*dx + dy*dy;
      double K, b;
      core_grad_d(core, d2, r[j], r[k], 1, &K, &b);
      const double wu = s[j] * lu[k] - s[k] * lu[j];
      const double wv = s[j] * lv[k] - s[k] * lv[j];
      const double q = dx * wv - dy * wu;
      ax += K * wv + b * dx * q;
      ay += -K * wu + b * dy * q;
      as -= (lu[j] * (-dy) + lv[j] * dx) * K;
    }
    gx[k] += INV2PI * ax;
    gy[k] += INV2PI * ay;
    gs[k] += INV2PI * as;
  }
}

/* Enstrophy-weighted centroid separation of two labelled patches:
 *   X_P = sum_{i in P} s_i^2 x_i / sum_{i in P} s_i^2,   L = |X_0 - X_1|^2.
 * Returns L; writes dL/dx, dL/dy (at these positions) and the direct dL/ds. */
double o_centroid_loss_d(int n, const double* x, const double* y, const double* s, const int* label,
                         double* gx, double* gy, double* gs) {
  double w[2] = {0, 0}, cx[2] = {0, 0}, cy[2] = {0, 0};
  for (int i = 0; i < n; ++i) {
    const int p = label[i] ? 1 : 0;
    const double wi = s[i] * s[i];
    w[p] += wi; cx[p] += wi * x[i]; cy[p] += wi * y[i];
  }
  for (int p = 0; p < 2; ++p) { cx[p] /= w[p]; cy[p] /= w[p]; }
  const double ex = cx[0] - cx[1], ey = cy[0] - cy[1];
  for (int i = 0; i < n; ++i) {
    const int p = label[i] ? 1 : 0;
    const double sg = p == 0 ? 1.0 : -1.0;
    const double wi = s[i] * s[i];
    if (gx) gx[i] = 2.0 * ex * sg * wi / w[p];
    if (gy) gy[i] = 2.0 * ey * sg * wi / w[p];
    if (gs) gs[i] = 2.0 * sg * (ex * (x[i] - cx[p]) + ey * (y[i] - cy[p])) * 2.0 * s[i] / w[p];
  }
  return ex * ex + ey * ey;
}

static void vel_d(int core, int n, const double* x, const double* y, const double* r, const double* s,
                  double fsx, double fsy, double* u, double* v) {
  memset(u, 0, sizeof(double) * (size_t)n);
  memset(v, 0, sizeof(double) * (size_t)n);
  o_points_affect_points_d(core, 1, n, x, y, r, s, n, x, y, r, u, v, 0, 0, 0, 0);
  o_finalize_vels_d(n, u, v, fsx, fsy);
}

/* Ralston RK2 (src/Convection.h:390-466) forward for nsteps, then the loss above and its
 * gradient w.r.t. the initial strengths (and initial positions), by a full reverse sweep that
 * stores every stage (small n only; the GPU engine checkpoints instead).  Returns L. */
double o_rk2_centroid_grad_d(int core, int n, const double* x0, const double* y0, const double* r,
                             const double* s, const int* label, double fsx, double fsy,
                             double dt, int nsteps, double* gs_out, double* gx_out, double* gy_out) {
  const size_t N = (size_t)n;
  double* X = (double*)malloc(sizeof(double) * N * (size_t)(nsteps + 1));
  double* Y = (double*)malloc(sizeof(double) * N * (size_t)(nsteps + 1));
  double* Y2x = (double*)malloc(sizeof(double) * N * (size_t)nsteps);
  double* Y2y = (double*)malloc(sizeof(double) * N * (size_t)nsteps);
  double* u1 = (double*)malloc(sizeof(double) * N);
  double* v1 = (double*)malloc(sizeof(double) * N);
  double* u2 = (double*)malloc(sizeof(double) * N);
  double* v2 = (double*)malloc(sizeof(double) * N);
  const double tt = 2.0 / 3.0;
  memcpy(X, x0, sizeof(double) * N);
  memcpy(Y, y0, sizeof(double) * N);
  for (int k = 0; k < nsteps; ++k) {
    const double* xk = X + N * k; const double* yk = Y + N * k;
    double* yx = Y2x + N * k; double* yy = Y2y + N * k;
    vel_d(core, n, xk, yk, r, s, fsx, fsy, u1, v1);
    for (size_t i = 0; i < N; ++i) { yx[i] = xk[i] + tt * dt * u1[i]; yy[i] = yk[i] + tt * dt * v1[i]; }
    vel_d(core, n, yx, yy, r, s, fsx, fsy, u2, v2);
    double* xn = X + N * (k + 1); double* yn = Y + N * (k + 1);
    for (size_t i = 0; i < N; ++i) {
      xn[i] = xk[i] + dt * (0.25 * u1[i] + 0.75 * u2[i]);
      yn[i] = yk[i] + dt * (0.25 * v1[i] + 0.75 * v2[i]);
    }
  }
  double* lx = (double*)malloc(sizeof(double) * N);
  double* ly = (double*)malloc(sizeof(double) * N);
  double* gs = (double*)calloc(N, sizeof(double));
  double* bx = (double*)malloc(sizeof(double) * N);
  double* by = (double*)malloc(sizeof(double) * N);
  const double L = o_centroid_loss_d(n, X + N * nsteps, Y + N * nsteps, s, label, lx, ly, gs);
  for (int k = nsteps - 1; k >= 0; --k) {
    const double* xk = X + N * k; const double* yk = Y + N * k;
    const double* yx = Y2x + N * k; const double* yy = Y2y + N * k;
    /* x_{k+1} = x_k + dt (1/4 u(x_k) + 3/4 u(y)),  y = x_k + 2/3 dt u(x_k) */
    for (size_t i = 0; i < N; ++i) { u2[i] = 0.75 * dt * lx[i]; v2[i] = 0.75 * dt * ly[i]; }
    memset(bx, 0, sizeof(double) * N); memset(by, 0, sizeof(double) * N);
    o_self_vjp_d(core, n, yx, yy, r, s, u2, v2, bx, by, gs);         /* ybar, sbar */
    for (size_t i = 0; i < N; ++i) {
      u1[i] = 0.25 * dt * lx[i] + tt * dt * bx[i];
      v1[i] = 0.25 * dt * ly[i] + tt * dt * by[i];
      lx[i] += bx[i];
      ly[i] += by[i];
    }
    memset(bx, 0, sizeof(double) * N); memset(by, 0, sizeof(double) * N);
    o_self_vjp_d(core, n, xk, yk, r, s, u1, v1, bx, by, gs);
    for (size_t i = 0; i < N; ++i) { lx[i] += bx[i]; ly[i] += by[i]; }
  }
  if (gs_out) memcpy(gs_out, gs, sizeof(double) * N);
  if (gx_out) memcpy(gx_out, lx, sizeof(double) * N);
  if (gy_out) memcpy(gy_out, ly, sizeof(double) * N);
  free(X); free(Y); free(Y2x); free(Y2y); free(u1); free(v1); free(u2); free(v2);
  free(lx); free(ly); free(gs); free(bx); free(by);
  return L;
}

/* forward only: loss after nsteps of RK2 (for finite differences) */
double o_rk2_centroid_loss_d(int core, int n, const double* x0, const double* y0, const double* r,
                             const double* s, const int* label, double fsx, double fsy,
                             double dt, int nsteps) {
  double* x = (double*)malloc(sizeof(double) * (size_t)n);
  double* y = (double*)malloc(sizeof(double) * (size_t)n);
  memcpy(x, x0, sizeof(double) * (size_t)n);
  memcpy(y, y0, sizeof(double) * (size_t)n);
  o_advect_2nd_ralston_d(core, n, x, y, r, s, fsx, fsy, dt, nsteps);
  const double L = o_centroid_loss_d(n, x, y, s, label, 0, 0, 0);
  free(x); free(y);
  return L;
}
