// panels.h -- host-side declarations for the panel, BEM-matrix and dense-solve launchers.
#pragma once

#include "obs_context.h"

namespace obs {

// A set of straight panels on device: node coordinates and node-index pairs per panel
// (src/Surfaces.h:682-724 geometry; Int = uint32_t indices, src/Omega2D.h:26).
struct PanelSet {
  int nnodes;
  const float* nx;
  const float* ny;
  int npan;
  const unsigned* idx;   // 2 * npan
};

int run_panels_affect_points(obs_context* ctx, const PanelSet& ps, const float* vs, const float* ss,
                             int accum, int flags, double fsx, double fsy,
                             int nt, const float* tx, const float* ty, float* tu, float* tv);
int run_points_affect_panels(obs_context* ctx, int ns, const float* sx, const float* sy, const float* ss,
                             const PanelSet& ps, int accum, int flags, double fsx, double fsy,
                             float* pu, float* pv);
// reverse mode of panels_affect_points w.r.t. the panel strengths (cotangents of the finalized
// point velocities); gvs, gss (optional) accumulate
int run_panels_affect_points_vjp(obs_context* ctx, const PanelSet& ps, int nt, const float* tx, const float* ty,
                                 const float* lu, const float* lv, int accum, float* gvs, float* gss);
// panels_affect_panels (src/Influence.h:774-795) through the reference's collocation points
int run_panels_affect_panels(obs_context* ctx, const PanelSet& src, const float* vs, const float* ss, int accum,
                             int flags, double fsx, double fsy, const PanelSet& targ, float* pu, float* pv);
// Rotation augmentation of one body's self block (src/Coefficients.h:429-572): Aa receives the
// (n+1)^2 column-major block, n = npan * nunk; vol, (cx, cy) from geom_center_host.
void geom_center_host(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, double* vol,
                      double* cx, double* cy);
int run_panels_on_panels_coeff_augmented(obs_context* ctx, const PanelSet& ps, int nunk, int accum, double vol,
                                         double cx, double cy, double* Aa);
// Several bodies joined in one panel set, some rotating: panel unknowns first, then one rotation
// unknown per augmented body (panel range [p0, p1) of the joined set, 2 * area); cx, cy: the
// augmented bodies' centres; panel_off[0..nbodies]: every body's panel range (each body is its
// own target for the unit-rotation velocity, so its collocation spacing follows its own first
// panel).  Aa receives the (nunk * npan + naug)^2 column-major matrix.
constexpr int kMaxAugBodies = 64;
struct AugBodies {
  int naug;
  int p0[kMaxAugBodies];
  int p1[kMaxAugBodies];
  double vol2[kMaxAugBodies];
};
int run_panels_on_panels_coeff_bodies_augmented(obs_context* ctx, const PanelSet& ps, int nunk, int accum,
                                                const AugBodies& ab, const float* cx, const float* cy,
                                                int nbodies, const int* panel_off, double* Aa);
int run_panels_on_panels_coeff(obs_context* ctx, const PanelSet& src, const PanelSet& targ, int nunk, int self,
                               float* A32, double* A64);
int run_vels_to_rhs(obs_context* ctx, const PanelSet& ps, int nunk, const float* pu, const float* pv,
                    const float* bcn, float* rhs32, double* rhs64);

// FP64 dense solve A x = b (column-major n x n) by LU with partial pivoting on the device.
// A is factored in place in `lu` (n*n doubles, caller-owned device memory); piv receives n
// pivot rows.  rel_residual (optional) = ||A x - b|| / ||b|| using the unfactored A.
int lu_factor_f64(obs_context* ctx, int n, double* lu, int* piv);
int lu_solve_f64(obs_context* ctx, int n, const double* lu, const int* piv, double* x /* in: b, out: x */);
// Restarted GMRES in FP64 (gmres.cu): x in = initial guess, out = solution; OBS_ERR_NO_CONVERGENCE
// when maxiter iterations end above tol (relative residual ||b - A x|| / ||b||).
int gmres_f64(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol, int restart,
              int maxiter, int* iters_out, double* rel_residual);
int residual_f64(obs_context* ctx, int n, const double* A, const double* x, const double* b, double* rel_residual);

}  // namespace obs
