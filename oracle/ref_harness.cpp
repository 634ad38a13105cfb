// ref_harness.cpp -- C-ABI wrapper around the reference's own influence code (test infrastructure).
//
// This file is compiled, by oracle/build_ref.py, against the reference's unmodified headers
// (src/Influence.h, src/Kernels.h, src/CoreFunc.h, src/Coefficients.h, src/RHS.h, src/Reflect.h,
// src/Points.h, src/Surfaces.h, src/ElementBase.h), once per core-function macro (src/CoreFunc.h:35-39).
// The resulting libraries live in oracle/_ref/ and are used ONLY as a checker by the tests and
// by tests/golden/make_golden.py; nothing in the product path links or loads them.
//
// Every entry point below builds the reference's own element containers from flat SoA arrays,
// calls the reference driver, and copies the result back out.  Where the reference has no
// driver for a kernel (kernelug_0v_0b, kernelu_1v_0p-only panels), the loop mirrors the
// velocity-only driver loop it sits beside and calls the reference kernel function per pair.

#include "Omega2D.h"
#include "Collection.h"
#include "Influence.h"
#include "InfluenceVort.h"
#include "Coefficients.h"
#include "RHS.h"
#include "Reflect.h"

#include <cstdio>
#include <cstring>
#include <vector>
#include <unistd.h>
#include <fcntl.h>

namespace {

// The reference prints several lines per driver call (std::cout and printf).  Silence both for
// the duration of a call so test output and timing stay clean.
struct Quiet {
  int saved_fd;
  std::streambuf* saved_buf;
  Quiet() {
    fflush(stdout);
    saved_fd = dup(1);
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) { dup2(devnull, 1); close(devnull); }
    saved_buf = std::cout.rdbuf(nullptr);
  }
  ~Quiet() {
    fflush(stdout);
    std::cout.rdbuf(saved_buf);
    if (saved_fd >= 0) { dup2(saved_fd, 1); close(saved_fd); }
  }
};

template <class S>
Points<S> make_points(int n, const S* x, const S* y, const S* r, const S* s, bool is_field_point) {
  std::vector<S> xy(2 * (size_t)n);
  for (int i = 0; i < n; ++i) { xy[2*i] = x[i]; xy[2*i+1] = y[i]; }
  std::vector<S> val;
  if (!is_field_point) val.assign(s, s + n);
  ElementPacket<S> pk(xy, std::vector<Int>(), val, (size_t)n, 0);
  Points<S> p(pk, is_field_point ? inert : active, lagrangian, nullptr, 1.0f);
  if (!is_field_point) {
    Vector<S>& rr = p.get_rad();
    for (int i = 0; i < n; ++i) rr[i] = r[i];
  }
  return p;
}

template <class S>
Surfaces<S> make_surfaces(int nnodes, const S* nx, const S* ny, int npan, const unsigned* idx,
                          const S* v0, const S* v1, elem_t etype) {
  std::vector<float> xy(2 * (size_t)nnodes);
  for (int i = 0; i < nnodes; ++i) { xy[2*i] = (float)nx[i]; xy[2*i+1] = (float)ny[i]; }
  std::vector<Int> id(idx, idx + 2 * (size_t)npan);
  std::vector<float> val(2 * (size_t)npan, 0.0f);
  for (int i = 0; i < npan; ++i) {
    val[2*i]   = v0 ? (float)v0[i] : 0.0f;
    val[2*i+1] = v1 ? (float)v1[i] : 0.0f;
  }
  ElementPacket<float> pk(xy, id, val, (size_t)npan, 1);
  return Surfaces<S>(pk, etype, fixed, nullptr);
}

template <class S>
void copy_in_vel(Points<S>& p, int n, const S* u, const S* v) {
  auto& vel = p.get_vel();
  for (int i = 0; i < n; ++i) { vel[0][i] = u[i]; vel[1][i] = v[i]; }
}

template <class S>
void copy_out_vel(const Points<S>& p, int n, S* u, S* v) {
  const auto& vel = p.get_vel();
  for (int i = 0; i < n; ++i) { u[i] = vel[0][i]; v[i] = vel[1][i]; }
}

// points_affect_points (src/Influence.h:56-416), x86 branch; restype as results_t
template <class S, class A>
int ppts(int ns, const S* sx, const S* sy, const S* sr, const S* ss,
         int nt, const S* tx, const S* ty, const S* tr, int restype,
         S* tu, S* tv, S* textra) {
  Quiet q;
  Points<S> src = make_points<S>(ns, sx, sy, sr, ss, false);
  std::vector<S> dummy_s(nt, S(0));
  Points<S> targ = make_points<S>(nt, tx, ty, tr, dummy_s.data(), tr == nullptr);
  copy_in_vel(targ, nt, tu, tv);
  if (restype == velandvort) {
    Vector<S>& w = targ.get_vort();
    for (int i = 0; i < nt; ++i) w[i] = textra[i];
  } else if (restype == velandshear) {
    Vector<S>& e = targ.get_shear();
    for (int i = 0; i < nt; ++i) e[i] = textra[i];
  }
  points_affect_points<S, A>(src, targ, ResultsType((results_t)restype), ExecEnv(true, direct, cpu_x86));
  copy_out_vel(targ, nt, tu, tv);
  if (restype == velandvort) {
    const Vector<S>& w = targ.get_vort();
    for (int i = 0; i < nt; ++i) textra[i] = w[i];
  } else if (restype == velandshear) {
    const Vector<S>& e = targ.get_shear();
    for (int i = 0; i < nt; ++i) textra[i] = e[i];
  }
  return 0;
}

}  // namespace

extern "C" {

int ref_points_affect_points_f(int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                               int nt, const float* tx, const float* ty, const float* tr, int restype,
                               float* tu, float* tv, float* textra) {
  return ppts<float, double>(ns, sx, sy, sr, ss, nt, tx, ty, tr, restype, tu, tv, textra);
}

int ref_points_affect_points_d(int ns, const double* sx, const double* sy, const double* sr, const double* ss,
                               int nt, const double* tx, const double* ty, const double* tr, int restype,
                               double* tu, double* tv, double* textra) {
  return ppts<double, double>(ns, sx, sy, sr, ss, nt, tx, ty, tr, restype, tu, tv, textra);
}

// kernelug_0v_0b (src/Kernels.h:112-133) has no driver in the reference; this loop mirrors the
// velonly x86 loop of src/Influence.h:347-363 with the gradient kernel in its place.
// grads: [ux, vx, uy, vy] accumulated (+=) like the velocity.
int ref_velgrad_thick_f(int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                        int nt, const float* tx, const float* ty, const float* tr,
                        float* tu, float* tv, float* tux, float* tvx, float* tuy, float* tvy) {
  #pragma omp parallel for
  for (int i = 0; i < nt; ++i) {
    double au = 0, av = 0, aux = 0, avx = 0, auy = 0, avy = 0;
    for (int j = 0; j < ns; ++j) {
      kernelug_0v_0b<float, double>(sx[j], sy[j], sr[j], ss[j], tx[i], ty[i], tr[i],
                                    &au, &av, &aux, &avx, &auy, &avy);
    }
    tu[i] += au; tv[i] += av; tux[i] += aux; tvx[i] += avx; tuy[i] += auy; tvy[i] += avy;
  }
  return 0;
}

int ref_velgrad_thick_d(int ns, const double* sx, const double* sy, const double* sr, const double* ss,
                        int nt, const double* tx, const double* ty, const double* tr,
                        double* tu, double* tv, double* tux, double* tvx, double* tuy, double* tvy) {
  #pragma omp parallel for
  for (int i = 0; i < nt; ++i) {
    double au = 0, av = 0, aux = 0, avx = 0, auy = 0, avy = 0;
    for (int j = 0; j < ns; ++j) {
      kernelug_0v_0b<double, double>(sx[j], sy[j], sr[j], ss[j], tx[i], ty[i], tr[i],
                                     &au, &av, &aux, &avx, &auy, &avy);
    }
    tu[i] += au; tv[i] += av; tux[i] += aux; tvx[i] += avx; tuy[i] += auy; tvy[i] += avy;
  }
  return 0;
}

// kernelp_0v_0b / kernelp_0v_0p (src/Kernels.h:52-74) have no dispatching driver in the
// reference (points_affect_points asserts psionly off, src/Influence.h:60); this loop mirrors
// the velonly x86 loop of src/Influence.h:347-363 (0b) and :199-210 (0p) with the
// streamfunction kernel in its place.  tr == NULL selects the field-point (0p) kernel.
// tp accumulates (+=) like the velocity.
}  // extern "C"
template <class S>
int psi_loop(int ns, const S* sx, const S* sy, const S* sr, const S* ss,
             int nt, const S* tx, const S* ty, const S* tr, S* tp) {
  #pragma omp parallel for
  for (int i = 0; i < nt; ++i) {
    double ap = 0;
    if (tr) {
      for (int j = 0; j < ns; ++j)
        kernelp_0v_0b<S, double>(sx[j], sy[j], sr[j], ss[j], tx[i], ty[i], tr[i], &ap);
    } else {
      for (int j = 0; j < ns; ++j)
        kernelp_0v_0p<S, double>(sx[j], sy[j], sr[j], ss[j], tx[i], ty[i], &ap);
    }
    tp[i] += ap;
  }
  return 0;
}
extern "C" {

int ref_psi_f(int ns, const float* sx, const float* sy, const float* sr, const float* ss,
              int nt, const float* tx, const float* ty, const float* tr, float* tp) {
  return psi_loop<float>(ns, sx, sy, sr, ss, nt, tx, ty, tr, tp);
}

int ref_psi_d(int ns, const double* sx, const double* sy, const double* sr, const double* ss,
              int nt, const double* tx, const double* ty, const double* tr, double* tp) {
  return psi_loop<double>(ns, sx, sy, sr, ss, nt, tx, ty, tr, tp);
}

// panels_affect_points (src/Influence.h:422-614): active panels carrying vortex (vs) and
// source (ss) sheet strengths; the reference always takes the kernelu_1vs_0p branch here
// because active Surfaces always hold both strength arrays (src/Surfaces.h:86-92, 139-156).
int ref_panels_affect_points_f(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                               const float* vs, const float* ss,
                               int nt, const float* tx, const float* ty, float* tu, float* tv) {
  Quiet q;
  Surfaces<float> src = make_surfaces<float>(nnodes, nx, ny, npan, idx, vs, ss, active);
  Points<float> targ = make_points<float>(nt, tx, ty, nullptr, nullptr, true);
  copy_in_vel(targ, nt, tu, tv);
  panels_affect_points<float, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  copy_out_vel(targ, nt, tu, tv);
  return 0;
}

int ref_panels_affect_points_d(int nnodes, const double* nx, const double* ny, int npan, const unsigned* idx,
                               const double* vs, const double* ss,
                               int nt, const double* tx, const double* ty, double* tu, double* tv) {
  Quiet q;
  Surfaces<double> src = make_surfaces<double>(nnodes, nx, ny, npan, idx, vs, ss, active);
  // node positions pass through the float ElementPacket; restore them at full precision
  auto& px = src.get_pos();
  for (int i = 0; i < nnodes; ++i) { px[0][i] = nx[i]; px[1][i] = ny[i]; }
  auto& pv = src.get_str();
  for (int i = 0; i < npan; ++i) pv[i] = vs[i];
  auto& ps = src.get_src_str();
  for (int i = 0; i < npan; ++i) ps[i] = ss ? ss[i] : 0.0;
  Points<double> targ = make_points<double>(nt, tx, ty, nullptr, nullptr, true);
  copy_in_vel(targ, nt, tu, tv);
  panels_affect_points<double, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  copy_out_vel(targ, nt, tu, tv);
  return 0;
}

// vortex-only panel branch of src/Influence.h:576-594 (kernelu_1v_0p per pair)
int ref_panels_affect_points_vortex_f(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                      const float* vs, int nt, const float* tx, const float* ty,
                                      float* tu, float* tv) {
  #pragma omp parallel for
  for (int i = 0; i < nt; ++i) {
    double au = 0, av = 0, ru = 0, rv = 0;
    for (int j = 0; j < npan; ++j) {
      const unsigned j0 = idx[2*j], j1 = idx[2*j+1];
      kernelu_1v_0p<float, double>(nx[j0], ny[j0], nx[j1], ny[j1], vs[j], tx[i], ty[i], &ru, &rv);
      au += ru; av += rv;
    }
    tu[i] += au; tv[i] += av;
  }
  return 0;
}

// points_affect_panels (src/Influence.h:633-771): mean velocity on each reactive target panel
int ref_points_affect_panels_f(int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                               int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                               float* pu, float* pv) {
  Quiet q;
  Points<float> src = make_points<float>(ns, sx, sy, sr, ss, false);
  Surfaces<float> targ = make_surfaces<float>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  auto& vel = targ.get_vel();
  for (int i = 0; i < npan; ++i) { vel[0][i] = pu[i]; vel[1][i] = pv[i]; }
  points_affect_panels<float, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  for (int i = 0; i < npan; ++i) { pu[i] = vel[0][i]; pv[i] = vel[1][i]; }
  return 0;
}

int ref_points_affect_panels_d(int ns, const double* sx, const double* sy, const double* sr, const double* ss,
                               int nnodes, const double* nx, const double* ny, int npan, const unsigned* idx,
                               double* pu, double* pv) {
  Quiet q;
  Points<double> src = make_points<double>(ns, sx, sy, sr, ss, false);
  Surfaces<double> targ = make_surfaces<double>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  auto& px = targ.get_pos();
  for (int i = 0; i < nnodes; ++i) { px[0][i] = nx[i]; px[1][i] = ny[i]; }
  targ.transform(0.0);   // recompute bases and areas from the full-precision nodes
  auto& vel = targ.get_vel();
  for (int i = 0; i < npan; ++i) { vel[0][i] = pu[i]; vel[1][i] = pv[i]; }
  points_affect_panels<double, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  for (int i = 0; i < npan; ++i) { pu[i] = vel[0][i]; pv[i] = vel[1][i]; }
  return 0;
}

// panels_on_panels_coeff (src/Coefficients.h:155-573), self block (src == targ): column-major
// (2*npan) x (2*npan) matrix, already scaled by 1/(2 pi), self terms pi/(2 pi).
int ref_panels_on_panels_coeff_f(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                 float* out) {
  Quiet q;
  Surfaces<float> s = make_surfaces<float>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  Vector<float> c = panels_on_panels_coeff<float>(s, s);
  std::memcpy(out, c.data(), c.size() * sizeof(float));
  return (int)c.size();
}

int ref_panels_on_panels_coeff_d(int nnodes, const double* nx, const double* ny, int npan, const unsigned* idx,
                                 double* out) {
  Quiet q;
  Surfaces<double> s = make_surfaces<double>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  auto& px = s.get_pos();
  for (int i = 0; i < nnodes; ++i) { px[0][i] = nx[i]; px[1][i] = ny[i]; }
  s.transform(0.0);
  Vector<double> c = panels_on_panels_coeff<double>(s, s);
  std::memcpy(out, c.data(), c.size() * sizeof(double));
  return (int)c.size();
}

// off-diagonal block: distinct source and target collections (no self term)
// One off-diagonal block of a multi-body system whose bodies both rotate (augmented BEM), the
// way solve_bem assembles it (src/BEMHelper.h:183-216): the source body's unit-rotation sheet
// acts on the target's panels (panels_affect_panels, finalized with zero freestream), then
// panels_on_panels_coeff(src, targ) adds the source's augmented column and the target's
// augmented row (src/Coefficients.h:429-572).  Output: (2 tnp + 1) x (2 snp + 1), column-major.
int ref_panels_on_panels_coeff_augmented_pair_f(int snn, const float* snx, const float* sny, int snp,
                                                const unsigned* sidx, int tnn, const float* tnx, const float* tny,
                                                int tnp, const unsigned* tidx, float* out) {
  Quiet q;
  auto make = [](int nn, const float* nx, const float* ny, int np, const unsigned* idx) {
    std::vector<float> xy(2 * (size_t)nn);
    for (int i = 0; i < nn; ++i) { xy[2*i] = nx[i]; xy[2*i+1] = ny[i]; }
    std::vector<Int> id(idx, idx + 2 * (size_t)np);
    std::vector<float> val(2 * (size_t)np, 0.0f);
    ElementPacket<float> pk(xy, id, val, (size_t)np, 1);
    return Surfaces<float>(pk, reactive, fixed, std::make_shared<Body>());
  };
  Surfaces<float> src = make(snn, snx, sny, snp, sidx);
  Surfaces<float> targ = make(tnn, tnx, tny, tnp, tidx);
  src.set_geom_center();
  targ.set_geom_center();
  targ.zero_vels();
  src.zero_strengths();
  src.add_unit_rot_strengths();
  panels_affect_panels<float, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  src.zero_strengths();
  targ.finalize_vels(std::array<double, Dimensions>({0.0, 0.0}));
  Vector<float> c = panels_on_panels_coeff<float>(src, targ);
  std::copy(c.begin(), c.end(), out);
  return (int)c.size();
}

int ref_panels_on_panels_coeff_pair_f(int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                                      int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                                      float* out) {
  Quiet q;
  Surfaces<float> s = make_surfaces<float>(snn, snx, sny, snp, sidx, nullptr, nullptr, reactive);
  Surfaces<float> t = make_surfaces<float>(tnn, tnx, tny, tnp, tidx, nullptr, nullptr, reactive);
  Vector<float> c = panels_on_panels_coeff<float>(s, t);
  std::memcpy(out, c.data(), c.size() * sizeof(float));
  return (int)c.size();
}

// vels_to_rhs_panels (src/RHS.h:54-115) with 2 unknowns per panel
int ref_vels_to_rhs_panels_f(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                             const float* pu, const float* pv, const float* bct, const float* bcn, float* rhs) {
  Quiet q;
  Surfaces<float> s = make_surfaces<float>(nnodes, nx, ny, npan, idx, bct, bcn, reactive);
  auto& vel = s.get_vel();
  for (int i = 0; i < npan; ++i) { vel[0][i] = pu[i]; vel[1][i] = pv[i]; }
  std::vector<float> r = vels_to_rhs_panels<float>(s);
  std::memcpy(rhs, r.data(), r.size() * sizeof(float));
  return (int)r.size();
}

// Surfaces::finalize_vels (src/Surfaces.h:764-774) on panel-centre velocities
int ref_finalize_panel_vels_f(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                              double fsx, double fsy, float* pu, float* pv) {
  Quiet q;
  Surfaces<float> s = make_surfaces<float>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  auto& vel = s.get_vel();
  for (int i = 0; i < npan; ++i) { vel[0][i] = pu[i]; vel[1][i] = pv[i]; }
  s.finalize_vels({fsx, fsy});
  for (int i = 0; i < npan; ++i) { pu[i] = vel[0][i]; pv[i] = vel[1][i]; }
  return 0;
}

// ElementBase::finalize_vels (src/ElementBase.h:215-234)
int ref_finalize_vels_f(int n, float* u, float* v, double fsx, double fsy) {
  Quiet q;
  std::vector<float> x(n, 0.0f), r(n, 1.0f), s(n, 0.0f);
  Points<float> p = make_points<float>(n, x.data(), x.data(), r.data(), s.data(), false);
  copy_in_vel(p, n, u, v);
  p.finalize_vels({fsx, fsy});
  copy_out_vel(p, n, u, v);
  return 0;
}

// Convection::advect_1st (src/Convection.h:274-303) without bodies: per step
// zero_vels -> points_affect_points(p, p) -> finalize_vels(fs) -> move(dt)
int ref_advect_1st_f(int n, float* x, float* y, const float* r, const float* s,
                     double fsx, double fsy, double dt, int nsteps) {
  Quiet q;
  Points<float> p = make_points<float>(n, x, y, r, s, false);
  double t = 0.0;
  for (int k = 0; k < nsteps; ++k) {
    p.zero_vels();
    points_affect_points<float, double>(p, p, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p.finalize_vels({fsx, fsy});
    p.move(t, dt, 1.0, p);
    t += dt;
  }
  const auto& px = p.get_pos();
  for (int i = 0; i < n; ++i) { x[i] = px[0][i]; y[i] = px[1][i]; }
  return 0;
}

// Convection::advect_2nd_ralston (src/Convection.h:390-466) without bodies
int ref_advect_2nd_ralston_f(int n, float* x, float* y, const float* r, const float* s,
                             double fsx, double fsy, double dt, int nsteps) {
  Quiet q;
  Points<float> p = make_points<float>(n, x, y, r, s, false);
  double t = 0.0;
  const double twothirds = 2.0 / 3.0;
  for (int k = 0; k < nsteps; ++k) {
    p.zero_vels();
    points_affect_points<float, double>(p, p, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p.finalize_vels({fsx, fsy});
    Points<float> p2 = p;
    p2.move(t, twothirds * dt, 1.0, p2);
    p2.zero_vels();
    points_affect_points<float, double>(p2, p2, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p2.finalize_vels({fsx, fsy});
    p.move(t, dt, 0.25, p, 0.75, p2);
    t += dt;
  }
  const auto& px = p.get_pos();
  for (int i = 0; i < n; ++i) { x[i] = px[0][i]; y[i] = px[1][i]; }
  return 0;
}

// Convection::advect_2nd_heun (src/Convection.h:310-387) without bodies
int ref_advect_2nd_heun_f(int n, float* x, float* y, const float* r, const float* s,
                          double fsx, double fsy, double dt, int nsteps) {
  Quiet q;
  Points<float> p = make_points<float>(n, x, y, r, s, false);
  double t = 0.0;
  for (int k = 0; k < nsteps; ++k) {
    p.zero_vels();
    points_affect_points<float, double>(p, p, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p.finalize_vels({fsx, fsy});
    Points<float> p2 = p;
    p2.move(t, dt, 1.0, p2);
    p2.zero_vels();
    points_affect_points<float, double>(p2, p2, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p2.finalize_vels({fsx, fsy});
    p.move(t, dt, 0.5, p, 0.5, p2);
    t += dt;
  }
  const auto& px = p.get_pos();
  for (int i = 0; i < n; ++i) { x[i] = px[0][i]; y[i] = px[1][i]; }
  return 0;
}

// Convection::advect_3rd (src/Convection.h:473-598) without bodies
int ref_advect_3rd_f(int n, float* x, float* y, const float* r, const float* s,
                     double fsx, double fsy, double dt, int nsteps) {
  Quiet q;
  Points<float> p = make_points<float>(n, x, y, r, s, false);
  double t = 0.0;
  for (int k = 0; k < nsteps; ++k) {
    p.zero_vels();
    points_affect_points<float, double>(p, p, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p.finalize_vels({fsx, fsy});
    Points<float> p1 = p;
    p1.move(t, 0.5 * dt, 1.0, p1);
    p1.zero_vels();
    points_affect_points<float, double>(p1, p1, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p1.finalize_vels({fsx, fsy});
    Points<float> p2 = p;
    p2.move(t, 0.75 * dt, 1.0, p1);
    p2.zero_vels();
    points_affect_points<float, double>(p2, p2, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
    p2.finalize_vels({fsx, fsy});
    p.move(t, dt, 2.0 / 9.0, p, 3.0 / 9.0, p1, 4.0 / 9.0, p2);
    t += dt;
  }
  const auto& px = p.get_pos();
  for (int i = 0; i < n; ++i) { x[i] = px[0][i]; y[i] = px[1][i]; }
  return 0;
}

// points_affect_points_vorticity (src/InfluenceVort.h:47-126), x86 branch: tw accumulated
int ref_points_affect_points_vorticity_f(int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                         int nt, const float* tx, const float* ty, float* tw) {
  Quiet q;
  Points<float> src = make_points<float>(ns, sx, sy, sr, ss, false);
  Points<float> targ = make_points<float>(nt, tx, ty, nullptr, nullptr, true);
  Vector<float>& w = targ.get_vort();
  w.resize((size_t)nt);
  for (int i = 0; i < nt; ++i) w[i] = tw[i];
  points_affect_points_vorticity<float, double>(src, targ, ExecEnv(true, direct, cpu_x86));
  for (int i = 0; i < nt; ++i) tw[i] = w[i];
  return 0;
}

// panels_affect_panels (src/Influence.h:774-795): panel-centre velocities of the target body
// (accumulated) from the active source panels, through the reference's collocation points
int ref_panels_affect_panels_f(int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                               const float* vs, const float* ss,
                               int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                               float* pu, float* pv) {
  Quiet q;
  Surfaces<float> src = make_surfaces<float>(snn, snx, sny, snp, sidx, vs, ss, active);
  Surfaces<float> targ = make_surfaces<float>(tnn, tnx, tny, tnp, tidx, nullptr, nullptr, reactive);
  auto& vel = targ.get_vel();
  for (int i = 0; i < tnp; ++i) { vel[0][i] = pu[i]; vel[1][i] = pv[i]; }
  panels_affect_panels<float, double>(src, targ, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  for (int i = 0; i < tnp; ++i) { pu[i] = vel[0][i]; pv[i] = vel[1][i]; }
  return 0;
}

// The augmented self block of one rotating-capable body (src/Coefficients.h:155-573 with the
// preparation of src/BEMHelper.h:197-205): the reactive surface gets a Body, its geometric
// centre and area (Surfaces::set_geom_center), the unit-rotation strengths, their induced
// panel velocities (panels_affect_panels, finalized with zero freestream), then
// panels_on_panels_coeff returns the (2 npan + 1)^2 column-major block.
int ref_panels_on_panels_coeff_augmented_f(int nnodes, const float* nx, const float* ny, int npan,
                                           const unsigned* idx, float* out, double* geom) {
  Quiet q;
  std::shared_ptr<Body> bp = std::make_shared<Body>();
  std::vector<float> xy(2 * (size_t)nnodes);
  for (int i = 0; i < nnodes; ++i) { xy[2*i] = nx[i]; xy[2*i+1] = ny[i]; }
  std::vector<Int> id(idx, idx + 2 * (size_t)npan);
  std::vector<float> val(2 * (size_t)npan, 0.0f);
  ElementPacket<float> pk(xy, id, val, (size_t)npan, 1);
  Surfaces<float> surf(pk, reactive, fixed, bp);
  surf.set_geom_center();
  surf.zero_vels();
  surf.zero_strengths();
  surf.add_unit_rot_strengths();
  panels_affect_panels<float, double>(surf, surf, ResultsType(velonly), ExecEnv(true, direct, cpu_x86));
  surf.zero_strengths();
  surf.finalize_vels(std::array<double, Dimensions>({0.0, 0.0}));
  Vector<float> c = panels_on_panels_coeff<float>(surf, surf);
  std::copy(c.begin(), c.end(), out);
  geom[0] = surf.get_vol();
  return (int)c.size();
}

// clear_inner_panp2 (src/Reflect.h:491-729): one body's panels clear the particles (or field
// points when r is null) inside the cutoff layer; method 0 crops with the cut tables, 1 pushes.
// Updates x, y, s in place; returns the circulation removed.  Run it single-threaded
// (OMP_NUM_THREADS=1) for a reproducible sum.
float ref_clear_inner_f(int method, float cutoff_mult, float ips, int nnodes, const float* nx, const float* ny,
                        int npan, const unsigned* idx, int n, float* x, float* y, float* s, const float* r) {
  Quiet q;
  Surfaces<float> surf = make_surfaces<float>(nnodes, nx, ny, npan, idx, nullptr, nullptr, reactive);
  Points<float> pts = make_points<float>(n, x, y, r, s, r == nullptr);
  const float lost = clear_inner_panp2<float>(method, surf, pts, cutoff_mult, ips);
  const auto& pos = pts.get_pos();
  for (int i = 0; i < n; ++i) { x[i] = pos[0][i]; y[i] = pos[1][i]; }
  if (r) {
    const auto& st = pts.get_str();
    for (int i = 0; i < n; ++i) s[i] = st[i];
  }
  return lost;
}

// flop counts the reference attaches to each kernel (src/Kernels.h flops*, src/CoreFunc.h flops_*)
int ref_flop_counts(int* out) {
  out[0] = (int)flopsu_0v_0b<float, double>();
  out[1] = (int)flopsu_0v_0p<float, double>();
  out[2] = (int)flopsug_0v_0b<float, double>();
  out[3] = (int)flopsuw_0v_0b<float, double>();
  out[4] = (int)flopsue_0v_0b<float, double>();
  out[5] = (int)flopsu_1v_0p<float, double>();
  out[6] = (int)flopsu_1vs_0p<float, double>();
  out[7] = (int)flopsu_1vos_0p<float, double>();
  return 8;
}

}  // extern "C"
