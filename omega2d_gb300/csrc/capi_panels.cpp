// capi_panels.cpp -- C ABI for the panel path: panels -> points, points -> panels, the
// panel-on-panel matrix, the BEM right-hand side, the FP64 dense solve and the whole
// single-body BEM solve (src/BEMHelper.h:43-260).
#include <algorithm>
#include <cstring>
#include <vector>

#include "obs_context.h"
#include "panels.h"

using obs::PanelSet;

namespace {

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

// Host-pointer staging into ctx->io: reserve all regions first, then copy in.
struct Stage {
  obs_context* ctx;
  std::vector<size_t> sizes;
  char* base = nullptr;
  size_t off = 0;
  cudaError_t err = cudaSuccess;
  explicit Stage(obs_context* c) : ctx(c) {}
  void reserve(size_t bytes) { sizes.push_back(al(bytes)); }
  int commit() {
    size_t tot = 0;
    for (size_t s : sizes) tot += s;
    const int s = ctx->io.ensure(tot + 256, ctx->stream);
    if (s) return s;
    base = ctx->io.as<char>();
    return OBS_OK;
  }
  template <class T> T* take(const T* host, size_t n) {
    T* d = reinterpret_cast<T*>(base + off);
    off += al(n * sizeof(T));
    if (host && n && err == cudaSuccess)
      err = cudaMemcpyAsync(d, host, n * sizeof(T), cudaMemcpyHostToDevice, ctx->stream);
    return d;
  }
};

int check_panels(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx) {
  if (nnodes < 0 || npan < 0) return OBS_ERR_ARG;
  if (npan > 0 && (!nx || !ny || !idx || nnodes < 2)) return OBS_ERR_ARG;
  return OBS_OK;
}

int check_host_idx(int nnodes, int npan, const unsigned* idx) {
  for (size_t k = 0; k < 2 * (size_t)npan; ++k)
    if (idx[k] >= (unsigned)nnodes) return OBS_ERR_ARG;
  return OBS_OK;
}

int copy_back(obs_context* ctx, std::initializer_list<std::pair<void*, std::pair<const void*, size_t>>> items) {
  // device -> temporaries -> caller, so a failure leaves the caller's arrays untouched
  std::vector<std::vector<char>> tmp;
  cudaError_t e = cudaSuccess;
  for (auto& it : items) {
    tmp.emplace_back(it.second.second);
    if (it.second.second && e == cudaSuccess)
      e = cudaMemcpyAsync(tmp.back().data(), it.second.first, it.second.second, cudaMemcpyDeviceToHost, ctx->stream);
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return obs::cuda_status(e);
  size_t k = 0;
  for (auto& it : items) {
    if (it.second.second) std::memcpy(it.first, tmp[k].data(), it.second.second);
    ++k;
  }
  return OBS_OK;
}

}  // namespace

extern "C" {

// ---- panels_affect_points (src/Influence.h:422-614)
int obs_panels_affect_points_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                 const float* vs, const float* ss,
                                 int nt, const float* tx, const float* ty, float* tu, float* tv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (nt < 0 || (npan > 0 && !vs) || (nt > 0 && (!tx || !ty || !tu || !tv))) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet ps{nnodes, nx, ny, npan, idx};
  return obs::run_panels_affect_points(ctx, ps, vs, ss, accum, flags, fsx, fsy, nt, tx, ty, tu, tv);
}

int obs_panels_affect_points(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                             const float* vs, const float* ss,
                             int nt, const float* tx, const float* ty, float* tu, float* tv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (nt < 0 || (npan > 0 && !vs) || (nt > 0 && (!tx || !ty || !tu || !tv))) return OBS_ERR_ARG;
  if (npan == 0 || nt == 0) return OBS_OK;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  if ((s = obs::bind(ctx))) return s;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)npan * 4);
  for (int k = 0; k < 4; ++k) g.reserve((size_t)nt * 4);
  if ((s = g.commit())) return s;
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  const float* dvs = g.take(vs, npan);
  const float* dss = ss ? g.take(ss, npan) : nullptr;
  if (!ss) g.take<float>(nullptr, npan);
  const float* dtx = g.take(tx, nt);
  const float* dty = g.take(ty, nt);
  float* dtu = g.take(tu, nt);
  float* dtv = g.take(tv, nt);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  s = obs::run_panels_affect_points(ctx, ps, dvs, dss, accum, flags, fsx, fsy, nt, dtx, dty, dtu, dtv);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  return copy_back(ctx, {{tu, {dtu, (size_t)nt * 4}}, {tv, {dtv, (size_t)nt * 4}}});
}

// ---- panels_affect_panels (src/Influence.h:774-795)
int obs_panels_affect_panels_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                                 const float* vs, const float* ss,
                                 int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                                 float* pu, float* pv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(snn, snx, sny, snp, sidx);
  if (!s) s = check_panels(tnn, tnx, tny, tnp, tidx);
  if (s) return s;
  if ((snp > 0 && !vs) || (tnp > 0 && (!pu || !pv))) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet src{snn, snx, sny, snp, sidx}, targ{tnn, tnx, tny, tnp, tidx};
  return obs::run_panels_affect_panels(ctx, src, vs, ss, accum, flags, fsx, fsy, targ, pu, pv);
}

int obs_panels_affect_panels(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                             const float* vs, const float* ss,
                             int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                             float* pu, float* pv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(snn, snx, sny, snp, sidx);
  if (!s) s = check_panels(tnn, tnx, tny, tnp, tidx);
  if (s) return s;
  if ((snp > 0 && !vs) || (tnp > 0 && (!pu || !pv))) return OBS_ERR_ARG;
  if (snp == 0 || tnp == 0) return OBS_OK;
  if ((s = check_host_idx(snn, snp, sidx)) || (s = check_host_idx(tnn, tnp, tidx))) return s;
  if ((s = obs::bind(ctx))) return s;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)snn * 4);
  g.reserve((size_t)snp * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)snp * 4);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)tnn * 4);
  g.reserve((size_t)tnp * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)tnp * 4);
  if ((s = g.commit())) return s;
  const float* dsnx = g.take(snx, snn);
  const float* dsny = g.take(sny, snn);
  const unsigned* dsidx = g.take(sidx, 2 * (size_t)snp);
  const float* dvs = g.take(vs, snp);
  const float* dss = ss ? g.take(ss, snp) : nullptr;
  if (!ss) g.take<float>(nullptr, snp);
  const float* dtnx = g.take(tnx, tnn);
  const float* dtny = g.take(tny, tnn);
  const unsigned* dtidx = g.take(tidx, 2 * (size_t)tnp);
  float* dpu = g.take(pu, tnp);
  float* dpv = g.take(pv, tnp);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet src{snn, dsnx, dsny, snp, dsidx}, targ{tnn, dtnx, dtny, tnp, dtidx};
  s = obs::run_panels_affect_panels(ctx, src, dvs, dss, accum, flags, fsx, fsy, targ, dpu, dpv);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  return copy_back(ctx, {{pu, {dpu, (size_t)tnp * 4}}, {pv, {dpv, (size_t)tnp * 4}}});
}

// ---- points_affect_panels (src/Influence.h:633-771)
int obs_points_affect_panels_dev(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                                 int ns, const float* sx, const float* sy, const float* ss,
                                 int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                                 float* pu, float* pv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (ns < 0 || (ns > 0 && (!sx || !sy || !ss)) || (npan > 0 && (!pu || !pv))) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet ps{nnodes, nx, ny, npan, idx};
  return obs::run_points_affect_panels(ctx, ns, sx, sy, ss, ps, accum, flags, fsx, fsy, pu, pv);
}

int obs_points_affect_panels(obs_context* ctx, int accum, int flags, double fsx, double fsy,
                             int ns, const float* sx, const float* sy, const float* ss,
                             int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                             float* pu, float* pv) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (ns < 0 || (ns > 0 && (!sx || !sy || !ss)) || (npan > 0 && (!pu || !pv))) return OBS_ERR_ARG;
  if (npan == 0) return OBS_OK;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  if ((s = obs::bind(ctx))) return s;
  Stage g(ctx);
  for (int k = 0; k < 3; ++k) g.reserve((size_t)ns * 4);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)npan * 4);
  if ((s = g.commit())) return s;
  const float* dsx = g.take(sx, ns);
  const float* dsy = g.take(sy, ns);
  const float* dss = g.take(ss, ns);
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  float* dpu = g.take(pu, npan);
  float* dpv = g.take(pv, npan);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  s = obs::run_points_affect_panels(ctx, ns, dsx, dsy, dss, ps, accum, flags, fsx, fsy, dpu, dpv);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  return copy_back(ctx, {{pu, {dpu, (size_t)npan * 4}}, {pv, {dpv, (size_t)npan * 4}}});
}

// ---- reverse mode of panels_affect_points w.r.t. the panel strengths
int obs_panels_affect_points_vjp_dev(obs_context* ctx, int accum, int nnodes, const float* nx, const float* ny,
                                     int npan, const unsigned* idx, int nt, const float* tx, const float* ty,
                                     const float* lu, const float* lv, float* gvs, float* gss) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (nt < 0 || (nt > 0 && (!tx || !ty || !lu || !lv)) || (npan > 0 && !gvs)) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet ps{nnodes, nx, ny, npan, idx};
  return obs::run_panels_affect_points_vjp(ctx, ps, nt, tx, ty, lu, lv, accum, gvs, gss);
}

int obs_panels_affect_points_vjp(obs_context* ctx, int accum, int nnodes, const float* nx, const float* ny,
                                 int npan, const unsigned* idx, int nt, const float* tx, const float* ty,
                                 const float* lu, const float* lv, float* gvs, float* gss) {
  if (!ctx) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (nt < 0 || (nt > 0 && (!tx || !ty || !lu || !lv)) || (npan > 0 && !gvs)) return OBS_ERR_ARG;
  if (npan == 0) return OBS_OK;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  if ((s = obs::bind(ctx))) return s;
  Stage g(ctx);
  for (int k = 0; k < 4; ++k) g.reserve((size_t)nt * 4);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)npan * 4);
  if ((s = g.commit())) return s;
  const float* dtx = g.take(tx, nt);
  const float* dty = g.take(ty, nt);
  const float* dlu = g.take(lu, nt);
  const float* dlv = g.take(lv, nt);
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  float* dgv = g.take(gvs, npan);
  float* dgs = gss ? g.take(gss, npan) : g.take<float>(nullptr, npan);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  s = obs::run_panels_affect_points_vjp(ctx, ps, nt, dtx, dty, dlu, dlv, accum, dgv, gss ? dgs : nullptr);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  if (gss) return copy_back(ctx, {{gvs, {dgv, (size_t)npan * 4}}, {gss, {dgs, (size_t)npan * 4}}});
  return copy_back(ctx, {{gvs, {dgv, (size_t)npan * 4}}});
}

// ---- panels_on_panels_coeff (src/Coefficients.h:155-427)
int obs_panels_on_panels_coeff_dev(obs_context* ctx, int nunk, int self_block,
                                   int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                                   int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                                   float* A32, double* A64) {
  if (!ctx || (nunk != 1 && nunk != 2) || (!A32 && !A64)) return OBS_ERR_ARG;
  int s = check_panels(snn, snx, sny, snp, sidx);
  if (!s) s = check_panels(tnn, tnx, tny, tnp, tidx);
  if (s) return s;
  if (self_block && snp != tnp) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet sp{snn, snx, sny, snp, sidx}, tp{tnn, tnx, tny, tnp, tidx};
  return obs::run_panels_on_panels_coeff(ctx, sp, tp, nunk, self_block, A32, A64);
}

int obs_panels_on_panels_coeff(obs_context* ctx, int nunk, int self_block,
                               int snn, const float* snx, const float* sny, int snp, const unsigned* sidx,
                               int tnn, const float* tnx, const float* tny, int tnp, const unsigned* tidx,
                               float* A32, double* A64) {
  if (!ctx || (nunk != 1 && nunk != 2) || (!A32 && !A64)) return OBS_ERR_ARG;
  int s = check_panels(snn, snx, sny, snp, sidx);
  if (!s) s = check_panels(tnn, tnx, tny, tnp, tidx);
  if (s) return s;
  if (self_block && snp != tnp) return OBS_ERR_ARG;
  if (snp == 0 || tnp == 0) return OBS_OK;
  if ((s = check_host_idx(snn, snp, sidx)) || (s = check_host_idx(tnn, tnp, tidx))) return s;
  if ((s = obs::bind(ctx))) return s;
  const size_t nel = (size_t)snp * nunk * tnp * nunk;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)snn * 4);
  g.reserve((size_t)snp * 8);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)tnn * 4);
  g.reserve((size_t)tnp * 8);
  g.reserve(A32 ? nel * 4 : 0);
  g.reserve(A64 ? nel * 8 : 0);
  if ((s = g.commit())) return s;
  const float* dsx = g.take(snx, snn);
  const float* dsy = g.take(sny, snn);
  const unsigned* dsi = g.take(sidx, 2 * (size_t)snp);
  const float* dtx = g.take(tnx, tnn);
  const float* dty = g.take(tny, tnn);
  const unsigned* dti = g.take(tidx, 2 * (size_t)tnp);
  float* d32 = A32 ? g.take<float>(nullptr, nel) : nullptr;
  double* d64 = A64 ? g.take<double>(nullptr, nel) : nullptr;
  if (g.err) return obs::cuda_status(g.err);
  PanelSet sp{snn, dsx, dsy, snp, dsi}, tp{tnn, dtx, dty, tnp, dti};
  s = obs::run_panels_on_panels_coeff(ctx, sp, tp, nunk, self_block, d32, d64);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  return copy_back(ctx, {{A32, {d32, A32 ? nel * 4 : 0}}, {A64, {d64, A64 ? nel * 8 : 0}}});
}

// ---- vels_to_rhs_panels (src/RHS.h:54-115)
int obs_vels_to_rhs_panels_dev(obs_context* ctx, int nunk, int nnodes, const float* nx, const float* ny, int npan,
                               const unsigned* idx, const float* pu, const float* pv, const float* bcn,
                               float* rhs32, double* rhs64) {
  if (!ctx || (nunk != 1 && nunk != 2) || (!rhs32 && !rhs64)) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (npan > 0 && (!pu || !pv)) return OBS_ERR_ARG;
  if ((s = obs::bind(ctx))) return s;
  PanelSet ps{nnodes, nx, ny, npan, idx};
  return obs::run_vels_to_rhs(ctx, ps, nunk, pu, pv, bcn, rhs32, rhs64);
}

int obs_vels_to_rhs_panels(obs_context* ctx, int nunk, int nnodes, const float* nx, const float* ny, int npan,
                           const unsigned* idx, const float* pu, const float* pv, const float* bcn,
                           float* rhs32, double* rhs64) {
  if (!ctx || (nunk != 1 && nunk != 2) || (!rhs32 && !rhs64)) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (npan > 0 && (!pu || !pv)) return OBS_ERR_ARG;
  if (npan == 0) return OBS_OK;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  if ((s = obs::bind(ctx))) return s;
  const size_t n = (size_t)npan * nunk;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  for (int k = 0; k < 3; ++k) g.reserve((size_t)npan * 4);
  g.reserve(rhs32 ? n * 4 : 0);
  g.reserve(rhs64 ? n * 8 : 0);
  if ((s = g.commit())) return s;
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  const float* dpu = g.take(pu, npan);
  const float* dpv = g.take(pv, npan);
  const float* dbc = bcn ? g.take(bcn, npan) : nullptr;
  if (!bcn) g.take<float>(nullptr, npan);
  float* d32 = rhs32 ? g.take<float>(nullptr, n) : nullptr;
  double* d64 = rhs64 ? g.take<double>(nullptr, n) : nullptr;
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  s = obs::run_vels_to_rhs(ctx, ps, nunk, dpu, dpv, dbc, d32, d64);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  return copy_back(ctx, {{rhs32, {d32, rhs32 ? n * 4 : 0}}, {rhs64, {d64, rhs64 ? n * 8 : 0}}});
}

// ---- FP64 dense solve of A x = b (column-major), LU with partial pivoting on the device
int obs_solve_dense_f64_dev(obs_context* ctx, int n, const double* A, const double* b, double* x,
                            double* rel_residual) {
  if (!ctx || n <= 0 || !A || !b || !x) return OBS_ERR_ARG;
  int s = obs::bind(ctx);
  if (s) return s;
  const size_t nn = (size_t)n * n;
  s = ctx->dense.ensure(nn * sizeof(double) + al((size_t)n * sizeof(int)) + 256, ctx->stream);
  if (s) return s;
  double* lu = ctx->dense.as<double>();
  int* piv = ctx->dense.as<int>(nn * sizeof(double));
  cudaError_t e = cudaMemcpyAsync(lu, A, nn * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
  if (e == cudaSuccess && x != b) e = cudaMemcpyAsync(x, b, (size_t)n * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
  if (e != cudaSuccess) return obs::cuda_status(e);
  ctx->bem_n = 0;
  ctx->bem_lu = false;
  obs::timing_begin(ctx);
  obs::timing_main_begin(ctx);
  s = obs::lu_factor_f64(ctx, n, lu, piv);
  obs::timing_main_end(ctx);
  if (!s) s = obs::lu_solve_f64(ctx, n, lu, piv, x);
  obs::timing_end(ctx);
  if (!s) s = obs::take_device_status(ctx);
  if (!s && rel_residual) s = obs::residual_f64(ctx, n, A, x, b, rel_residual);
  return s;
}

int obs_solve_dense_f64(obs_context* ctx, int n, const double* A, const double* b, double* x,
                        double* rel_residual) {
  if (!ctx || n <= 0 || !A || !b || !x) return OBS_ERR_ARG;
  int s = obs::bind(ctx);
  if (s) return s;
  Stage g(ctx);
  g.reserve((size_t)n * n * 8);
  g.reserve((size_t)n * 8);
  g.reserve((size_t)n * 8);
  if ((s = g.commit())) return s;
  const double* dA = g.take(A, (size_t)n * n);
  const double* db = g.take(b, n);
  double* dx = g.take<double>(nullptr, n);
  if (g.err) return obs::cuda_status(g.err);
  s = obs_solve_dense_f64_dev(ctx, n, dA, db, dx, rel_residual);
  if (s) return s;
  return copy_back(ctx, {{x, {dx, (size_t)n * 8}}});
}

/*
 * One reactive body, the whole of solve_bem (src/BEMHelper.h:43-260) for a fixed body:
 * panel velocities from the particles (points_affect_panels), finalize with the freestream,
 * right-hand side (vels_to_rhs_panels), the influence matrix (panels_on_panels_coeff, self
 * block), FP64 LU solve, and the strengths written back (src/Surfaces.h:266-297).
 * flags & OBS_BEM_REUSE_MATRIX reuses the factorisation from the previous call of the same
 * order (the reference's is_A_current, src/BEM.h:49-51).  All arrays on the host.
 */
int obs_solve_gmres_f64_dev(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol,
                            int restart, int maxiter, int* iterations, double* rel_residual) {
  if (!ctx || n <= 0 || !A || !b || !x || !(tol > 0.0) || restart <= 0 || maxiter <= 0) return OBS_ERR_ARG;
  int s = obs::bind(ctx);
  if (s) return s;
  s = obs::gmres_f64(ctx, n, A, b, x, tol, restart, maxiter, iterations, rel_residual);
  if (s && s != OBS_ERR_NO_CONVERGENCE) return s;
  const int d = obs::take_device_status(ctx);
  return d ? d : s;
}

int obs_solve_gmres_f64(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol,
                        int restart, int maxiter, int* iterations, double* rel_residual) {
  if (!ctx || n <= 0 || !A || !b || !x || !(tol > 0.0) || restart <= 0 || maxiter <= 0) return OBS_ERR_ARG;
  int s = obs::bind(ctx);
  if (s) return s;
  const size_t nn = (size_t)n * n;
  Stage g(ctx);
  g.reserve(nn * 8);
  g.reserve((size_t)n * 8);
  g.reserve((size_t)n * 8);
  if ((s = g.commit())) return s;
  const double* dA = g.take(A, nn);
  const double* db = g.take(b, (size_t)n);
  double* dx = g.take(static_cast<const double*>(x), (size_t)n);
  if (g.err) return obs::cuda_status(g.err);
  s = obs::gmres_f64(ctx, n, dA, db, dx, tol, restart, maxiter, iterations, rel_residual);
  if (s && s != OBS_ERR_NO_CONVERGENCE) return s;
  const int d = obs::take_device_status(ctx);
  if (d) return d;
  const int c = copy_back(ctx, {{x, {dx, (size_t)n * 8}}});
  return c ? c : s;
}

}  // extern "C"

namespace {

// Bodies joined in one panel set, some of them rotating (the rotation-augmented BEM).
struct BodySpec {
  int nbodies;            // bodies in the panel set, in order
  const int* panel_off;   // nbodies + 1 panel offsets
  const int* augmented;   // per body: nonzero adds its rotation row and column
  const double* circ;     // per body: the right-hand side of its rotation row
  double* omega;          // per body: receives its rotation rate (augmented bodies only)
};

int check_bodies(const BodySpec* b, int npan, int* naug) {
  *naug = 0;
  if (!b) return OBS_OK;
  if (b->nbodies < 1 || !b->panel_off || !b->augmented || !b->circ) return OBS_ERR_ARG;
  if (b->panel_off[0] != 0 || b->panel_off[b->nbodies] != npan) return OBS_ERR_ARG;
  for (int k = 0; k < b->nbodies; ++k) {
    if (b->panel_off[k + 1] <= b->panel_off[k]) return OBS_ERR_ARG;
    if (b->augmented[k]) ++*naug;
  }
  return *naug > obs::kMaxAugBodies ? OBS_ERR_UNSUPPORTED : OBS_OK;
}

// The augmented matrix of bodies joined in the device panel set ps (host copies nx, ny, idx give
// each rotating body's area and centre, src/Surfaces.h:629-660); geom (optional) receives
// (area, cx, cy) per body.
int bodies_augmented_matrix(obs_context* ctx, const PanelSet& ps, int nunk, int accum, int nnodes, const float* nx,
                            const float* ny, const unsigned* idx, const BodySpec* b, double* dA, double* geom) {
  obs::AugBodies ab;
  std::memset(&ab, 0, sizeof(ab));
  std::vector<float> cx, cy;
  for (int k = 0; k < b->nbodies; ++k) {
    double vol, gx, gy;
    const int p0 = b->panel_off[k], p1 = b->panel_off[k + 1];
    obs::geom_center_host(nnodes, nx, ny, p1 - p0, idx + 2 * (size_t)p0, &vol, &gx, &gy);
    if (geom) { geom[3 * k] = vol; geom[3 * k + 1] = gx; geom[3 * k + 2] = gy; }
    if (!b->augmented[k]) continue;
    ab.p0[ab.naug] = p0;
    ab.p1[ab.naug] = p1;
    ab.vol2[ab.naug] = 2.0 * vol;
    cx.push_back((float)gx);
    cy.push_back((float)gy);
    ++ab.naug;
  }
  return obs::run_panels_on_panels_coeff_bodies_augmented(ctx, ps, nunk, accum, ab, cx.data(), cy.data(),
                                                          b->nbodies, b->panel_off, dA);
}

// solve_bem (src/BEMHelper.h:43-260) over one panel set: one body, or several joined (their
// matrix is the reference's block assembly).  Each rotating body (`bodies`) adds a rotation row
// and column (src/Coefficients.h:429-572) and the circulation value of its right-hand side
// (src/BEMHelper.h:114-135); the extra unknowns are the rotation rates, after the panel unknowns.
int solve_bem_impl(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                   int ns, const float* sx, const float* sy, const float* ss,
                   int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, const float* bcn,
                   const BodySpec* bodies, float* vs_out, float* ss_out, double* rel_residual) {
  if (!ctx || (nunk != 1 && nunk != 2) || npan <= 0 || !vs_out || (nunk == 2 && !ss_out)) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if (ns < 0 || (ns > 0 && (!sx || !sy || !ss))) return OBS_ERR_ARG;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  int naug = 0;
  if ((s = check_bodies(bodies, npan, &naug))) return s;
  if ((s = obs::bind(ctx))) return s;
  const bool augment = naug > 0;
  const int nb = npan * nunk;               // panel unknowns
  const int n = nb + naug;                  // system order
  const size_t nn = (size_t)n * n;
  const bool use_lu = (flags & OBS_BEM_DIRECT_LU) != 0;
  // ctx->dense: A (FP64, kept for reuse and residuals) | LU factors | pivots; bem_n > 0 marks a
  // matrix of that order, bem_lu a factorisation of it
  const bool reuse = !augment && (flags & OBS_BEM_REUSE_MATRIX) && ctx->bem_n == n && (!use_lu || ctx->bem_lu);
  Stage g(ctx);
  for (int k = 0; k < 3; ++k) g.reserve((size_t)ns * 4);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  for (int k = 0; k < 3; ++k) g.reserve((size_t)npan * 4);
  g.reserve((size_t)n * 8);   // rhs
  g.reserve((size_t)n * 8);   // x
  if ((s = g.commit())) return s;
  const float* dsx = g.take(sx, ns);
  const float* dsy = g.take(sy, ns);
  const float* dss = g.take(ss, ns);
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  float* dpu = g.take<float>(nullptr, npan);
  float* dpv = g.take<float>(nullptr, npan);
  const float* dbc = bcn ? g.take(bcn, npan) : nullptr;
  if (!bcn) g.take<float>(nullptr, npan);
  double* drhs = g.take<double>(nullptr, n);
  double* dx = g.take<double>(nullptr, n);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  cudaError_t e = cudaSuccess;
  if (ns == 0) {
    // no particles: the panel velocities are the freestream alone
    std::vector<float> fx((size_t)npan, (float)fsx), fy((size_t)npan, (float)fsy);
    e = cudaMemcpyAsync(dpu, fx.data(), (size_t)npan * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dpv, fy.data(), (size_t)npan * 4, cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) return obs::cuda_status(e);
  } else {
    e = cudaMemsetAsync(dpu, 0, (size_t)npan * 4, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(dpv, 0, (size_t)npan * 4, ctx->stream);
    if (e != cudaSuccess) return obs::cuda_status(e);
    s = obs::run_points_affect_panels(ctx, ns, dsx, dsy, dss, ps, accum, OBS_FLAG_FINALIZE, fsx, fsy, dpu, dpv);
  }
  if (!s) s = obs::run_vels_to_rhs(ctx, ps, nunk, dpu, dpv, dbc, nullptr, drhs);
  if (s) return s;
  if (augment) {
    std::vector<double> circ;
    for (int k = 0; k < bodies->nbodies; ++k)
      if (bodies->augmented[k]) circ.push_back(bodies->circ[k]);
    e = cudaMemcpyAsync(drhs + nb, circ.data(), circ.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);   // circ is a host temporary
    if (e != cudaSuccess) return obs::cuda_status(e);
  }
  const size_t lu_bytes = use_lu ? nn * sizeof(double) : 0;
  if (!reuse) {
    ctx->bem_n = 0;
    ctx->bem_lu = false;
    s = ctx->dense.ensure(nn * sizeof(double) + lu_bytes + al((size_t)n * sizeof(int)) + 256, ctx->stream);
    if (s) return s;
  }
  double* dA = ctx->dense.as<double>();
  double* lu = ctx->dense.as<double>(nn * sizeof(double));
  int* piv = ctx->dense.as<int>(nn * sizeof(double) + lu_bytes);
  if (!reuse) {
    if (augment && bodies->nbodies == 1) {
      double vol, cx, cy;
      obs::geom_center_host(nnodes, nx, ny, npan, idx, &vol, &cx, &cy);
      s = obs::run_panels_on_panels_coeff_augmented(ctx, ps, nunk, accum, vol, cx, cy, dA);
    } else if (augment) {
      s = bodies_augmented_matrix(ctx, ps, nunk, accum, nnodes, nx, ny, idx, bodies, dA, nullptr);
    } else {
      s = obs::run_panels_on_panels_coeff(ctx, ps, ps, nunk, 1, nullptr, dA);
    }
    if (s) return s;
    ctx->bem_n = augment ? 0 : n;   // an augmented matrix is not offered for reuse
  }
  if (use_lu) {
    if (!reuse) {
      e = cudaMemcpyAsync(lu, dA, nn * sizeof(double), cudaMemcpyDeviceToDevice, ctx->stream);
      if (e != cudaSuccess) return obs::cuda_status(e);
      if ((s = obs::lu_factor_f64(ctx, n, lu, piv))) return s;
      ctx->bem_lu = true;
    }
    e = cudaMemcpyAsync(dx, drhs, (size_t)n * 8, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return obs::cuda_status(e);
    s = obs::lu_solve_f64(ctx, n, lu, piv, dx);
    if (!s) s = obs::take_device_status(ctx);
    if (!s && rel_residual) s = obs::residual_f64(ctx, n, dA, dx, drhs, rel_residual);
    if (s) return s;
  } else {
    // the reference's method (src/BEM.h:169-234), in FP64: GMRES from a zero guess
    e = cudaMemsetAsync(dx, 0, (size_t)n * 8, ctx->stream);
    if (e != cudaSuccess) return obs::cuda_status(e);
    double rel = 0.0;
    s = obs::gmres_f64(ctx, n, dA, drhs, dx, 1e-13, std::min(n, 60), 2 * n, nullptr, &rel);
    if (rel_residual) *rel_residual = rel;
    if (!s) s = obs::take_device_status(ctx);
    if (s) return s;
  }
  std::vector<double> hx(n);
  e = cudaMemcpyAsync(hx.data(), dx, (size_t)n * 8, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return obs::cuda_status(e);
  for (int i = 0; i < npan; ++i) {
    if (nunk == 2) {
      vs_out[i] = (float)hx[2 * i];
      ss_out[i] = (float)hx[2 * i + 1];
    } else {
      vs_out[i] = (float)hx[i];
    }
  }
  if (augment && bodies->omega) {
    int a = 0;
    for (int k = 0; k < bodies->nbodies; ++k)
      if (bodies->augmented[k]) bodies->omega[k] = hx[nb + a++];
  }
  return OBS_OK;
}


}  // namespace

extern "C" {

int obs_solve_bem(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                  int ns, const float* sx, const float* sy, const float* ss,
                  int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, const float* bcn,
                  float* vs_out, float* ss_out, double* rel_residual) {
  return solve_bem_impl(ctx, nunk, accum, flags, fsx, fsy, ns, sx, sy, ss, nnodes, nx, ny, npan, idx, bcn, nullptr,
                        vs_out, ss_out, rel_residual);
}

int obs_solve_bem_bodies(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                         int ns, const float* sx, const float* sy, const float* ss,
                         int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                         const float* bcn, int nbodies, const int* panel_off, const int* augmented,
                         const double* circ_rhs, float* vs_out, float* ss_out, double* omega_out,
                         double* rel_residual) {
  const BodySpec b{nbodies, panel_off, augmented, circ_rhs, omega_out};
  return solve_bem_impl(ctx, nunk, accum, flags, fsx, fsy, ns, sx, sy, ss, nnodes, nx, ny,
                        npan, idx, bcn, &b, vs_out, ss_out, rel_residual);
}

int obs_panels_on_panels_coeff_bodies(obs_context* ctx, int nunk, int accum, int nnodes, const float* nx,
                                      const float* ny, int npan, const unsigned* idx, int nbodies,
                                      const int* panel_off, const int* augmented, double* A64, double* geom) {
  if (!ctx || (nunk != 1 && nunk != 2) || npan <= 0 || !A64) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  std::vector<double> zero((size_t)std::max(nbodies, 0), 0.0);
  const BodySpec b{nbodies, panel_off, augmented, zero.data(), nullptr};
  int naug = 0;
  if ((s = check_bodies(&b, npan, &naug))) return s;
  if ((s = obs::bind(ctx))) return s;
  const int n = npan * nunk + naug;
  const size_t nn = (size_t)n * n;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  g.reserve(nn * 8);
  if ((s = g.commit())) return s;
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  double* dA = g.take<double>(nullptr, nn);
  if (g.err) return obs::cuda_status(g.err);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  std::vector<double> hg(3 * (size_t)nbodies);
  s = naug ? bodies_augmented_matrix(ctx, ps, nunk, accum, nnodes, nx, ny, idx, &b, dA, hg.data())
           : obs::run_panels_on_panels_coeff(ctx, ps, ps, nunk, 1, nullptr, dA);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  if (geom && naug) std::memcpy(geom, hg.data(), hg.size() * sizeof(double));
  return copy_back(ctx, {{A64, {dA, nn * 8}}});
}

int obs_solve_bem_augmented(obs_context* ctx, int nunk, int accum, int flags, double fsx, double fsy,
                            int ns, const float* sx, const float* sy, const float* ss,
                            int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx,
                            const float* bcn, double circ_rhs, float* vs_out, float* ss_out, double* omega_out,
                            double* rel_residual) {
  const int one = 1;
  const int off[2] = {0, npan};
  const BodySpec b{1, off, &one, &circ_rhs, omega_out};
  return solve_bem_impl(ctx, nunk, accum, flags, fsx, fsy, ns, sx, sy, ss, nnodes, nx, ny, npan, idx, bcn, &b,
                        vs_out, ss_out, rel_residual);
}

int obs_panels_on_panels_coeff_augmented(obs_context* ctx, int nunk, int accum, int nnodes, const float* nx,
                                         const float* ny, int npan, const unsigned* idx, double* A64,
                                         double* geom) {
  if (!ctx || (nunk != 1 && nunk != 2) || npan <= 0 || !A64) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  int s = check_panels(nnodes, nx, ny, npan, idx);
  if (s) return s;
  if ((s = check_host_idx(nnodes, npan, idx))) return s;
  if ((s = obs::bind(ctx))) return s;
  const int n = npan * nunk + 1;
  const size_t nn = (size_t)n * n;
  Stage g(ctx);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nnodes * 4);
  g.reserve((size_t)npan * 8);
  g.reserve(nn * 8);
  if ((s = g.commit())) return s;
  const float* dnx = g.take(nx, nnodes);
  const float* dny = g.take(ny, nnodes);
  const unsigned* didx = g.take(idx, 2 * (size_t)npan);
  double* dA = g.take<double>(nullptr, nn);
  if (g.err) return obs::cuda_status(g.err);
  double vol, cx, cy;
  obs::geom_center_host(nnodes, nx, ny, npan, idx, &vol, &cx, &cy);
  PanelSet ps{nnodes, dnx, dny, npan, didx};
  s = obs::run_panels_on_panels_coeff_augmented(ctx, ps, nunk, accum, vol, cx, cy, dA);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  if (geom) { geom[0] = vol; geom[1] = cx; geom[2] = cy; }
  return copy_back(ctx, {{A64, {dA, nn * 8}}});
}

}  // extern "C"
