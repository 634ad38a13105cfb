// capi_adjoint.cpp -- C ABI of the reverse mode: VJPs of the velocity sums and of the time
// stepping (forward/backward op pairs).  No counterpart in the reference.
#include <algorithm>
#include <cstring>
#include <vector>

#include "adjoint.h"
#include "obs_context.h"

namespace {

size_t al(size_t b) { return (b + 255) & ~(size_t)255; }

// gt += (1/2pi) G^T lam with G = [[ux, uy], [vx, vy]] (unscaled gradient sums)
__global__ void target_grad_kernel(int n, const float* __restrict__ ux, const float* __restrict__ vx,
                                   const float* __restrict__ uy, const float* __restrict__ vy,
                                   const float* __restrict__ lu, const float* __restrict__ lv,
                                   float* __restrict__ gtx, float* __restrict__ gty) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double c = 0.15915494309189535;
  if (gtx) gtx[i] = (float)((double)gtx[i] + c * ((double)ux[i] * lu[i] + (double)vx[i] * lv[i]));
  if (gty) gty[i] = (float)((double)gty[i] + c * ((double)uy[i] * lu[i] + (double)vy[i] * lv[i]));
}

struct HostStage {
  obs_context* ctx;
  size_t tot = 0;
  char* base = nullptr;
  size_t off = 0;
  cudaError_t err = cudaSuccess;
  explicit HostStage(obs_context* c) : ctx(c) {}
  void reserve(size_t bytes) { tot += al(bytes); }
  int commit() {
    const int s = ctx->io.ensure(tot + 256, ctx->stream);
    if (!s) base = ctx->io.as<char>();
    return s;
  }
  float* take(const float* host, size_t n) {
    float* d = reinterpret_cast<float*>(base + off);
    off += al(n * 4);
    if (host && n && err == cudaSuccess)
      err = cudaMemcpyAsync(d, host, n * 4, cudaMemcpyHostToDevice, ctx->stream);
    return d;
  }
};

int fetch(obs_context* ctx, std::vector<std::pair<float*, const float*>> outs, size_t n) {
  std::vector<std::vector<float>> tmp(outs.size(), std::vector<float>(n));
  cudaError_t e = cudaSuccess;
  for (size_t k = 0; k < outs.size(); ++k)
    if (outs[k].first && e == cudaSuccess)
      e = cudaMemcpyAsync(tmp[k].data(), outs[k].second, n * 4, cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return obs::cuda_status(e);
  for (size_t k = 0; k < outs.size(); ++k)
    if (outs[k].first) std::memcpy(outs[k].first, tmp[k].data(), n * 4);
  return OBS_OK;
}

bool bad_core_accum(int core, int accum) {
  return core < OBS_CORE_RM || core > OBS_CORE_COMPACT_EXP || (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED);
}

}  // namespace

extern "C" {

int obs_points_affect_points_vjp_dev(obs_context* ctx, int core, int accum,
                                     int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                     int nt, const float* tx, const float* ty, const float* tr,
                                     const float* lu, const float* lv,
                                     float* gsx, float* gsy, float* gss, float* gtx, float* gty) {
  if (!ctx || bad_core_accum(core, accum) || ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (ns > 0 && (!sx || !sy || !ss || (core != OBS_CORE_SINGULAR && !sr))) return OBS_ERR_ARG;
  if (nt > 0 && (!tx || !ty || !lu || !lv)) return OBS_ERR_ARG;
  if (ns == 0 || nt == 0) return OBS_OK;
  int s = obs::bind(ctx);
  if (s) return s;
  if (gsx || gsy || gss) {
    s = obs::run_adjoint(ctx, core, accum, 0, ns, sx, sy, sr, ss, nt, tx, ty, tr, nullptr, lu, lv, gsx, gsy, gss, 0);
    if (s) return s;
  }
  if (gtx || gty) {
    // target side: (1/2pi) (velocity-gradient sum)^T lam
    const size_t N = (size_t)nt;
    s = ctx->state.ensure(6 * N * 4 + 1024, ctx->stream);
    if (s) return s;
    float* g = ctx->state.as<float>();
    cudaError_t e = cudaMemsetAsync(g, 0, 6 * N * 4, ctx->stream);
    if (e != cudaSuccess) return obs::cuda_status(e);
    obs::P2PRequest rq;
    std::memset(&rq, 0, sizeof(rq));
    rq.core = core; rq.result = OBS_VELANDGRAD; rq.accum = accum;
    rq.ns = ns; rq.sx = sx; rq.sy = sy; rq.sr = sr; rq.ss = ss;
    rq.nt = nt; rq.tx = tx; rq.ty = ty; rq.tr = tr;
    rq.tu = g; rq.tv = g + N;
    for (int k = 0; k < 4; ++k) rq.extra[k] = g + (2 + k) * N;
    s = obs::run_p2p(ctx, rq);
    if (s) return s;
    target_grad_kernel<<<(nt + 255) / 256, 256, 0, ctx->stream>>>(nt, g + 2 * N, g + 3 * N, g + 4 * N, g + 5 * N,
                                                                  lu, lv, gtx, gty);
    ctx->launches++;
    s = obs::cuda_status(cudaGetLastError());
  }
  return s;
}

int obs_points_affect_points_vjp(obs_context* ctx, int core, int accum,
                                 int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                 int nt, const float* tx, const float* ty, const float* tr,
                                 const float* lu, const float* lv,
                                 float* gsx, float* gsy, float* gss, float* gtx, float* gty) {
  if (!ctx || bad_core_accum(core, accum) || ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (ns > 0 && (!sx || !sy || !ss || (core != OBS_CORE_SINGULAR && !sr))) return OBS_ERR_ARG;
  if (nt > 0 && (!tx || !ty || !lu || !lv)) return OBS_ERR_ARG;
  if (ns == 0 || nt == 0) return OBS_OK;
  int s = obs::bind(ctx);
  if (s) return s;
  HostStage g(ctx);
  for (int k = 0; k < 4; ++k) g.reserve((size_t)ns * 4);
  for (int k = 0; k < 5; ++k) g.reserve((size_t)nt * 4);
  for (int k = 0; k < 3; ++k) g.reserve((size_t)ns * 4);
  for (int k = 0; k < 2; ++k) g.reserve((size_t)nt * 4);
  if ((s = g.commit())) return s;
  float *dsx = g.take(sx, ns), *dsy = g.take(sy, ns), *dsr = g.take(sr, ns), *dss = g.take(ss, ns);
  float *dtx = g.take(tx, nt), *dty = g.take(ty, nt), *dtr = g.take(tr, nt), *dlu = g.take(lu, nt), *dlv = g.take(lv, nt);
  float *gx = g.take(gsx, ns), *gy = g.take(gsy, ns), *gg = g.take(gss, ns);
  float *ttx = g.take(gtx, nt), *tty = g.take(gty, nt);
  if (g.err) return obs::cuda_status(g.err);
  s = obs_points_affect_points_vjp_dev(ctx, core, accum, ns, dsx, dsy, sr ? dsr : nullptr, dss, nt, dtx, dty,
                                       tr ? dtr : nullptr, dlu, dlv, gsx ? gx : nullptr, gsy ? gy : nullptr,
                                       gss ? gg : nullptr, gtx ? ttx : nullptr, gty ? tty : nullptr);
  if (!s) s = obs::take_device_status(ctx);
  if (s) return s;
  s = fetch(ctx, {{gsx, gx}, {gsy, gy}, {gss, gg}}, ns);
  if (s) return s;
  return fetch(ctx, {{gtx, ttx}, {gty, tty}}, nt);
}

int obs_points_affect_points_vjp_self_dev(obs_context* ctx, int core, int accum, int n, const float* x, const float* y,
                                          const float* r, const float* s, const float* lu, const float* lv,
                                          float* gx, float* gy, float* gs) {
  if (!ctx || bad_core_accum(core, accum) || n < 0) return OBS_ERR_ARG;
  if (n > 0 && (!x || !y || !r || !s || !lu || !lv)) return OBS_ERR_ARG;
  if (n == 0) return OBS_OK;
  int st = obs::bind(ctx);
  if (st) return st;
  return obs::run_adjoint(ctx, core, accum, 1, n, x, y, r, s, n, x, y, r, s, lu, lv, gx, gy, gs, 0);
}

int obs_points_affect_points_vjp_self(obs_context* ctx, int core, int accum, int n, const float* x, const float* y,
                                      const float* r, const float* s, const float* lu, const float* lv,
                                      float* gx, float* gy, float* gs) {
  if (!ctx || bad_core_accum(core, accum) || n < 0) return OBS_ERR_ARG;
  if (n > 0 && (!x || !y || !r || !s || !lu || !lv)) return OBS_ERR_ARG;
  if (n == 0) return OBS_OK;
  int st = obs::bind(ctx);
  if (st) return st;
  HostStage g(ctx);
  for (int k = 0; k < 9; ++k) g.reserve((size_t)n * 4);
  if ((st = g.commit())) return st;
  float *dx = g.take(x, n), *dy = g.take(y, n), *dr = g.take(r, n), *ds = g.take(s, n);
  float *dlu = g.take(lu, n), *dlv = g.take(lv, n);
  float *ox = g.take(gx, n), *oy = g.take(gy, n), *og = g.take(gs, n);
  if (g.err) return obs::cuda_status(g.err);
  st = obs::run_adjoint(ctx, core, accum, 1, n, dx, dy, dr, ds, n, dx, dy, dr, ds, dlu, dlv,
                        gx ? ox : nullptr, gy ? oy : nullptr, gs ? og : nullptr, 0);
  if (!st) st = obs::take_device_status(ctx);
  if (st) return st;
  return fetch(ctx, {{gx, ox}, {gy, oy}, {gs, og}}, n);
}

int obs_advect_dev(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
                   const float* s, double fsx, double fsy, double dt, int nsteps) {
  if (!ctx || bad_core_accum(core, accum) || !obs::advect_order_ok(order) || n < 0 || nsteps < 0) return OBS_ERR_ARG;
  if (n > 0 && (!x || !y || !r || !s)) return OBS_ERR_ARG;
  int st = obs::bind(ctx);
  if (st) return st;
  return obs::run_advect(ctx, core, accum, order, n, x, y, r, s, fsx, fsy, dt, nsteps);
}

int obs_advect(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
               const float* s, double fsx, double fsy, double dt, int nsteps) {
  if (!ctx || bad_core_accum(core, accum) || !obs::advect_order_ok(order) || n < 0 || nsteps < 0) return OBS_ERR_ARG;
  if (n > 0 && (!x || !y || !r || !s)) return OBS_ERR_ARG;
  if (n == 0 || nsteps == 0) return OBS_OK;
  int st = obs::bind(ctx);
  if (st) return st;
  HostStage g(ctx);
  for (int k = 0; k < 4; ++k) g.reserve((size_t)n * 4);
  if ((st = g.commit())) return st;
  float *dx = g.take(x, n), *dy = g.take(y, n), *dr = g.take(r, n), *ds = g.take(s, n);
  if (g.err) return obs::cuda_status(g.err);
  st = obs::run_advect(ctx, core, accum, order, n, dx, dy, dr, ds, fsx, fsy, dt, nsteps);
  if (!st) st = obs::take_device_status(ctx);
  if (st) return st;
  return fetch(ctx, {{x, dx}, {y, dy}}, n);
}

int obs_advect_record_dev(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y,
                          const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                          int checkpoint_every) {
  if (!ctx || bad_core_accum(core, accum) || !obs::advect_order_ok(order) || n < 0 || nsteps < 0 ||
      checkpoint_every < OBS_TAPE_ALL)
    return OBS_ERR_ARG;
  if (n > 0 && (!x || !y || !r || !s)) return OBS_ERR_ARG;
  int st = obs::bind(ctx);
  if (st) return st;
  return obs::run_advect_record(ctx, core, accum, order, n, x, y, r, s, fsx, fsy, dt, nsteps, checkpoint_every);
}

int obs_advect_vjp_tape_dev(obs_context* ctx, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                            long long* peak_bytes) {
  if (!ctx || !lx || !ly) return OBS_ERR_ARG;
  if (!ctx->tape_info.valid) return OBS_ERR_ARG;
  int st = obs::bind(ctx);
  if (st) return st;
  return obs::run_advect_vjp_tape(ctx, lx, ly, gs, gx0, gy0, peak_bytes);
}

int obs_advect_vjp_dev(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                       const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                       int checkpoint_every, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                       long long* peak_bytes) {
  if (!ctx || bad_core_accum(core, accum) || !obs::advect_order_ok(order) || n < 0 || nsteps < 0 ||
      checkpoint_every < OBS_TAPE_ALL)
    return OBS_ERR_ARG;
  if (n > 0 && (!x0 || !y0 || !r || !s || !lx || !ly)) return OBS_ERR_ARG;
  int st = obs::bind(ctx);
  if (st) return st;
  return obs::run_advect_vjp(ctx, core, accum, order, n, x0, y0, r, s, fsx, fsy, dt, nsteps, checkpoint_every,
                             lx, ly, gs, gx0, gy0, peak_bytes);
}

int obs_advect_vjp(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                   const float* r, const float* s, double fsx, double fsy, double dt, int nsteps,
                   int checkpoint_every, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                   long long* peak_bytes) {
  if (!ctx || bad_core_accum(core, accum) || !obs::advect_order_ok(order) || n < 0 || nsteps < 0 ||
      checkpoint_every < OBS_TAPE_ALL)
    return OBS_ERR_ARG;
  if (n > 0 && (!x0 || !y0 || !r || !s || !lx || !ly)) return OBS_ERR_ARG;
  if (n == 0 || nsteps == 0) return OBS_OK;
  int st = obs::bind(ctx);
  if (st) return st;
  HostStage g(ctx);
  for (int k = 0; k < 9; ++k) g.reserve((size_t)n * 4);
  if ((st = g.commit())) return st;
  float *dx = g.take(x0, n), *dy = g.take(y0, n), *dr = g.take(r, n), *ds = g.take(s, n);
  float *dlx = g.take(lx, n), *dly = g.take(ly, n);
  float *ogs = g.take(gs, n), *ogx = g.take(gx0, n), *ogy = g.take(gy0, n);
  if (g.err) return obs::cuda_status(g.err);
  st = obs::run_advect_vjp(ctx, core, accum, order, n, dx, dy, dr, ds, fsx, fsy, dt, nsteps, checkpoint_every,
                           dlx, dly, gs ? ogs : nullptr, gx0 ? ogx : nullptr, gy0 ? ogy : nullptr, peak_bytes);
  if (!st) st = obs::take_device_status(ctx);
  if (st) return st;
  return fetch(ctx, {{gs, ogs}, {gx0, ogx}, {gy0, ogy}}, n);
}

}  // extern "C"
