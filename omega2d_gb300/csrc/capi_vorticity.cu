// capi_vorticity.cpp -- C ABI of the Gaussian blob vorticity sum (points_affect_points_vorticity).
#include <cstring>
#include <vector>

#include "obs_context.h"
#include "obs_device.cuh"

namespace {

int check_vort(int accum, int ns, const float* sx, const float* sy, const float* sr, const float* ss, int nt,
               const float* tx, const float* ty, const float* tw) {
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  if (ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (ns > 0 && (!sx || !sy || !sr || !ss)) return OBS_ERR_ARG;
  if (nt > 0 && (!tx || !ty || !tw)) return OBS_ERR_ARG;
  return OBS_OK;
}

obs::P2PRequest vort_request(int accum, int flags, int ns, const float* sx, const float* sy, const float* sr,
                             const float* ss, int nt, const float* tx, const float* ty, float* tw) {
  obs::P2PRequest rq;
  std::memset(&rq, 0, sizeof(rq));
  rq.core = obs::CORE_GAUSS;
  rq.result = obs::RES_BLOBVORT;
  rq.accum = accum;
  rq.flags = flags & OBS_FLAG_FINALIZE;
  rq.ns = ns; rq.sx = sx; rq.sy = sy; rq.sr = sr; rq.ss = ss;
  rq.nt = nt; rq.tx = tx; rq.ty = ty; rq.tr = nullptr;
  rq.extra[0] = tw;
  return rq;
}

}  // namespace

extern "C" {

int obs_points_affect_points_vorticity_dev(obs_context* ctx, int accum, int flags, int ns, const float* sx,
                                           const float* sy, const float* sr, const float* ss, int nt,
                                           const float* tx, const float* ty, float* tw) {
  if (!ctx) return OBS_ERR_ARG;
  int s = check_vort(accum, ns, sx, sy, sr, ss, nt, tx, ty, tw);
  if (s || ns == 0 || nt == 0) return s;
  if ((s = obs::bind(ctx))) return s;
  return obs::run_p2p(ctx, vort_request(accum, flags, ns, sx, sy, sr, ss, nt, tx, ty, tw));
}

int obs_points_affect_points_vorticity(obs_context* ctx, int accum, int flags, int ns, const float* sx,
                                       const float* sy, const float* sr, const float* ss, int nt, const float* tx,
                                       const float* ty, float* tw) {
  if (!ctx) return OBS_ERR_ARG;
  int s = check_vort(accum, ns, sx, sy, sr, ss, nt, tx, ty, tw);
  if (s || ns == 0 || nt == 0) return s;
  if ((s = obs::bind(ctx))) return s;
  const size_t S = (size_t)ns, T = (size_t)nt;
  auto al = [](size_t n) { return (n + 63) & ~(size_t)63; };
  if ((s = ctx->io.ensure((4 * al(S) + 3 * al(T)) * sizeof(float), ctx->stream))) return s;
  float* base = ctx->io.as<float>();
  float *dsx = base, *dsy = dsx + al(S), *dsr = dsy + al(S), *dss = dsr + al(S);
  float *dtx = dss + al(S), *dty = dtx + al(T), *dtw = dty + al(T);
  cudaStream_t st = ctx->stream;
  const std::pair<float*, const float*> up[] = {{dsx, sx}, {dsy, sy}, {dsr, sr}, {dss, ss}};
  cudaError_t e = cudaSuccess;
  for (const auto& u : up)
    if (e == cudaSuccess) e = cudaMemcpyAsync(u.first, u.second, S * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtx, tx, T * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dty, ty, T * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dtw, tw, T * sizeof(float), cudaMemcpyHostToDevice, st);
  if (e != cudaSuccess) return obs::cuda_status(e);
  s = obs::run_p2p(ctx, vort_request(accum, flags, ns, dsx, dsy, dsr, dss, nt, dtx, dty, dtw));
  if (s) {
    cudaStreamSynchronize(st);
    return s;
  }
  if ((s = obs::take_device_status(ctx))) return s;
  std::vector<float> hw(T);
  e = cudaMemcpyAsync(hw.data(), dtw, T * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  if (e != cudaSuccess) return obs::cuda_status(e);
  std::memcpy(tw, hw.data(), T * sizeof(float));
  return OBS_OK;
}

}  // extern "C"
