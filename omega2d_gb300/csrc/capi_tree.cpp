// capi_tree.cpp -- C ABI of the treecode (tree.cu): host and device entry points.
#include <cmath>
#include <cstring>
#include <vector>

#include "obs_context.h"

namespace obs {
int run_tree(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta, int order, int ns,
             const float* sx, const float* sy, const float* sr, const float* ss, int nt, const float* tx,
             const float* ty, const float* tr, float* tu, float* tv);
}

namespace {

int check_tree(obs_context* ctx, int core, double* theta, int* order, int ns, const float* sx, const float* sy,
               const float* sr, const float* ss, int nt, const float* tx, const float* ty, float* tu, float* tv) {
  if (!ctx || core < OBS_CORE_RM || core > OBS_CORE_COMPACT_EXP || ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (*theta == 0.0) *theta = OBS_TREE_THETA_DEFAULT;
  if (*order == 0) *order = OBS_TREE_ORDER_DEFAULT;
  if (!(*theta > 0.0 && *theta < 1.0) || *order < 1 || *order > OBS_TREE_ORDER_MAX) return OBS_ERR_ARG;
  if (ns > 0 && (!sx || !sy || !ss || (core != OBS_CORE_SINGULAR && !sr))) return OBS_ERR_ARG;
  if (nt > 0 && (!tx || !ty || !tu || !tv)) return OBS_ERR_ARG;
  return OBS_OK;
}

}  // namespace

extern "C" {

int obs_points_affect_points_tree_dev(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta,
                                      int order, int ns, const float* sx, const float* sy, const float* sr,
                                      const float* ss, int nt, const float* tx, const float* ty, const float* tr,
                                      float* tu, float* tv, double* flops) {
  int s = check_tree(ctx, core, &theta, &order, ns, sx, sy, sr, ss, nt, tx, ty, tu, tv);
  if (s) return s;
  if (flops) *flops = obs::p2p_flops(core, OBS_VELONLY, tr != nullptr, ns, nt);
  if (ns == 0 || nt == 0) return OBS_OK;
  if ((s = obs::bind(ctx))) return s;
  return obs::run_tree(ctx, core, flags, fsx, fsy, theta, order, ns, sx, sy, core == OBS_CORE_SINGULAR ? nullptr : sr,
                       ss, nt, tx, ty, tr, tu, tv);
}

int obs_points_affect_points_tree(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta,
                                  int order, int ns, const float* sx, const float* sy, const float* sr,
                                  const float* ss, int nt, const float* tx, const float* ty, const float* tr,
                                  float* tu, float* tv, double* flops) {
  int s = check_tree(ctx, core, &theta, &order, ns, sx, sy, sr, ss, nt, tx, ty, tu, tv);
  if (s) return s;
  if (flops) *flops = obs::p2p_flops(core, OBS_VELONLY, tr != nullptr, ns, nt);
  if (ns == 0 || nt == 0) return OBS_OK;
  if ((s = obs::bind(ctx))) return s;
  const bool rad = core != OBS_CORE_SINGULAR;
  const size_t S = (size_t)ns, T = (size_t)nt;
  auto al = [](size_t n) { return (n + 63) & ~(size_t)63; };
  // staging (floats): sx sy sr ss | tx ty tr | tu tv
  const size_t nfloat = 4 * al(S) + 5 * al(T);
  if ((s = ctx->io.ensure(nfloat * sizeof(float), ctx->stream))) return s;
  float* base = ctx->io.as<float>();
  size_t off = 0;
  auto take = [&](size_t n) { float* p = base + off; off += al(n); return p; };
  float *dsx = take(S), *dsy = take(S), *dsr = take(S), *dss = take(S);
  float *dtx = take(T), *dty = take(T), *dtr = take(T), *dtu = take(T), *dtv = take(T);
  cudaStream_t st = ctx->stream;
  auto h2d = [&](float* d, const float* h, size_t n) {
    return cudaMemcpyAsync(d, h, n * sizeof(float), cudaMemcpyHostToDevice, st);
  };
  cudaError_t e = h2d(dsx, sx, S);
  if (!e) e = h2d(dsy, sy, S);
  if (!e && rad) e = h2d(dsr, sr, S);
  if (!e) e = h2d(dss, ss, S);
  if (!e) e = h2d(dtx, tx, T);
  if (!e) e = h2d(dty, ty, T);
  if (!e && tr) e = h2d(dtr, tr, T);
  if (!e) e = h2d(dtu, tu, T);
  if (!e) e = h2d(dtv, tv, T);
  if (e) return obs::cuda_status(e);
  s = obs::run_tree(ctx, core, flags, fsx, fsy, theta, order, ns, dsx, dsy, rad ? dsr : nullptr, dss, nt, dtx, dty,
                    tr ? dtr : nullptr, dtu, dtv);
  if (s) { cudaStreamSynchronize(st); return s; }
  if ((s = obs::take_device_status(ctx))) return s;
  std::vector<float> hu(T), hv(T);
  e = cudaMemcpyAsync(hu.data(), dtu, T * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(hv.data(), dtv, T * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return obs::cuda_status(e);
  std::memcpy(tu, hu.data(), T * sizeof(float));
  std::memcpy(tv, hv.data(), T * sizeof(float));
  return OBS_OK;
}

}  // extern "C"
