// external.cu -- the reference's own external direct-solver hook, served by this engine.
//
// src/Influence.h:31-38 declares three extern "C" functions that points_affect_points calls
// (src/Influence.h:74-98) when the reference is built with -DEXTERNAL_VEL_SOLVE
// (CMakeLists.txt:113-117).  Linking the reference against this library instead of its
// treecode makes every particle-on-particle evaluation run here, unchanged on the caller side.
#include <cmath>
#include <mutex>
#include <vector>

#include "obs_context.h"
#include "obs_device.cuh"

namespace {

std::mutex g_mu;
obs_context* g_ctx = nullptr;
int g_core = OBS_CORE_V2;        // the reference's compiled-in default (src/CoreFunc.h:38)
int g_accum = OBS_COMPENSATED;   // closest to the reference's double accumulators
int g_summation = OBS_SUMMATION_DIRECT;
double g_theta = OBS_TREE_THETA_DEFAULT;
int g_order = OBS_TREE_ORDER_DEFAULT;

obs_context* global_ctx() {
  if (!g_ctx) {
    if (obs_create(&g_ctx, 0) != OBS_OK) g_ctx = nullptr;
  }
  return g_ctx;
}

// FP64 field-point kernel for external_vel_solver_d_ (velocity only, 0p core forms, the
// reference's core_func(distsq, sr) overloads in double).
__device__ double core_vel_0p_d(int core, double d2, double sr) {
  const double s2 = sr * sr;
  switch (core) {
    case OBS_CORE_RM: return 1.0 / (d2 + s2);
    case OBS_CORE_GAUSSIAN: {
      const double ood2 = 1.0 / d2, corefac = 1.0 / s2, reld2 = corefac / ood2;
      if (reld2 > 16.0) return ood2;
      if (reld2 < 0.001) return corefac;
      return ood2 * (1.0 - exp(-reld2));
    }
    case OBS_CORE_V2: return 1.0 / sqrt(d2 * d2 + s2 * s2);
    case OBS_CORE_WL: { const double dd = d2 + s2; return (dd + s2) / (dd * dd); }
    case OBS_CORE_V3: return 1.0 / cbrt(d2 * d2 * d2 + s2 * s2 * s2);
    case OBS_CORE_SINGULAR: return d2 > 0.0 ? 1.0 / d2 : 0.0;
    default: {  // compact exponential
      const double x = d2 / s2, y = x * sqrt(x);
      if (y > 16.0) return 1.0 / d2;
      if (y < 0.001) return sqrt(d2) / (s2 * sqrt(s2)) * (1.0 - 0.5 * y);
      return (1.0 - exp(-y)) / d2;
    }
  }
}

__global__ void p2p_fp64_kernel(int core, int ns, const double* __restrict__ sx, const double* __restrict__ sy,
                                const double* __restrict__ ss, const double* __restrict__ sr,
                                int nt, const double* __restrict__ tx, const double* __restrict__ ty,
                                double* __restrict__ tu, double* __restrict__ tv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nt) return;
  double au = 0.0, av = 0.0;
  const double x = tx[i], y = ty[i];
  for (int j = 0; j < ns; ++j) {
    const double dx = x - sx[j], dy = y - sy[j];
    const double r2 = ss[j] * core_vel_0p_d(core, dx * dx + dy * dy, sr[j]);
    au -= r2 * dy;
    av += r2 * dx;
  }
  tu[i] += au;
  tv[i] += av;
}

float run_external_f(int* ns, const float* sx, const float* sy, const float* ss, const float* sr,
                     int* nt, const float* tx, const float* ty, const float* tr, float* tu, float* tv) {
  if (!ns || !nt) return -1.0f;
  std::lock_guard<std::mutex> lk(g_mu);
  obs_context* ctx = global_ctx();
  if (!ctx) return -1.0f;
  double flops = 0.0;
  const int s = g_summation == OBS_SUMMATION_TREE
                    ? obs_points_affect_points_tree(ctx, g_core, 0, 0.0, 0.0, g_theta, g_order, *ns, sx, sy, sr, ss,
                                                    *nt, tx, ty, tr, tu, tv, &flops)
                    : obs_points_affect_points(ctx, g_core, OBS_VELONLY, g_accum, 0, 0.0, 0.0,
                                               *ns, sx, sy, sr, ss, *nt, tx, ty, tr, tu, tv,
                                               nullptr, nullptr, nullptr, nullptr, &flops);
  return s == OBS_OK ? (float)flops : -1.0f;
}

}  // namespace

extern "C" {

int obs_external_configure_summation(int summation, double theta, int order) {
  if (summation != OBS_SUMMATION_DIRECT && summation != OBS_SUMMATION_TREE) return OBS_ERR_ARG;
  if (theta == 0.0) theta = OBS_TREE_THETA_DEFAULT;
  if (order == 0) order = OBS_TREE_ORDER_DEFAULT;
  if (!(theta > 0.0 && theta < 1.0) || order < 1 || order > OBS_TREE_ORDER_MAX) return OBS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  g_summation = summation;
  g_theta = theta;
  g_order = order;
  return OBS_OK;
}

int obs_external_configure(int core, int accum) {
  if (core < OBS_CORE_RM || core > OBS_CORE_COMPACT_EXP) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  std::lock_guard<std::mutex> lk(g_mu);
  g_core = core;
  g_accum = accum;
  return OBS_OK;
}

float external_vel_solver_f_(int* ns, const float* sx, const float* sy, const float* ss, const float* sr,
                             int* nt, const float* tx, const float* ty, float* tu, float* tv) {
  return run_external_f(ns, sx, sy, ss, sr, nt, tx, ty, nullptr, tu, tv);
}

float external_vel_solver_tr_f_(int* ns, const float* sx, const float* sy, const float* ss, const float* sr,
                                int* nt, const float* tx, const float* ty, const float* tr,
                                float* tu, float* tv) {
  if (!tr) return -1.0f;
  return run_external_f(ns, sx, sy, ss, sr, nt, tx, ty, tr, tu, tv);
}

float external_vel_solver_d_(int* ns, const double* sx, const double* sy, const double* ss, const double* sr,
                             int* nt, const double* tx, const double* ty, double* tu, double* tv) {
  if (!ns || !nt || *ns < 0 || *nt < 0) return -1.0f;
  const int S = *ns, T = *nt;
  if (S == 0 || T == 0) return 0.0f;
  if (!sx || !sy || !ss || !sr || !tx || !ty || !tu || !tv) return -1.0f;
  std::lock_guard<std::mutex> lk(g_mu);
  obs_context* ctx = global_ctx();
  if (!ctx) return -1.0f;
  if (obs::bind(ctx)) return -1.0f;
  const size_t nd = 4 * (size_t)S + 4 * (size_t)T;
  if (ctx->io.ensure(nd * sizeof(double), ctx->stream)) return -1.0f;
  double* b = ctx->io.as<double>();
  double *dsx = b, *dsy = dsx + S, *dss = dsy + S, *dsr = dss + S;
  double *dtx = dsr + S, *dty = dtx + T, *dtu = dty + T, *dtv = dtu + T;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(dsx, sx, S * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dsy, sy, S * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dss, ss, S * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dsr, sr, S * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dtx, tx, T * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dty, ty, T * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dtu, tu, T * sizeof(double), cudaMemcpyHostToDevice, st);
  if (!e) e = cudaMemcpyAsync(dtv, tv, T * sizeof(double), cudaMemcpyHostToDevice, st);
  if (e) { cudaGetLastError(); return -1.0f; }
  p2p_fp64_kernel<<<(T + 127) / 128, 128, 0, st>>>(g_core, S, dsx, dsy, dss, dsr, T, dtx, dty, dtu, dtv);
  ctx->launches++;
  e = cudaGetLastError();
  std::vector<double> hu(T), hv(T);
  if (!e) e = cudaMemcpyAsync(hu.data(), dtu, T * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaMemcpyAsync(hv.data(), dtv, T * sizeof(double), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) { cudaGetLastError(); return -1.0f; }
  for (int i = 0; i < T; ++i) { tu[i] = hu[i]; tv[i] = hv[i]; }
  return (float)obs::p2p_flops(g_core, OBS_VELONLY, false, S, T);
}

}  // extern "C"
