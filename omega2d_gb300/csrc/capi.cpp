// capi.cpp -- C ABI of the engine: contexts, status codes, timing, particle-on-particle calls and
// the reference-compatible external_vel_solver_* hook.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>

#include "obs_context.h"

namespace obs {

int DevBuf::ensure(size_t bytes, cudaStream_t st) {
  if (bytes <= cap) return OBS_OK;
  if (p) {
    cudaStreamSynchronize(st);
    cudaFree(p);
    p = nullptr;
    cap = 0;
  }
  const size_t want = std::max(bytes + bytes / 4, (size_t)1 << 20);
  if (cudaMalloc(&p, want) != cudaSuccess) {
    cudaGetLastError();
    p = nullptr;
    if (cudaMalloc(&p, bytes) != cudaSuccess) {
      cudaGetLastError();
      p = nullptr;
      return OBS_ERR_ALLOC;
    }
    cap = bytes;
    return OBS_OK;
  }
  cap = want;
  return OBS_OK;
}

void DevBuf::release() {
  if (p) cudaFree(p);
  p = nullptr;
  cap = 0;
}

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return OBS_OK;
  cudaGetLastError();
  if (e == cudaErrorMemoryAllocation) return OBS_ERR_ALLOC;
  if (e == cudaErrorNoDevice || e == cudaErrorInvalidDevice || e == cudaErrorInsufficientDriver)
    return OBS_ERR_NO_DEVICE;
  return OBS_ERR_CUDA;
}

int bind(obs_context* ctx) {
  return cuda_status(cudaSetDevice(ctx->device));
}

int take_device_status(obs_context* ctx) {
  int w[4] = {0, 0, 0, 0};
  cudaError_t e = cudaMemcpyAsync(w, ctx->d_status, sizeof(w), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e);
  if (w[0]) {
    for (int k = 0; k < 4; ++k) ctx->last_failure[k] = w[k];
    cudaMemsetAsync(ctx->d_status, 0, sizeof(w), ctx->stream);
    cudaStreamSynchronize(ctx->stream);
    if (w[0] & 1) return OBS_ERR_TIMEOUT;
    if (w[0] & 8) return OBS_ERR_SINGULAR;
    if (w[0] & 4) return OBS_ERR_ARG;      // a device-side index check failed (bad node index)
    return OBS_ERR_CUDA;
  }
  return OBS_OK;
}

void timing_begin(obs_context* ctx) {
  if (ctx->timing.on) cudaEventRecord(ctx->timing.ev[0], ctx->stream);
}
void timing_main_begin(obs_context* ctx) {
  if (ctx->timing.on) cudaEventRecord(ctx->timing.ev[1], ctx->stream);
}
void timing_main_end(obs_context* ctx) {
  if (ctx->timing.on) cudaEventRecord(ctx->timing.ev[2], ctx->stream);
}
void timing_end(obs_context* ctx) {
  if (ctx->timing.on) {
    cudaEventRecord(ctx->timing.ev[3], ctx->stream);
    ctx->timing.pending = true;
  }
}

}  // namespace obs

using obs::bind;
using obs::cuda_status;

namespace {

bool bad_ptrs(std::initializer_list<const void*> ps) {
  for (const void* p : ps)
    if (!p) return true;
  return false;
}

int check_p2p_args(int core, int result, int accum, int ns, const float* sx, const float* sy,
                   const float* ss, int nt, const float* tx, const float* ty,
                   float* tu, float* tv, float* const* extra) {
  if (core < OBS_CORE_RM || core > OBS_CORE_COMPACT_EXP) return OBS_ERR_ARG;
  if (result < OBS_VELONLY || result > OBS_VELANDSHEAR) return OBS_ERR_ARG;
  if (accum != OBS_PLAIN_F32 && accum != OBS_COMPENSATED) return OBS_ERR_ARG;
  if (ns < 0 || nt < 0) return OBS_ERR_ARG;
  if (ns > 0 && bad_ptrs({sx, sy, ss})) return OBS_ERR_ARG;
  if (nt > 0 && bad_ptrs({tx, ty})) return OBS_ERR_ARG;
  if (nt > 0 && result != OBS_PSIONLY && bad_ptrs({tu, tv})) return OBS_ERR_ARG;
  const int nextra = result == OBS_VELANDGRAD ? 4 : (result == OBS_VELONLY ? 0 : 1);
  for (int k = 0; k < nextra; ++k)
    if (nt > 0 && !extra[k]) return OBS_ERR_ARG;
  return OBS_OK;
}

}  // namespace

extern "C" {

const char* obs_status_string(int s) {
  switch (s) {
    case OBS_OK: return "ok";
    case OBS_ERR_ARG: return "invalid argument";
    case OBS_ERR_ALLOC: return "allocation failed";
    case OBS_ERR_CUDA: return "CUDA runtime error";
    case OBS_ERR_TIMEOUT: return "device wait timed out";
    case OBS_ERR_NO_DEVICE: return "no usable CUDA device";
    case OBS_ERR_SINGULAR: return "singular matrix";
    case OBS_ERR_UNSUPPORTED: return "unsupported combination";
    case OBS_ERR_SCRATCH_LIMIT: return "size exceeds the fixed scratch of the no-allocation entry point";
    case OBS_ERR_NO_CONVERGENCE: return "iterative solve did not reach its tolerance";
    default: return "unknown status";
  }
}

int obs_create(obs_context** out, int device) {
  if (!out) return OBS_ERR_ARG;
  *out = nullptr;
  int ndev = 0;
  cudaError_t e = cudaGetDeviceCount(&ndev);
  if (e != cudaSuccess || ndev <= 0) { cudaGetLastError(); return OBS_ERR_NO_DEVICE; }
  if (device < 0 || device >= ndev) return OBS_ERR_ARG;
  obs_context* ctx = new (std::nothrow) obs_context();
  if (!ctx) return OBS_ERR_ALLOC;
  ctx->device = device;
  int s = bind(ctx);
  if (!s) s = cuda_status(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
  if (!s) s = cuda_status(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
  if (!s) s = cuda_status(cudaMalloc(&ctx->d_status, 4 * sizeof(int)));
  if (!s) s = cuda_status(cudaMemset(ctx->d_status, 0, 4 * sizeof(int)));
  for (int k = 0; k < 4 && !s; ++k) s = cuda_status(cudaEventCreate(&ctx->timing.ev[k]));
  if (s) {
    obs_destroy(ctx);
    return s;
  }
  ctx->stream = ctx->own_stream;
  *out = ctx;
  return OBS_OK;
}

int obs_destroy(obs_context* ctx) {
  if (!ctx) return OBS_ERR_ARG;
  cudaSetDevice(ctx->device);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  ctx->work.release();
  ctx->io.release();
  ctx->dense.release();
  ctx->state.release();
  ctx->tape.release();
  if (ctx->d_status) cudaFree(ctx->d_status);
  for (int k = 0; k < 4; ++k)
    if (ctx->timing.ev[k]) cudaEventDestroy(ctx->timing.ev[k]);
  if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
  cudaGetLastError();
  delete ctx;
  return OBS_OK;
}

int obs_set_stream(obs_context* ctx, void* stream) {
  if (!ctx) return OBS_ERR_ARG;
  ctx->stream = static_cast<cudaStream_t>(stream);
  return OBS_OK;
}

int obs_use_own_stream(obs_context* ctx) {
  if (!ctx) return OBS_ERR_ARG;
  ctx->stream = ctx->own_stream;
  return OBS_OK;
}

int obs_synchronize(obs_context* ctx) {
  if (!ctx) return OBS_ERR_ARG;
  int s = bind(ctx);
  if (s) return s;
  return obs::take_device_status(ctx);
}

int obs_enable_timing(obs_context* ctx, int on) {
  if (!ctx) return OBS_ERR_ARG;
  ctx->timing.on = on != 0;
  ctx->timing.pending = false;
  return OBS_OK;
}

int obs_last_timing(obs_context* ctx, float* main_ms, float* call_ms) {
  if (!ctx) return OBS_ERR_ARG;
  if (!ctx->timing.pending) return OBS_ERR_ARG;
  int s = bind(ctx);
  if (s) return s;
  s = cuda_status(cudaEventSynchronize(ctx->timing.ev[3]));
  if (s) return s;
  float m = 0.0f, c = 0.0f;
  s = cuda_status(cudaEventElapsedTime(&m, ctx->timing.ev[1], ctx->timing.ev[2]));
  if (!s) s = cuda_status(cudaEventElapsedTime(&c, ctx->timing.ev[0], ctx->timing.ev[3]));
  if (s) return s;
  if (main_ms) *main_ms = m;
  if (call_ms) *call_ms = c;
  return OBS_OK;
}

int obs_last_failure(obs_context* ctx, int* bits, int* code, int* v1, int* v2) {
  if (!ctx) return OBS_ERR_ARG;
  if (bits) *bits = ctx->last_failure[0];
  if (code) *code = ctx->last_failure[1];
  if (v1) *v1 = ctx->last_failure[2];
  if (v2) *v2 = ctx->last_failure[3];
  return OBS_OK;
}

int obs_selftest_bounded_wait(obs_context* ctx, int which, int max_polls) {
  if (!ctx) return OBS_ERR_ARG;
  int s = obs::bind(ctx);
  if (s) return s;
  return obs::selftest_bounded_wait(ctx, which, max_polls);
}

int obs_set_kernel_variant(obs_context* ctx, int variant) {
  if (!ctx) return OBS_ERR_ARG;
  if (variant != OBS_VARIANT_AUTO && variant != OBS_VARIANT_GENERIC && variant != OBS_VARIANT_PACKED2 &&
      variant != OBS_VARIANT_PACKED3 && variant != OBS_VARIANT_PACKED4)
    return OBS_ERR_ARG;
  ctx->kernel_variant = variant;
  return OBS_OK;
}

int obs_set_target_order(obs_context* ctx, int order) {
  if (!ctx) return OBS_ERR_ARG;
  if (order != OBS_ORDER_AUTO && order != OBS_ORDER_INPUT && order != OBS_ORDER_BINNED &&
      order != OBS_ORDER_BINNED_TARGETS)
    return OBS_ERR_ARG;
  ctx->target_order = order;
  return OBS_OK;
}

int obs_morton_order_dev(obs_context* ctx, int n, const float* x, const float* y, int* perm) {
  if (!ctx || n < 0 || (n > 0 && (!x || !y || !perm))) return OBS_ERR_ARG;
  if (n == 0) return OBS_OK;
  int s = bind(ctx);
  if (s) return s;
  s = ctx->work.ensure(obs::bin_scratch_bytes(n), ctx->stream);
  if (s) return s;
  int nl = 0;
  s = cuda_status(obs::bin_order(x, y, n, ctx->work.p, perm, ctx->stream, &nl));
  ctx->launches += nl;
  return s;
}

long long obs_launch_count(obs_context* ctx) {
  return ctx ? ctx->launches : -1;
}

int obs_flops_per_pair(int core, int result, int thick) {
  const double f = obs::p2p_flops(core, result, thick != 0, 1, 1);
  if (f < 0) return -1;
  // p2p_flops(.., 1, 1) = per-target extra + per-pair count; remove the per-target part
  const int extra = result == OBS_PSIONLY ? 1 : (result == OBS_VELANDVORT || result == OBS_VELANDSHEAR ? 3 : 2);
  return (int)f - extra;
}

int obs_points_affect_points_dev(obs_context* ctx, int core, int result, int accum, int flags,
                                 double fsx, double fsy,
                                 int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                                 int nt, const float* tx, const float* ty, const float* tr,
                                 float* tu, float* tv,
                                 float* e0, float* e1, float* e2, float* e3, double* flops) {
  if (!ctx) return OBS_ERR_ARG;
  float* extra[4] = {e0, e1, e2, e3};
  int s = check_p2p_args(core, result, accum, ns, sx, sy, ss, nt, tx, ty, tu, tv, extra);
  if (s) return s;
  if ((core != OBS_CORE_SINGULAR) && ns > 0 && !sr) return OBS_ERR_ARG;
  s = bind(ctx);
  if (s) return s;
  obs::P2PRequest rq;
  rq.core = core; rq.result = result; rq.accum = accum; rq.flags = flags;
  rq.fsx = fsx; rq.fsy = fsy;
  rq.ns = ns; rq.sx = sx; rq.sy = sy; rq.sr = sr; rq.ss = ss;
  rq.nt = nt; rq.tx = tx; rq.ty = ty; rq.tr = tr;
  rq.tu = tu; rq.tv = tv;
  for (int k = 0; k < 4; ++k) rq.extra[k] = extra[k];
  s = obs::run_p2p(ctx, rq);
  if (flops) *flops = obs::p2p_flops(core, result, tr != nullptr, ns, nt);
  return s;
}

int obs_points_affect_points(obs_context* ctx, int core, int result, int accum, int flags,
                             double fsx, double fsy,
                             int ns, const float* sx, const float* sy, const float* sr, const float* ss,
                             int nt, const float* tx, const float* ty, const float* tr,
                             float* tu, float* tv,
                             float* e0, float* e1, float* e2, float* e3, double* flops) {
  if (!ctx) return OBS_ERR_ARG;
  float* extra[4] = {e0, e1, e2, e3};
  int s = check_p2p_args(core, result, accum, ns, sx, sy, ss, nt, tx, ty, tu, tv, extra);
  if (s) return s;
  if ((core != OBS_CORE_SINGULAR) && ns > 0 && !sr) return OBS_ERR_ARG;
  if (flops) *flops = obs::p2p_flops(core, result, tr != nullptr, ns, nt);
  if (ns == 0 || nt == 0) return OBS_OK;
  s = bind(ctx);
  if (s) return s;
  const int nextra = result == OBS_VELANDGRAD ? 4 : (result == OBS_VELONLY ? 0 : 1);
  const bool vel = result != OBS_PSIONLY;
  // staging layout (floats): sx sy sr ss | tx ty tr | tu tv | extras
  const size_t S = (size_t)ns, T = (size_t)nt;
  // 13 sub-arrays, each rounded up to a multiple of 64 floats
  const size_t nfloat = 4 * S + 3 * T + 2 * T + 4 * T + 13 * 64;
  s = ctx->io.ensure(nfloat * sizeof(float), ctx->stream);
  if (s) return s;
  float* base = ctx->io.as<float>();
  auto align = [](size_t n) { return (n + 63) & ~(size_t)63; };
  size_t off = 0;
  auto take = [&](size_t n) { float* p = base + off; off += align(n); return p; };
  float *dsx = take(S), *dsy = take(S), *dsr = take(S), *dss = take(S);
  float *dtx = take(T), *dty = take(T), *dtr = take(T);
  float *dtu = take(T), *dtv = take(T);
  float* dex[4] = {take(T), take(T), take(T), take(T)};
  cudaStream_t st = ctx->stream;
  auto h2d = [&](float* d, const float* h, size_t n) {
    return cudaMemcpyAsync(d, h, n * sizeof(float), cudaMemcpyHostToDevice, st);
  };
  cudaError_t e = cudaSuccess;
  e = h2d(dsx, sx, S);
  if (!e) e = h2d(dsy, sy, S);
  if (!e && sr) e = h2d(dsr, sr, S);
  if (!e) e = h2d(dss, ss, S);
  if (!e) e = h2d(dtx, tx, T);
  if (!e) e = h2d(dty, ty, T);
  if (!e && tr) e = h2d(dtr, tr, T);
  if (!e && vel) e = h2d(dtu, tu, T);
  if (!e && vel) e = h2d(dtv, tv, T);
  for (int k = 0; k < nextra && !e; ++k) e = h2d(dex[k], extra[k], T);
  if (e) return cuda_status(e);
  obs::P2PRequest rq;
  rq.core = core; rq.result = result; rq.accum = accum; rq.flags = flags;
  rq.fsx = fsx; rq.fsy = fsy;
  rq.ns = ns; rq.sx = dsx; rq.sy = dsy; rq.sr = sr ? dsr : nullptr; rq.ss = dss;
  rq.nt = nt; rq.tx = dtx; rq.ty = dty; rq.tr = tr ? dtr : nullptr;
  rq.tu = dtu; rq.tv = dtv;
  for (int k = 0; k < 4; ++k) rq.extra[k] = dex[k];
  s = obs::run_p2p(ctx, rq);
  if (s) { cudaStreamSynchronize(st); return s; }
  s = obs::take_device_status(ctx);
  if (s) return s;
  // copy results out (into temporaries first so a failure leaves the caller's arrays intact)
  std::vector<float> hu, hv;
  std::vector<std::vector<float>> hx((size_t)nextra);
  if (vel) { hu.resize(T); hv.resize(T); }
  for (int k = 0; k < nextra; ++k) hx[k].resize(T);
  if (vel) {
    e = cudaMemcpyAsync(hu.data(), dtu, T * sizeof(float), cudaMemcpyDeviceToHost, st);
    if (!e) e = cudaMemcpyAsync(hv.data(), dtv, T * sizeof(float), cudaMemcpyDeviceToHost, st);
  }
  for (int k = 0; k < nextra && !e; ++k)
    e = cudaMemcpyAsync(hx[k].data(), dex[k], T * sizeof(float), cudaMemcpyDeviceToHost, st);
  if (!e) e = cudaStreamSynchronize(st);
  if (e) return cuda_status(e);
  if (vel) {
    std::memcpy(tu, hu.data(), T * sizeof(float));
    std::memcpy(tv, hv.data(), T * sizeof(float));
  }
  for (int k = 0; k < nextra; ++k) std::memcpy(extra[k], hx[k].data(), T * sizeof(float));
  return OBS_OK;
}

}  // extern "C"
