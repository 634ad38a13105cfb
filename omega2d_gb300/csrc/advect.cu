// advect.cu -- device-resident time stepping of the particles and its checkpointed reverse.
//
// Forward: the reference's convection schemes without bodies (src/Convection.h:274-598), all
// of the form  y_0 = x,  y_s = x + a_s dt u(y_{s-1})  (s = 1..S-1),  x += dt sum_s b_s u(y_s):
//   order 1  Euler (advect_1st, :274-303)            S = 1, b = (1)
//   order 2  Ralston RK2 (advect_2nd_ralston, :390-466) S = 2, a_1 = 2/3, b = (1/4, 3/4)
//   order 3  RK3 (advect_3rd, :473-598)              S = 3, a = (1/2, 3/4), b = (2/9, 3/9, 4/9)
//   order 4  Heun RK2 (advect_2nd_heun, :310-387)    S = 2, a_1 = 1, b = (1/2, 1/2)
// with u = fs + (1/2 pi) sum (finalize_vels) and the float/double mix of ElementBase::move
// (src/ElementBase.h:276-359): stage moves form (S)h * u in double, the final combination
// forms sum b_s u_s in double, stores it as float and adds (S)dt * u in one FMA.
// Reverse (no counterpart in the reference): given lam = dL/dx_{k+1},
//   c_s = b_s dt lam + a_{s+1} dt ybar_{s+1}   (s = S-1 .. 0; the second term absent for s = S-1)
//   ybar_s = (d u(y_s)/d y_s)^T c_s            (the fused self VJP of adjoint*.cu; dL/dG too)
//   lam <- lam + sum_s ybar_s
// Positions are recomputed per segment from checkpoints taken every `every` steps (sqrt(K) by
// default), so the tape holds K/every checkpoints plus one segment of stage positions.  The
// checkpoints can come from a recorded forward (obs_advect_record_dev), which the backward then
// reuses without running the forward sweep again; the recorded forward also keeps the last
// segment's positions and stage positions, which the backward reads first, so it recomputes
// every segment but that one.  every = OBS_TAPE_ALL keeps every step's
// position and stage positions instead (K*S*2N floats: 2 GB for 2M particles, 64 RK2 steps),
// and the backward then runs the VJP gathers alone, with no recomputed velocity sum.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "adjoint.h"
#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {

namespace {

struct Scheme {
  int S;
  double a[3];   // a[s]: stage s position = x + a[s] dt u(y_{s-1}); a[0] unused
  double b[3];   // final weights
};

bool scheme_of(int order, Scheme* sc) {
  switch (order) {
    case 1: *sc = Scheme{1, {0.0, 0.0, 0.0}, {1.0, 0.0, 0.0}}; return true;
    case 2: *sc = Scheme{2, {0.0, 2.0 / 3.0, 0.0}, {0.25, 0.75, 0.0}}; return true;
    case 3: *sc = Scheme{3, {0.0, 0.5, 0.75}, {2.0 / 9.0, 3.0 / 9.0, 4.0 / 9.0}}; return true;
    case 4: *sc = Scheme{2, {0.0, 1.0, 0.0}, {0.5, 0.5, 0.0}}; return true;
    default: return false;
  }
}

// ElementBase::move with one weight 1.0: x += (S)h * 1.0 * u, the product formed in double
__global__ void move1_kernel(int n, const float* __restrict__ x, const float* __restrict__ y,
                             const float* __restrict__ u, const float* __restrict__ v, float h,
                             float* __restrict__ xo, float* __restrict__ yo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  xo[i] = (float)((double)x[i] + (double)h * (double)u[i]);
  yo[i] = (float)((double)y[i] + (double)h * (double)v[i]);
}

// ElementBase::move with 2 or 3 weights: u = sum w_k u_k (double, stored as float); x += dt u
__global__ void movew_kernel(int n, float* __restrict__ x, float* __restrict__ y, int nw, double w0, double w1,
                             double w2, const float* __restrict__ vel, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const size_t N = (size_t)n;
  double cu = w0 * (double)vel[i], cv = w0 * (double)vel[N + i];
  if (nw > 1) { cu += w1 * (double)vel[2 * N + i]; cv += w1 * (double)vel[3 * N + i]; }
  if (nw > 2) { cu += w2 * (double)vel[4 * N + i]; cv += w2 * (double)vel[5 * N + i]; }
  x[i] = __fmaf_rn(dt, (float)cu, x[i]);
  y[i] = __fmaf_rn(dt, (float)cv, y[i]);
}

// out = a * p (+ b * q)
__global__ void axpby_kernel(int n, float a, const float* __restrict__ p, float b, const float* __restrict__ q,
                             float* __restrict__ out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  out[i] = q ? fmaf(a, p[i], b * q[i]) : a * p[i];
}

__global__ void add_kernel(int n, float* __restrict__ a, const float* __restrict__ b) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) a[i] += b[i];
}

int grid_of(int n) { return (n + 255) / 256; }

// finalized self-induced velocity into (u, v)
int velocity(obs_context* ctx, int core, int accum, int n, const float* x, const float* y, const float* r,
             const float* s, double fsx, double fsy, float* u, float* v) {
  cudaError_t e = cudaMemsetAsync(u, 0, (size_t)n * 4, ctx->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(v, 0, (size_t)n * 4, ctx->stream);
  if (e != cudaSuccess) return cuda_status(e);
  P2PRequest rq;
  std::memset(&rq, 0, sizeof(rq));
  rq.core = core; rq.result = OBS_VELONLY; rq.accum = accum; rq.flags = OBS_FLAG_FINALIZE;
  rq.fsx = fsx; rq.fsy = fsy;
  rq.ns = n; rq.sx = x; rq.sy = y; rq.sr = r; rq.ss = s;
  rq.nt = n; rq.tx = x; rq.ty = y; rq.tr = r;
  rq.tu = u; rq.tv = v;
  return run_p2p(ctx, rq);
}

struct Step {
  obs_context* ctx;
  int core, accum, n;
  Scheme sc;
  const float *r, *s;
  double fsx, fsy, dt;
};

// One forward step from x (2N floats: x | y).  vel: 2*S*N floats (u_s | v_s per stage).
// stages (optional): (S-1)*2N floats receiving y_1..y_{S-1}.  xo (2N, may alias x) receives
// the end position when want_end; otherwise the last stage velocity is not computed.
int step(const Step& p, const float* x, float* xo, float* vel, float* stages, bool want_end) {
  const size_t N = (size_t)p.n;
  obs_context* ctx = p.ctx;
  const int S = p.sc.S;
  const float* ys = x;
  for (int s = 0; s < S; ++s) {
    if (s > 0) {
      float* y = stages + (size_t)(s - 1) * 2 * N;
      move1_kernel<<<grid_of(p.n), 256, 0, ctx->stream>>>(p.n, x, x + N, vel + (size_t)(s - 1) * 2 * N,
                                                          vel + (size_t)(s - 1) * 2 * N + N,
                                                          (float)(p.sc.a[s] * p.dt), y, y + N);
      ctx->launches++;
      ys = y;
    }
    if (s == S - 1 && !want_end) break;
    int st = velocity(ctx, p.core, p.accum, p.n, ys, ys + N, p.r, p.s, p.fsx, p.fsy, vel + (size_t)s * 2 * N,
                      vel + (size_t)s * 2 * N + N);
    if (st) return st;
  }
  if (!want_end) return cuda_status(cudaGetLastError());
  if (S == 1) {
    move1_kernel<<<grid_of(p.n), 256, 0, ctx->stream>>>(p.n, x, x + N, vel, vel + N, (float)p.dt, xo, xo + N);
  } else {
    if (xo != x) {
      cudaError_t e = cudaMemcpyAsync(xo, x, 2 * N * 4, cudaMemcpyDeviceToDevice, ctx->stream);
      if (e != cudaSuccess) return cuda_status(e);
    }
    // vel holds (u_0 v_0 u_1 v_1 u_2 v_2): the kernel reads u_k at 2kN, v_k at (2k+1)N
    movew_kernel<<<grid_of(p.n), 256, 0, ctx->stream>>>(p.n, xo, xo + N, S, p.sc.b[0], p.sc.b[1], p.sc.b[2], vel,
                                                        (float)p.dt);
  }
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

int check_every(int every, int nsteps) {
  return every > 0 ? std::min(every, nsteps) : std::max(1, (int)std::ceil(std::sqrt((double)nsteps)));
}

// Forward sweep from (x0, y0) recording checkpoints at steps 0, C, 2C, ... into ctx->tape (after
// copies of r and s); the final positions go to (xf, yf) when given.
int record(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0, const float* r,
           const float* s, double fsx, double fsy, double dt, int nsteps, int every, float* xf, float* yf) {
  Scheme sc;
  if (!scheme_of(order, &sc)) return OBS_ERR_ARG;
  const size_t N = (size_t)n;
  const bool full = every == OBS_TAPE_ALL;
  const int C = full ? 1 : check_every(every, nsteps);
  const int nck = (nsteps + C - 1) / C;
  const size_t slot = (full ? (size_t)sc.S : 1) * 2 * N;   // floats per checkpoint
  // after the checkpoints: the last segment's x_k and stage positions, in the backward's
  // segment layout (S*2N floats per step), so the backward need not recompute that segment
  const int klast = (nck - 1) * C;
  const size_t lastf = full ? 0 : (size_t)(nsteps - klast) * sc.S * 2 * N;
  ctx->tape_info.valid = false;
  int st = ctx->tape.ensure(((size_t)2 * N + (size_t)nck * slot + lastf) * 4 + 1024, ctx->stream);
  if (st) return st;
  // state: vel 2SN | working positions 2N | stage positions (S-1)*2N (sized once, before any copy)
  if ((st = ctx->state.ensure(((size_t)2 * sc.S * N + 2 * N + (size_t)(sc.S - 1) * 2 * N) * 4 + 1024, ctx->stream)))
    return st;
  float* tr = ctx->tape.as<float>();
  float* ts = tr + N;
  float* ck = ts + N;
  float* vel = ctx->state.as<float>();
  float* w = vel + (size_t)2 * sc.S * N;
  float* stages = w + 2 * N;
  cudaStream_t strm = ctx->stream;
  auto copy = [&](float* d, const float* src, size_t cnt) {
    return cuda_status(cudaMemcpyAsync(d, src, cnt * 4, cudaMemcpyDeviceToDevice, strm));
  };
  if ((st = copy(tr, r, N)) || (st = copy(ts, s, N)) || (st = copy(w, x0, N)) || (st = copy(w + N, y0, N))) return st;
  Step p{ctx, core, accum, n, sc, tr, ts, fsx, fsy, dt};
  float* lastseg = ck + (size_t)nck * slot;
  for (int k = 0; k < nsteps; ++k) {
    float* sl = ck + (size_t)(k / C) * slot;
    if (k % C == 0 && (st = copy(sl, w, 2 * N))) return st;
    float* stg = stages;
    if (full) {
      stg = sl + 2 * N;                      // full tape: the stage positions follow x_k in its slot
    } else if (k >= klast) {
      float* xk = lastseg + (size_t)(k - klast) * sc.S * 2 * N;
      if ((st = copy(xk, w, 2 * N))) return st;
      stg = xk + 2 * N;
    }
    if ((st = step(p, w, w, vel, stg, true))) return st;
  }
  if (xf && (st = copy(xf, w, N))) return st;
  if (yf && (st = copy(yf, w + N, N))) return st;
  ctx->tape_info = AdvectTape{true, core, accum, order, n, nsteps, C, nck, fsx, fsy, dt, full, !full};
  return OBS_OK;
}

// Reverse sweep over the recorded tape: lx, ly = dL/d(final positions) in; accumulates dL/ds
// into gs and dL/d(initial positions) into gx0, gy0.
int reverse(obs_context* ctx, const float* lx_in, const float* ly_in, float* gs, float* gx0, float* gy0) {
  const AdvectTape& t = ctx->tape_info;
  if (!t.valid) return OBS_ERR_ARG;
  Scheme sc;
  scheme_of(t.order, &sc);
  const int n = t.n, C = t.every, S = sc.S;
  const size_t N = (size_t)n;
  // state (floats): segment C*S*2N (x_k, y_1..y_{S-1} per step; none for a full tape, whose
  //                 slots hold the same layout) | vel 2SN | lam 2N | cot 2N | cur 2N | prev 2N | acc 2N
  const size_t segf = t.full ? 0 : (size_t)C * S * 2 * N;
  const size_t total = segf + (size_t)2 * S * N + 10 * N;
  int st = ctx->state.ensure(total * 4 + 1024, ctx->stream);
  if (st) return st;
  float* seg = ctx->state.as<float>();
  float* vel = seg + segf;
  float* lam = vel + (size_t)2 * S * N;
  float* cot = lam + 2 * N;
  float* cur = cot + 2 * N;
  float* prev = cur + 2 * N;
  float* acc = prev + 2 * N;
  const float* tr = ctx->tape.as<float>();
  const float* ts = tr + N;
  const float* ck = ts + N;
  cudaStream_t strm = ctx->stream;
  auto copy = [&](float* d, const float* src, size_t cnt) {
    return cuda_status(cudaMemcpyAsync(d, src, cnt * 4, cudaMemcpyDeviceToDevice, strm));
  };
  auto zero = [&](float* d, size_t cnt) { return cuda_status(cudaMemsetAsync(d, 0, cnt * 4, strm)); };
  Step p{ctx, t.core, t.accum, n, sc, tr, ts, t.fsx, t.fsy, t.dt};
  // reverse of one step from its positions xk (x_k, then y_1..y_{S-1}): lam <- lam + sum_s ybar_s
  auto vjp_step = [&](const float* xk) -> int {
    int rc = zero(acc, 2 * N);
    if (rc) return rc;
    for (int s = S - 1; s >= 0; --s) {
      const float* ys = xk + (size_t)s * 2 * N;   // s = 0: x_k itself
      const float bdt = (float)(sc.b[s] * t.dt);
      if (s == S - 1) {
        axpby_kernel<<<grid_of(2 * n), 256, 0, strm>>>(2 * n, bdt, lam, 0.0f, nullptr, cot);
      } else {
        axpby_kernel<<<grid_of(2 * n), 256, 0, strm>>>(2 * n, bdt, lam, (float)(sc.a[s + 1] * t.dt), prev, cot);
      }
      ctx->launches++;
      if ((rc = zero(cur, 2 * N))) return rc;
      if ((rc = run_adjoint(ctx, t.core, t.accum, 1, n, ys, ys + N, tr, ts, n, ys, ys + N, tr, ts, cot, cot + N, cur,
                            cur + N, gs, 0)))
        return rc;
      add_kernel<<<grid_of(2 * n), 256, 0, strm>>>(2 * n, acc, cur);
      ctx->launches++;
      std::swap(cur, prev);
    }
    add_kernel<<<grid_of(2 * n), 256, 0, strm>>>(2 * n, lam, acc);
    ctx->launches++;
    return cudaGetLastError() != cudaSuccess ? OBS_ERR_CUDA : OBS_OK;
  };
  if ((st = copy(lam, lx_in, N)) || (st = copy(lam + N, ly_in, N))) return st;
  if (t.full) {
    for (int k = t.nsteps - 1; k >= 0; --k)
      if ((st = vjp_step(ck + (size_t)k * S * 2 * N))) return st;
  } else {
    for (int sg = t.nck - 1; sg >= 0; --sg) {
      const int k0 = sg * C, k1 = std::min(k0 + C, t.nsteps);
      const float* sp = seg;
      if (sg == t.nck - 1 && t.last_seg) {
        sp = ck + (size_t)t.nck * 2 * N;     // kept by the recorded forward
      } else {
        // recompute the segment's positions (x_k and its stage positions) from the checkpoint
        if ((st = copy(seg, ck + (size_t)sg * 2 * N, 2 * N))) return st;
        for (int k = k0; k < k1; ++k) {
          float* xk = seg + (size_t)(k - k0) * S * 2 * N;
          float* next = (k + 1 < k1) ? seg + (size_t)(k + 1 - k0) * S * 2 * N : nullptr;
          if ((st = step(p, xk, next ? next : xk, vel, xk + 2 * N, next != nullptr))) return st;
        }
      }
      for (int k = k1 - 1; k >= k0; --k)
        if ((st = vjp_step(sp + (size_t)(k - k0) * S * 2 * N))) return st;
    }
  }
  if (gx0) { add_kernel<<<grid_of(n), 256, 0, strm>>>(n, gx0, lam); ctx->launches++; }
  if (gy0) { add_kernel<<<grid_of(n), 256, 0, strm>>>(n, gy0, lam + N); ctx->launches++; }
  return cuda_status(cudaGetLastError());
}

}  // namespace

bool advect_order_ok(int order) {
  Scheme sc;
  return scheme_of(order, &sc);
}

int run_advect(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y,
               const float* r, const float* s, double fsx, double fsy, double dt, int nsteps) {
  Scheme sc;
  if (!scheme_of(order, &sc)) return OBS_ERR_ARG;
  if (n == 0 || nsteps == 0) return OBS_OK;
  const size_t N = (size_t)n;
  // vel 2SN | working positions 2N | stage positions (S-1)*2N
  int st = ctx->state.ensure(((size_t)2 * sc.S * N + 2 * N + (size_t)(sc.S - 1) * 2 * N) * 4 + 1024, ctx->stream);
  if (st) return st;
  float* vel = ctx->state.as<float>();
  float* w = vel + (size_t)2 * sc.S * N;
  float* stages = w + 2 * N;
  cudaStream_t strm = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(w, x, N * 4, cudaMemcpyDeviceToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(w + N, y, N * 4, cudaMemcpyDeviceToDevice, strm);
  if (e != cudaSuccess) return cuda_status(e);
  Step p{ctx, core, accum, n, sc, r, s, fsx, fsy, dt};
  for (int k = 0; k < nsteps && !st; ++k) st = step(p, w, w, vel, stages, true);
  if (st) return st;
  e = cudaMemcpyAsync(x, w, N * 4, cudaMemcpyDeviceToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(y, w + N, N * 4, cudaMemcpyDeviceToDevice, strm);
  return cuda_status(e);
}

int run_advect_record(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
                      const float* s, double fsx, double fsy, double dt, int nsteps, int every) {
  if (!advect_order_ok(order)) return OBS_ERR_ARG;
  if (n == 0 || nsteps == 0) {
    ctx->tape_info.valid = false;
    return OBS_OK;
  }
  return record(ctx, core, accum, order, n, x, y, r, s, fsx, fsy, dt, nsteps, every, x, y);
}

int run_advect_vjp_tape(obs_context* ctx, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                        long long* peak_bytes) {
  int st = reverse(ctx, lx, ly, gs, gx0, gy0);
  if (peak_bytes)
    *peak_bytes = (long long)(ctx->work.cap + ctx->io.cap + ctx->dense.cap + ctx->state.cap + ctx->tape.cap);
  return st;
}

int run_advect_vjp(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                   const float* r, const float* s, double fsx, double fsy, double dt, int nsteps, int every,
                   const float* lx, const float* ly, float* gs, float* gx0, float* gy0, long long* peak_bytes) {
  if (!advect_order_ok(order)) return OBS_ERR_ARG;
  if (n == 0 || nsteps == 0) return OBS_OK;
  int st = record(ctx, core, accum, order, n, x0, y0, r, s, fsx, fsy, dt, nsteps, every, nullptr, nullptr);
  if (st) return st;
  return run_advect_vjp_tape(ctx, lx, ly, gs, gx0, gy0, peak_bytes);
}

}  // namespace obs
