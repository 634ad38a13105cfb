// advect.cu -- device-resident time stepping of the particles and its checkpointed reverse.
//
// Forward: Convection::advect_1st / advect_2nd_ralston without bodies (src/Convection.h:274-466):
//   Euler:   x += dt u(x)
//   Ralston: u1 = u(x); y = x + 2/3 dt u1; u2 = u(y); x += dt (1/4 u1 + 3/4 u2)
// with u = fs + (1/2 pi) sum (finalize_vels) and the float/double mix of ElementBase::move
// (src/ElementBase.h:276-327).
// Reverse (no counterpart in the reference): given dL/dx_K, walk the steps backwards with the
// fused self-interaction VJP of adjoint.cu; positions are recomputed per segment from
// checkpoints stored by the forward pass every `every` steps (sqrt(K) by default), so the tape
// holds K/every checkpoints plus one segment of stage positions.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "adjoint.h"
#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {

namespace {

// ElementBase::move with one weight: x += (S)dt * wt * u, evaluated in double, stored in float
__global__ void move1_kernel(int n, const float* __restrict__ x, const float* __restrict__ y,
                             const float* __restrict__ u, const float* __restrict__ v, float h,
                             float* __restrict__ xo, float* __restrict__ yo) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  xo[i] = (float)((double)x[i] + (double)h * (double)u[i]);
  yo[i] = (float)((double)y[i] + (double)h * (double)v[i]);
}

// ElementBase::move with two weights: u = wt1 u1 + wt2 u2 (double -> float); x += (S)dt * u
__global__ void move2_kernel(int n, float* __restrict__ x, float* __restrict__ y,
                             const float* __restrict__ u1, const float* __restrict__ v1,
                             const float* __restrict__ u2, const float* __restrict__ v2, float dt) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float uu = (float)(0.25 * (double)u1[i] + 0.75 * (double)u2[i]);
  const float vv = (float)(0.25 * (double)v1[i] + 0.75 * (double)v2[i]);
  x[i] = x[i] + dt * uu;
  y[i] = y[i] + dt * vv;
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

// One forward step from (x, y) into (xo, yo) (may alias); ys/yy receive the RK2 stage position.
int step(obs_context* ctx, int core, int accum, int order, int n, const float* x, const float* y, const float* r,
         const float* s, double fsx, double fsy, double dt, float* xo, float* yo, float* tmp,
         float* stage_x, float* stage_y, bool want_end) {
  float *u1 = tmp, *v1 = tmp + n, *u2 = tmp + 2 * n, *v2 = tmp + 3 * n;
  int st = velocity(ctx, core, accum, n, x, y, r, s, fsx, fsy, u1, v1);
  if (st) return st;
  if (order == 1) {
    if (want_end) {
      move1_kernel<<<grid_of(n), 256, 0, ctx->stream>>>(n, x, y, u1, v1, (float)dt, xo, yo);
      ctx->launches++;
    }
    return cuda_status(cudaGetLastError());
  }
  move1_kernel<<<grid_of(n), 256, 0, ctx->stream>>>(n, x, y, u1, v1, (float)(2.0 / 3.0 * dt), stage_x, stage_y);
  ctx->launches++;
  if (!want_end) return cuda_status(cudaGetLastError());
  st = velocity(ctx, core, accum, n, stage_x, stage_y, r, s, fsx, fsy, u2, v2);
  if (st) return st;
  if (xo != x) {
    cudaError_t e = cudaMemcpyAsync(xo, x, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(yo, y, (size_t)n * 4, cudaMemcpyDeviceToDevice, ctx->stream);
    if (e != cudaSuccess) return cuda_status(e);
  }
  move2_kernel<<<grid_of(n), 256, 0, ctx->stream>>>(n, xo, yo, u1, v1, u2, v2, (float)dt);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

}  // namespace

int run_advect(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y,
               const float* r, const float* s, double fsx, double fsy, double dt, int nsteps) {
  if (n == 0 || nsteps == 0) return OBS_OK;
  int st = ctx->state.ensure((size_t)6 * n * 4 + 1024, ctx->stream);
  if (st) return st;
  float* tmp = ctx->state.as<float>();
  float* sx = tmp + 4 * (size_t)n;
  float* sy = sx + n;
  for (int k = 0; k < nsteps && !st; ++k)
    st = step(ctx, core, accum, order, n, x, y, r, s, fsx, fsy, dt, x, y, tmp, sx, sy, true);
  return st;
}

int run_advect_vjp(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                   const float* r, const float* s, double fsx, double fsy, double dt, int nsteps, int every,
                   const float* lx_in, const float* ly_in, float* gs, float* gx0, float* gy0,
                   long long* peak_bytes) {
  if (n == 0 || nsteps == 0) return OBS_OK;
  const int C = every > 0 ? std::min(every, nsteps) : std::max(1, (int)std::ceil(std::sqrt((double)nsteps)));
  const int nck = (nsteps + C - 1) / C;
  const size_t N = (size_t)n;
  // layout (floats): checkpoints nck*2N | segment x C*2N | segment stage C*2N | forward tmp 4N |
  //                  working x 2N | lambda 2N | cotangent 2N | vjp out 2N
  const size_t total = (size_t)nck * 2 * N + (size_t)C * 4 * N + 4 * N + 8 * N;
  int st = ctx->state.ensure(total * 4 + 1024, ctx->stream);
  if (st) return st;
  float* base = ctx->state.as<float>();
  float* ck = base;
  float* segx = ck + (size_t)nck * 2 * N;
  float* segy = segx + (size_t)C * 2 * N;
  float* tmp = segy + (size_t)C * 2 * N;
  float* wx = tmp + 4 * N;
  float* wy = wx + N;
  float* lx = wy + N;
  float* ly = lx + N;
  float* bu = ly + N;
  float* bv = bu + N;
  float* ox = bv + N;
  float* oy = ox + N;
  cudaStream_t strm = ctx->stream;
  auto copy = [&](float* d, const float* src, size_t cnt) {
    return cuda_status(cudaMemcpyAsync(d, src, cnt * 4, cudaMemcpyDeviceToDevice, strm));
  };
  // forward sweep storing checkpoints at steps 0, C, 2C, ...
  if ((st = copy(wx, x0, N)) || (st = copy(wy, y0, N))) return st;
  for (int k = 0; k < nsteps; ++k) {
    if (k % C == 0) {
      float* c = ck + (size_t)(k / C) * 2 * N;
      if ((st = copy(c, wx, N)) || (st = copy(c + N, wy, N))) return st;
    }
    if ((st = step(ctx, core, accum, order, n, wx, wy, r, s, fsx, fsy, dt, wx, wy, tmp, ox, oy, true))) return st;
  }
  if ((st = copy(lx, lx_in, N)) || (st = copy(ly, ly_in, N))) return st;
  // reverse, one segment at a time
  for (int seg = nck - 1; seg >= 0; --seg) {
    const int k0 = seg * C, k1 = std::min(k0 + C, nsteps);
    const float* c = ck + (size_t)seg * 2 * N;
    if ((st = copy(wx, c, N)) || (st = copy(wy, c + N, N))) return st;
    for (int k = k0; k < k1; ++k) {
      float* xk = segx + (size_t)(k - k0) * 2 * N;
      float* yk = segy + (size_t)(k - k0) * 2 * N;
      if ((st = copy(xk, wx, N)) || (st = copy(xk + N, wy, N))) return st;
      if ((st = step(ctx, core, accum, order, n, wx, wy, r, s, fsx, fsy, dt, wx, wy, tmp, yk, yk + N, k + 1 < k1)))
        return st;
    }
    for (int k = k1 - 1; k >= k0; --k) {
      const float* xk = segx + (size_t)(k - k0) * 2 * N;
      const float* yk = segy + (size_t)(k - k0) * 2 * N;
      if (order == 2) {
        // stage 2: cotangent 3/4 dt lam on u(y_k)
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)(0.75 * dt), lx, 0.0f, nullptr, bu);
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)(0.75 * dt), ly, 0.0f, nullptr, bv);
        ctx->launches += 2;
        cudaError_t e = cudaMemsetAsync(ox, 0, 2 * N * 4, strm);
        if (e != cudaSuccess) return cuda_status(e);
        if ((st = run_adjoint(ctx, core, accum, 1, n, yk, yk + N, r, s, n, yk, yk + N, r, s, bu, bv, ox, oy, gs, 0)))
          return st;
        // stage 1: 1/4 dt lam + 2/3 dt ybar on u(x_k); lam += ybar
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)(0.25 * dt), lx, (float)(2.0 / 3.0 * dt), ox, bu);
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)(0.25 * dt), ly, (float)(2.0 / 3.0 * dt), oy, bv);
        add_kernel<<<grid_of(n), 256, 0, strm>>>(n, lx, ox);
        add_kernel<<<grid_of(n), 256, 0, strm>>>(n, ly, oy);
        ctx->launches += 4;
      } else {
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)dt, lx, 0.0f, nullptr, bu);
        axpby_kernel<<<grid_of(n), 256, 0, strm>>>(n, (float)dt, ly, 0.0f, nullptr, bv);
        ctx->launches += 2;
      }
      cudaError_t e = cudaMemsetAsync(ox, 0, 2 * N * 4, strm);
      if (e != cudaSuccess) return cuda_status(e);
      if ((st = run_adjoint(ctx, core, accum, 1, n, xk, xk + N, r, s, n, xk, xk + N, r, s, bu, bv, ox, oy, gs, 0)))
        return st;
      add_kernel<<<grid_of(n), 256, 0, strm>>>(n, lx, ox);
      add_kernel<<<grid_of(n), 256, 0, strm>>>(n, ly, oy);
      ctx->launches += 2;
      if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
    }
  }
  if (gx0) { add_kernel<<<grid_of(n), 256, 0, strm>>>(n, gx0, lx); ctx->launches++; }
  if (gy0) { add_kernel<<<grid_of(n), 256, 0, strm>>>(n, gy0, ly); ctx->launches++; }
  if (peak_bytes)
    *peak_bytes = (long long)(ctx->work.cap + ctx->io.cap + ctx->dense.cap + ctx->state.cap);
  return cuda_status(cudaGetLastError());
}

}  // namespace obs
