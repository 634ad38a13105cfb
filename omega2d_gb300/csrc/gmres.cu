// gmres.cu -- restarted GMRES in FP64 on the device for the BEM panel strengths.
//
// The reference solves its BEM system with Eigen's GMRES in FP32 on the host (src/BEM.h:169-234:
// Eigen::GMRES<MatrixX<float>> with Eigen's defaults -- restart 30, diagonal preconditioner,
// tolerance = machine epsilon of the scalar).  Here the same Krylov method runs in FP64 on the
// GPU: right diagonal (Jacobi) preconditioning, classical Gram-Schmidt with one
// reorthogonalisation pass (CGS2), Givens rotations for the small least-squares problem, all on
// the device.  One restart cycle is launched without a host round trip; once the residual
// estimate drops below the tolerance the remaining kernels of the cycle return at once (a
// device flag), and the host reads back only the true residual at the end of each cycle.
//
// Cost per iteration: one FP64 matrix-vector product (n^2 doubles from HBM: the bound) plus
// O(n j) vector work.  Every reduction has a fixed order, so results are reproducible.
#include <cmath>
#include <vector>

#include "obs_context.h"
#include "obs_device.cuh"
#include "panels.h"

namespace obs {

namespace {

constexpr int GM_THREADS = 256;
constexpr int GM_CHUNK = 128;   // columns per matrix-vector partial

// device state of one solve
struct GmState {
  int done;        // 1: converged inside the cycle (later kernels of the cycle return)
  int kdone;       // iterations completed in this cycle
  double beta;     // residual norm at the start of the cycle
  double tolabs;   // absolute tolerance on the residual norm
};

// part[c][i] = sum_{j in chunk c} A[j*n + i] * (x[j] * dinv[j])   (column-major A)
__global__ void __launch_bounds__(GM_THREADS) gemv_part_kernel(const double* __restrict__ A, int n,
                                                               const double* __restrict__ x,
                                                               const double* __restrict__ dinv,
                                                               double* __restrict__ part, const GmState* st) {
  if (st && st->done) return;
  __shared__ double xs[GM_CHUNK];
  const int c = blockIdx.y;
  const int j0 = c * GM_CHUNK, j1 = min(n, j0 + GM_CHUNK);
  for (int j = j0 + threadIdx.x; j < j1; j += GM_THREADS) xs[j - j0] = dinv ? x[j] * dinv[j] : x[j];
  __syncthreads();
  const int i = blockIdx.x * GM_THREADS + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  const double* a = A + (size_t)j0 * n + i;
#pragma unroll 8
  for (int j = 0; j < j1 - j0; ++j) s = fma(a[(size_t)j * n], xs[j], s);
  part[(size_t)c * n + i] = s;
}

// y = sum_c part[c]  (or y = b - sum when b is given)
__global__ void gemv_sum_kernel(const double* __restrict__ part, int nchunk, int n, const double* __restrict__ b,
                                double* __restrict__ y, const GmState* st) {
  if (st && st->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * n + i];
  y[i] = b ? b[i] - s : s;
}

// block-wide sum of one value per thread (fixed order); result valid in thread 0
__device__ double block_sum(double v, double* sh) {
  const int t = threadIdx.x;
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((t & 31) == 0) sh[t >> 5] = v;
  __syncthreads();
  double s = 0.0;
  if (t == 0)
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += sh[w];
  __syncthreads();
  return s;
}

// h[k] (+)= V_k . w for k = 0..j (one block per k)
__global__ void __launch_bounds__(GM_THREADS) dots_kernel(const double* __restrict__ V, int n,
                                                          const double* __restrict__ w, double* __restrict__ h,
                                                          int accumulate, const GmState* st) {
  if (st->done) return;
  __shared__ double sh[GM_THREADS / 32];
  const int k = blockIdx.x;
  const double* v = V + (size_t)k * n;
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += GM_THREADS) s = fma(v[i], w[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) h[k] = accumulate ? h[k] + s : s;
}

// w -= sum_{k<=j} V_k c[k]
__global__ void update_kernel(const double* __restrict__ V, int n, int j, const double* __restrict__ c,
                              double* __restrict__ w, const GmState* st) {
  if (st->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = w[i];
  for (int k = 0; k <= j; ++k) s = fma(-V[(size_t)k * n + i], c[k], s);
  w[i] = s;
}

// h[k] += h2[k], k < cnt
__global__ void hadd_kernel(double* __restrict__ h, const double* __restrict__ h2, int cnt, const GmState* st) {
  if (st->done) return;
  for (int k = threadIdx.x; k < cnt; k += blockDim.x) h[k] += h2[k];
}

// ||w|| into *out (one block)
__global__ void __launch_bounds__(1024) norm_kernel(const double* __restrict__ w, int n, double* out,
                                                     const GmState* st) {
  if (st && st->done) return;
  __shared__ double sh[32];
  double s = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) s = fma(w[i], w[i], s);
  s = block_sum(s, sh);
  if (threadIdx.x == 0) *out = sqrt(s);
}

// v = w / *nrm
__global__ void scale_kernel(const double* __restrict__ w, int n, const double* nrm, double* __restrict__ v,
                             const GmState* st) {
  if (st && st->done) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = w[i] / *nrm;
}

// start of a cycle: beta = ||r||, g = (beta, 0, ...), V_0 = r / beta; done when beta is small
__global__ void cycle_start_kernel(GmState* st, const double* nrm, double* g, int m) {
  st->beta = *nrm;
  st->kdone = 0;
  st->done = (*nrm <= st->tolabs) ? 1 : 0;
  for (int k = 0; k <= m; ++k) g[k] = 0.0;
  g[0] = *nrm;
}

// Givens: rotate column j of H (ldh = m+1) by the previous rotations, make a new one, update g
__global__ void givens_kernel(double* H, int ldh, int j, double* cs, double* sn, double* g, GmState* st) {
  if (st->done) return;
  double* hc = H + (size_t)j * ldh;
  for (int k = 0; k < j; ++k) {
    const double t = cs[k] * hc[k] + sn[k] * hc[k + 1];
    hc[k + 1] = -sn[k] * hc[k] + cs[k] * hc[k + 1];
    hc[k] = t;
  }
  const double a = hc[j], b = hc[j + 1];
  const double r = hypot(a, b);
  const double c = (r == 0.0) ? 1.0 : a / r, s = (r == 0.0) ? 0.0 : b / r;
  cs[j] = c;
  sn[j] = s;
  hc[j] = r;
  hc[j + 1] = 0.0;
  g[j + 1] = -s * g[j];
  g[j] = c * g[j];
  st->kdone = j + 1;
  if (fabs(g[j + 1]) <= st->tolabs || b == 0.0) st->done = 1;
}

// y = R^{-1} g (R upper triangular k x k in H), into yv
__global__ void backsub_kernel(const double* H, int ldh, const double* g, double* yv, const GmState* st) {
  const int k = st->kdone;
  for (int i = k - 1; i >= 0; --i) {
    double s = g[i];
    for (int q = i + 1; q < k; ++q) s -= H[(size_t)q * ldh + i] * yv[q];
    yv[i] = s / H[(size_t)i * ldh + i];
  }
}

// x += Dinv V y
__global__ void xupdate_kernel(const double* __restrict__ V, int n, const double* __restrict__ yv,
                               const double* __restrict__ dinv, double* __restrict__ x, const GmState* st) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int k = 0; k < st->kdone; ++k) s = fma(V[(size_t)k * n + i], yv[k], s);
  x[i] += dinv ? s * dinv[i] : s;
}

__global__ void diag_inv_kernel(const double* __restrict__ A, int n, double* __restrict__ dinv) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double d = A[(size_t)i * n + i];
  dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
}

}  // namespace

int gmres_f64(obs_context* ctx, int n, const double* A, const double* b, double* x, double tol, int restart,
              int maxiter, int* iters_out, double* rel_residual) {
  if (n <= 0 || !A || !b || !x) return OBS_ERR_ARG;
  const int m = std::max(1, std::min(restart, n));
  const int nchunk = (n + GM_CHUNK - 1) / GM_CHUNK;
  const size_t N = (size_t)n;
  // work: state | V (m+1) n | H (m+1) m | g, cs, sn, y, h2 (m+1 each) | dinv n | w n | part nchunk n | nrm
  auto al = [](size_t b_) { return (b_ + 255) & ~(size_t)255; };
  const size_t o_st = 0;
  const size_t o_V = 256;
  const size_t o_H = o_V + al((size_t)(m + 1) * N * 8);
  const size_t o_g = o_H + al((size_t)(m + 1) * m * 8);
  const size_t o_cs = o_g + al((size_t)(m + 1) * 8);
  const size_t o_sn = o_cs + al((size_t)(m + 1) * 8);
  const size_t o_y = o_sn + al((size_t)(m + 1) * 8);
  const size_t o_h2 = o_y + al((size_t)(m + 1) * 8);
  const size_t o_d = o_h2 + al((size_t)(m + 1) * 8);
  const size_t o_w = o_d + al(N * 8);
  const size_t o_p = o_w + al(N * 8);
  const size_t o_n = o_p + al((size_t)nchunk * N * 8);
  const size_t total = o_n + 256;
  int s = ctx->work.ensure(total, ctx->stream);
  if (s) return s;
  GmState* st = ctx->work.as<GmState>(o_st);
  double* V = ctx->work.as<double>(o_V);
  double* H = ctx->work.as<double>(o_H);
  double* g = ctx->work.as<double>(o_g);
  double* cs = ctx->work.as<double>(o_cs);
  double* sn = ctx->work.as<double>(o_sn);
  double* yv = ctx->work.as<double>(o_y);
  double* h2 = ctx->work.as<double>(o_h2);
  double* dinv = ctx->work.as<double>(o_d);
  double* w = ctx->work.as<double>(o_w);
  double* part = ctx->work.as<double>(o_p);
  double* nrm = ctx->work.as<double>(o_n);
  cudaStream_t strm = ctx->stream;
  const int gb = (n + GM_THREADS - 1) / GM_THREADS;
  const dim3 ggrid(gb, nchunk);
  auto launched = [&](int k) { ctx->launches += k; };

  diag_inv_kernel<<<gb, GM_THREADS, 0, strm>>>(A, n, dinv);
  norm_kernel<<<1, 1024, 0, strm>>>(b, n, nrm, nullptr);
  launched(2);
  double bnorm = 0.0;
  cudaError_t e = cudaMemcpyAsync(&bnorm, nrm, 8, cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
  if (e != cudaSuccess) return cuda_status(e);
  const double bref = (bnorm == 0.0) ? 1.0 : bnorm;   // src/BEM.h:227-229 divides by 1 then
  GmState h0{0, 0, 0.0, tol * bref};
  if ((e = cudaMemcpyAsync(st, &h0, sizeof(h0), cudaMemcpyHostToDevice, strm)) != cudaSuccess) return cuda_status(e);

  int total_it = 0;
  double rel = 0.0;
  for (;;) {
    // r = b - A Dinv (D x) ... x is the unpreconditioned iterate: r = b - A x
    gemv_part_kernel<<<ggrid, GM_THREADS, 0, strm>>>(A, n, x, nullptr, part, nullptr);
    gemv_sum_kernel<<<gb, GM_THREADS, 0, strm>>>(part, nchunk, n, b, w, nullptr);
    norm_kernel<<<1, 1024, 0, strm>>>(w, n, nrm, nullptr);
    launched(3);
    double rn = 0.0;
    e = cudaMemcpyAsync(&rn, nrm, 8, cudaMemcpyDeviceToHost, strm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
    if (e != cudaSuccess) return cuda_status(e);
    rel = rn / bref;
    if (!(rn > tol * bref) || total_it >= maxiter) break;   // converged (or NaN) / out of budget
    cycle_start_kernel<<<1, 1, 0, strm>>>(st, nrm, g, m);
    scale_kernel<<<gb, GM_THREADS, 0, strm>>>(w, n, nrm, V, nullptr);
    launched(2);
    const int mc = std::min(m, maxiter - total_it);
    for (int j = 0; j < mc; ++j) {
      double* Hj = H + (size_t)j * (m + 1);
      // w = A Dinv v_j
      gemv_part_kernel<<<ggrid, GM_THREADS, 0, strm>>>(A, n, V + (size_t)j * N, dinv, part, st);
      gemv_sum_kernel<<<gb, GM_THREADS, 0, strm>>>(part, nchunk, n, nullptr, w, st);
      // CGS2: h = V^T w; w -= V h; h2 = V^T w; w -= V h2; h += h2
      dots_kernel<<<j + 1, GM_THREADS, 0, strm>>>(V, n, w, Hj, 0, st);
      update_kernel<<<gb, GM_THREADS, 0, strm>>>(V, n, j, Hj, w, st);
      dots_kernel<<<j + 1, GM_THREADS, 0, strm>>>(V, n, w, h2, 0, st);
      update_kernel<<<gb, GM_THREADS, 0, strm>>>(V, n, j, h2, w, st);
      hadd_kernel<<<1, 64, 0, strm>>>(Hj, h2, j + 1, st);
      norm_kernel<<<1, 1024, 0, strm>>>(w, n, Hj + j + 1, st);
      scale_kernel<<<gb, GM_THREADS, 0, strm>>>(w, n, Hj + j + 1, V + (size_t)(j + 1) * N, st);
      givens_kernel<<<1, 1, 0, strm>>>(H, m + 1, j, cs, sn, g, st);
      launched(10);
    }
    backsub_kernel<<<1, 1, 0, strm>>>(H, m + 1, g, yv, st);
    xupdate_kernel<<<gb, GM_THREADS, 0, strm>>>(V, n, yv, dinv, x, st);
    launched(2);
    int kd = 0;
    e = cudaMemcpyAsync(&kd, &st->kdone, 4, cudaMemcpyDeviceToHost, strm);
    if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
    if (e != cudaSuccess) return cuda_status(e);
    total_it += std::max(kd, 1);
  }
  if (iters_out) *iters_out = total_it;
  if (rel_residual) *rel_residual = rel;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  return (rel <= tol) ? OBS_OK : OBS_ERR_NO_CONVERGENCE;
}

}  // namespace obs
