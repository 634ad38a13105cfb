// lu.cu -- FP64 dense solve on the device for the BEM panel strengths.
//
// The reference solves its BEM system with Eigen's GMRES in FP32 on the host
// (src/BEM.h:169-234).  Here the system is solved in FP64 on the GPU by LU factorisation with
// partial pivoting (right-looking, one launch per column) followed by two triangular solves.
//
// Step k (kernel lu_step): pivot row p_k and a snapshot of column k (taken by the previous
// step, so no CTA reads a column another CTA is rewriting) are read; every CTA swaps rows k
// and p_k in its own columns and applies the rank-1 update to its columns right of k; the CTA
// owning column k writes the final L column; the CTA owning column k+1 snapshots it and finds
// the next pivot.  Columns are owned in slabs of LU_CW, so the update is coalesced down each
// column.
#include <cfloat>
#include <cmath>

#include "obs_context.h"
#include "obs_device.cuh"
#include "panels.h"

namespace obs {

namespace {

constexpr int LU_THREADS = 256;
constexpr int LU_CW = 8;   // columns per CTA

// block-wide argmax of |v| (value, index); ties keep the smaller index
__device__ void block_argmax(double v, int idx, double* s_val, int* s_idx, double* out_val, int* out_idx) {
  const int t = threadIdx.x;
  s_val[t] = v;
  s_idx[t] = idx;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (t < o) {
      const double a = s_val[t], b = s_val[t + o];
      const int ia = s_idx[t], ib = s_idx[t + o];
      if (b > a || (b == a && ib < ia)) { s_val[t] = b; s_idx[t] = ib; }
    }
    __syncthreads();
  }
  if (t == 0) { *out_val = s_val[0]; *out_idx = s_idx[0]; }
  __syncthreads();
}

// snapshot of column 0 and its pivot
__global__ void lu_init_kernel(const double* __restrict__ A, int n, double* __restrict__ col, int* __restrict__ piv) {
  __shared__ double s_val[LU_THREADS];
  __shared__ int s_idx[LU_THREADS];
  __shared__ double best;
  __shared__ int besti;
  double bv = -1.0;
  int bi = 0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double a = A[i];
    col[i] = a;
    const double m = fabs(a);
    if (m > bv) { bv = m; bi = i; }
  }
  block_argmax(bv, bi, s_val, s_idx, &best, &besti);
  if (threadIdx.x == 0) piv[0] = besti;
}

__global__ void __launch_bounds__(LU_THREADS)
lu_step_kernel(double* __restrict__ A, int n, int k, const double* __restrict__ col_cur,
               double* __restrict__ col_next, int* __restrict__ piv, int* status) {
  __shared__ double s_ak[LU_CW], s_ap[LU_CW];
  __shared__ double s_val[LU_THREADS];
  __shared__ int s_idx[LU_THREADS];
  __shared__ double best;
  __shared__ int besti;
  const int c0 = blockIdx.x * LU_CW;
  const int p = piv[k];
  const double apk = col_cur[p];
  if (apk == 0.0 && threadIdx.x == 0 && blockIdx.x == 0) record_failure(status, DEV_ERR_SINGULAR, 401, k, p);
  const double inv = 1.0 / apk;
  // row swap values of this CTA's columns
  if (threadIdx.x < LU_CW) {
    const int c = c0 + threadIdx.x;
    if (c < n) {
      s_ak[threadIdx.x] = A[(size_t)c * n + k];
      s_ap[threadIdx.x] = A[(size_t)c * n + p];
    }
  }
  __syncthreads();
  // update rows k+1.. of the columns right of k (the swapped-in old row k sits at row p)
  for (int i = k + 1 + threadIdx.x; i < n; i += LU_THREADS) {
    const double li = ((i == p) ? col_cur[k] : col_cur[i]) * inv;
#pragma unroll
    for (int q = 0; q < LU_CW; ++q) {
      const int c = c0 + q;
      if (c > k && c < n) {
        double* a = A + (size_t)c * n;
        const double v = (i == p) ? s_ak[q] : a[i];
        a[i] = fma(-li, s_ap[q], v);
      } else if (c == k) {
        A[(size_t)k * n + i] = li;     // final L column
      }
    }
  }
  // row k (and the L part's row swap) of this CTA's columns
  if (threadIdx.x < LU_CW) {
    const int c = c0 + threadIdx.x;
    if (c < n) {
      if (c < k && p != k) {          // swap the L part
        A[(size_t)c * n + k] = s_ap[threadIdx.x];
        A[(size_t)c * n + p] = s_ak[threadIdx.x];
      } else if (c >= k) {
        A[(size_t)c * n + k] = s_ap[threadIdx.x];
      }
    }
  }
  // the owner of column k+1 snapshots it and finds the next pivot
  const int c1 = k + 1;
  if (c1 < n && c1 >= c0 && c1 < c0 + LU_CW) {
    __syncthreads();
    const double* a = A + (size_t)c1 * n;
    double bv = -1.0;
    int bi = c1;
    for (int i = c1 + threadIdx.x; i < n; i += LU_THREADS) {
      const double v = a[i];
      col_next[i] = v;
      const double m = fabs(v);
      if (m > bv) { bv = m; bi = i; }
    }
    block_argmax(bv, bi, s_val, s_idx, &best, &besti);
    if (threadIdx.x == 0) piv[c1] = besti;
  }
}

// P b, then L y = P b (unit lower), then U x = y; b held in shared memory by one CTA
__global__ void __launch_bounds__(1024) lu_solve_kernel(const double* __restrict__ LU, int n,
                                                        const int* __restrict__ piv, double* __restrict__ x) {
  extern __shared__ double sb[];
  for (int i = threadIdx.x; i < n; i += blockDim.x) sb[i] = x[i];
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int k = 0; k < n; ++k) {
      const int p = piv[k];
      if (p != k) { const double t = sb[k]; sb[k] = sb[p]; sb[p] = t; }
    }
  }
  __syncthreads();
  for (int k = 0; k < n; ++k) {
    const double yk = sb[k];
    const double* col = LU + (size_t)k * n;
    for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x) sb[i] = fma(-col[i], yk, sb[i]);
    __syncthreads();
  }
  for (int k = n - 1; k >= 0; --k) {
    const double* col = LU + (size_t)k * n;
    const double xk = sb[k] / col[k];
    __syncthreads();
    if (threadIdx.x == 0) sb[k] = xk;
    for (int i = threadIdx.x; i < k; i += blockDim.x) sb[i] = fma(-col[i], xk, sb[i]);
    __syncthreads();
  }
  for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = sb[i];
}

// r = A x - b per row (column-major A: for fixed j consecutive rows are contiguous)
__global__ void residual_kernel(const double* __restrict__ A, int n, const double* __restrict__ x,
                                const double* __restrict__ b, double* __restrict__ r) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  double s = 0.0;
  for (int j = 0; j < n; ++j) s = fma(A[(size_t)j * n + i], x[j], s);
  r[i] = s - b[i];
}

__global__ void norms_kernel(const double* __restrict__ r, const double* __restrict__ b, int n, double* out) {
  __shared__ double s1[1024], s2[1024];
  double a = 0.0, c = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) { a += r[i] * r[i]; c += b[i] * b[i]; }
  s1[threadIdx.x] = a;
  s2[threadIdx.x] = c;
  __syncthreads();
  for (int o = blockDim.x / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) { s1[threadIdx.x] += s1[threadIdx.x + o]; s2[threadIdx.x] += s2[threadIdx.x + o]; }
    __syncthreads();
  }
  if (threadIdx.x == 0) { out[0] = sqrt(s1[0]); out[1] = sqrt(s2[0]); }
}

}  // namespace

int lu_factor_f64(obs_context* ctx, int n, double* lu, int* piv) {
  if (n <= 0) return OBS_ERR_ARG;
  const size_t need = 256 + 2 * (size_t)n * sizeof(double);
  int s = ctx->work.ensure(need, ctx->stream);
  if (s) return s;
  double* col0 = ctx->work.as<double>(256);
  double* col1 = col0 + n;
  cudaStream_t st = ctx->stream;
  lu_init_kernel<<<1, LU_THREADS, 0, st>>>(lu, n, col0, piv);
  ctx->launches++;
  const int blocks = (n + LU_CW - 1) / LU_CW;
  for (int k = 0; k < n; ++k) {
    const double* cur = (k & 1) ? col1 : col0;
    double* nxt = (k & 1) ? col0 : col1;
    lu_step_kernel<<<blocks, LU_THREADS, 0, st>>>(lu, n, k, cur, nxt, piv, ctx->d_status);
    ctx->launches++;
  }
  return cuda_status(cudaGetLastError());
}

int lu_solve_f64(obs_context* ctx, int n, const double* lu, const int* piv, double* x) {
  const size_t smem = (size_t)n * sizeof(double);
  if (smem > 200 * 1024) return OBS_ERR_UNSUPPORTED;
  cudaError_t e = cudaFuncSetAttribute(lu_solve_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  if (e != cudaSuccess) return cuda_status(e);
  lu_solve_kernel<<<1, 1024, smem, ctx->stream>>>(lu, n, piv, x);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

int residual_f64(obs_context* ctx, int n, const double* A, const double* x, const double* b, double* rel) {
  const size_t off = 256 + 2 * (size_t)n * sizeof(double);
  int s = ctx->work.ensure(off + ((size_t)n + 2) * sizeof(double), ctx->stream);
  if (s) return s;
  double* r = ctx->work.as<double>(off);
  double* nr = r + n;
  residual_kernel<<<(n + 255) / 256, 256, 0, ctx->stream>>>(A, n, x, b, r);
  norms_kernel<<<1, 1024, 0, ctx->stream>>>(r, b, n, nr);
  ctx->launches += 2;
  double h[2] = {0.0, 0.0};
  cudaError_t e = cudaMemcpyAsync(h, nr, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) return cuda_status(e);
  // the reference divides by 1 when ||b|| = 0 (src/BEM.h:227-229)
  *rel = h[0] / (h[1] == 0.0 ? 1.0 : h[1]);
  return OBS_OK;
}

}  // namespace obs
