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
// Cost per iteration (per-step path): one FP64 matrix-vector product (n^2 doubles from HBM)
// plus O(n j) vector work; the fused cycle below reads the FP32 plane of A from L2 instead.
// Every reduction has a fixed order, so results are reproducible.
#include <algorithm>
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
  double tolcyc;   // the cycle's target: tolabs, or a relative reduction when the cycle's
                   // products use the FP32 plane of A (iterative refinement)
};

// part[c][i] = sum_{j in chunk c} A[j*n + i] * (x[j] * dinv[j])   (column-major A); nothing when
// nz is given and *nz == 0 (x known to be zero)
__global__ void __launch_bounds__(GM_THREADS) gemv_part_kernel(const double* __restrict__ A, int n,
                                                               const double* __restrict__ x,
                                                               const double* __restrict__ dinv,
                                                               double* __restrict__ part, const GmState* st,
                                                               const unsigned* nz = nullptr) {
  if ((st && st->done) || (nz && *nz == 0)) return;
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

// start of a cycle, on thread 0: beta = ||r||, g = (beta, 0, ...); done when beta is at most
// tolabs = tol ||b|| (tol alone when b = 0, src/BEM.h:227-229); the cycle's target is
// max(tolabs, eta beta), eta applying only when the plane's flag says that A's entries were
// rounded to FP32 (bit 1); the grid barrier's arrival counter cleared for the cycle launch
// that follows.  Over the grid: V_0 = r / beta.
__global__ void cycle_start_scale_kernel(GmState* st, const double* nrm, const double* bnrm, double tol, double* g,
                                         int m, double eta, const unsigned* plane_flag, const double* __restrict__ w,
                                         int n, double* __restrict__ v, unsigned* bar) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i == 0) {
    st->tolabs = tol * ((*bnrm == 0.0) ? 1.0 : *bnrm);
    st->beta = *nrm;
    st->kdone = 0;
    st->done = (*nrm <= st->tolabs) ? 1 : 0;
    st->tolcyc = fmax(st->tolabs, ((*plane_flag & 2u) ? eta : 0.0) * *nrm);
    for (int k = 0; k <= m; ++k) g[k] = 0.0;
    g[0] = *nrm;
    *bar = 0u;
  }
  if (i < n) v[i] = w[i] / *nrm;
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
  if (fabs(g[j + 1]) <= st->tolcyc || b == 0.0) st->done = 1;
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

// The last block of a grid to arrive (a counter that it resets) sums the blocks' partials in
// block order: the sum does not depend on timing.  Returns the total in thread 0 of that block.
__device__ bool last_block_sum(double v, double* bpart, unsigned* cnt, double* sh, double* total) {
  __shared__ bool last;
  v = block_sum(v, sh);
  if (threadIdx.x == 0) {
    bpart[blockIdx.x] = v;
    __threadfence();
    last = atomicAdd(cnt, 1u) == gridDim.x - 1;
  }
  __syncthreads();
  if (!last) return false;
  __threadfence();
  if (threadIdx.x < 32) {
    double t = 0.0;
    for (int k = threadIdx.x; k < (int)gridDim.x; k += 32) t += __ldcg(bpart + k);
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (threadIdx.x == 0) {
      *total = t;
      *cnt = 0u;
    }
  }
  return true;
}

// Start of a solve: Dinv = 1 / diag(A) (1 where the diagonal is 0), *nz = 1 when any x[i] != 0,
// *bnrm = ||b||
__global__ void __launch_bounds__(GM_THREADS) prep_kernel(const double* __restrict__ A, const double* __restrict__ b,
                                                          const double* __restrict__ x, int n, double* __restrict__ dinv,
                                                          double* bpart, unsigned* cnt, double* bnrm, unsigned* nz) {
  __shared__ double sh[32];
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double bb = 0.0;
  int z = 0;
  if (i < n) {
    const double d = A[(size_t)i * n + i];
    dinv[i] = (d != 0.0) ? 1.0 / d : 1.0;
    bb = b[i] * b[i];
    z = x[i] != 0.0;
  }
  if (__syncthreads_or(z) && threadIdx.x == 0) atomicOr(nz, 1u);
  double t;
  if (last_block_sum(bb, bpart, cnt, sh, &t) && threadIdx.x == 0) *bnrm = sqrt(t);
}

// y = b - sum_c part[c] (y = b when nz is given and *nz == 0) and *out = ||y|| (*alt then)
__global__ void __launch_bounds__(GM_THREADS) gemv_sum_norm_kernel(const double* __restrict__ part, int nchunk, int n,
                                                                   const double* __restrict__ b, double* __restrict__ y,
                                                                   const unsigned* nz, double* bpart, unsigned* cnt,
                                                                   double* out, const double* alt) {
  __shared__ double sh[32];
  const bool zero = nz && *nz == 0;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  double r = 0.0;
  if (i < n) {
    if (zero) {
      r = b[i];
    } else {
      double s = 0.0;
      for (int c = 0; c < nchunk; ++c) s += part[(size_t)c * n + i];
      r = b[i] - s;
    }
    y[i] = r;
  }
  if (zero) {
    if (blockIdx.x == 0 && threadIdx.x == 0) *out = *alt;
    return;
  }
  double t;
  if (last_block_sum(r * r, bpart, cnt, sh, &t) && threadIdx.x == 0) *out = sqrt(t);
}

// ---------------------------------------------------------------- one restart cycle in one launch
// FP64 arithmetic runs at a small fraction of the FP32 rate on this GPU, and the FP64 matrix
// (8 n^2 bytes) does not fit in L2, so the operator product of the fused cycle uses the FP32
// plane of A (hi: its top 24 significand bits, 4 n^2 bytes, which stays in L2 across the
// cycle's iterations) against the vector in double-float (hi + lo), each product formed exactly
// with an FMA and summed in an unevaluated (S, s) pair.  The cycle thus solves with A_hi, whose
// entries carry a relative error below 2^-23, and stops at a relative reduction of 2^-20; the
// restart residual b - A x is formed with the FP64 matrix, so every restart corrects the
// solution against A itself (iterative refinement): the final residual meets the FP64
// tolerance.  A matrix whose entries are all exact in FP32 (bit 1 of the split's flag clear)
// is its own plane: its cycles run to the tolerance.  Inside the cycle the basis, w, the Gram-Schmidt dot products, the sums over
// blocks and the updates are double-float (hi + lo FP32 pairs, about 2^-48) on the FP32 pipes;
// the preconditioner is Dinv rounded to FP32 (used alike in the operator and in the update of
// x); the Hessenberg matrix, Givens rotations, back substitution and the update of x are FP64.
// Measured on the 4096 unknowns of a 2048-panel circle: an FP32 basis left each cycle's true
// residual 7x above its estimate (72 iterations instead of 57, the FP64 count); the
// double-float basis reproduces the FP64 cycle's residuals.

constexpr double kRefineEta = 9.5367431640625e-7;   // 2^-20: a cycle's relative reduction on A_hi
constexpr int GC_THREADS = 1024;
constexpr int GC_WARPS = GC_THREADS / 32;
constexpr int GC_MAXM = 64;                     // restart length supported by the fused kernel

// hi plane of A, from the bits of each double without FP64 arithmetic (double <-> float
// conversions run on the slow FP64 path of this GPU): the sign, the exponent and the top 23
// stored significand bits (truncated: relative error below 2^-23).  Flags entries outside
// 2^+-99 (other than 0), where the plane would lose precision or overflow.
__device__ __forceinline__ float hi_bits(double a, int& bad) {
  const unsigned long long u = (unsigned long long)__double_as_longlong(a);
  const int e = (int)((u >> 52) & 0x7ff);
  const unsigned long long mant = u & ((1ull << 52) - 1);
  const unsigned sign = (unsigned)(u >> 63) << 31;
  bad |= (e != 0 && (e < 1023 - 99 || e > 1023 + 99)) || (e == 0 && mant != 0);
  // bit 1: an entry the plane truncates (A_hi != A)
  bad |= (mant & ((1ull << 29) - 1)) ? 2 : 0;
  if (e == 0) return __uint_as_float(sign);
  return __uint_as_float(sign | ((unsigned)(e - 1023 + 127) << 23) | (unsigned)(mant >> 29));
}

// hi plane in column pairs, AH[(c/2) * n + i] = (hi(A[c][i]), hi(A[c+1][i])) (a zero column
// pads an odd order), so one 8-byte load feeds the f32x2 product of two columns
__global__ void split_hi_kernel(const double* __restrict__ A, int n, float2* __restrict__ AH,
                                int* __restrict__ range_flag) {
  // column pairs over blockIdx.y (grid-stride), rows over the block's threads: coalesced reads
  // of both columns and writes of the pair, no integer division per element
  int bad = 0;
  const size_t N = (size_t)n;
  const int npairs = (n + 1) / 2;
  for (int cp = blockIdx.y; cp < npairs; cp += gridDim.y) {
    const size_t c = 2 * (size_t)cp;
    const double* a0 = A + c * N;
    const double* a1 = A + (c + 1) * N;
    const bool two = c + 1 < N;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const float lo = hi_bits(a0[i], bad);
      const float hi = two ? hi_bits(a1[i], bad) : 0.0f;
      AH[(size_t)cp * N + i] = make_float2(lo, hi);
    }
  }
  bad = __syncthreads_or(bad & 1) | (__syncthreads_or(bad & 2) ? 2 : 0);
  if (bad && threadIdx.x == 0) atomicOr(range_flag, bad);
}

struct GcArgs {
  const float2* AH;                             // hi plane of A in column pairs
  const double* dinv;
  int n, m, mc;                                 // order, restart length, iterations this cycle
  int gpb;                                      // row groups a block owns (at most)
  const double* V0;                             // v_0 (n)
  float4* vsp;                                  // per column pair: hi of Dinv v_j, then negated
  float2* vsl;                                  // per column pair: negated lo of Dinv v_j
  double* x;
  float2* P;                                    // partials (double-float): [2][grid][m+2]
  unsigned* bar;                                // arrival counter, zeroed before each launch
  const unsigned* plane_flag;                   // bit 0: entries out of the plane's range
  GmState* st;
  int* status;
};

__device__ __forceinline__ void red_release_gpu(unsigned* p, unsigned v) {
  asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ unsigned ld_acquire_gpu(const unsigned* p) {
  unsigned v;
  asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// grid barrier number `nb` (0, 1, 2, ...) over co-resident blocks: a monotone arrival counter
// with release adds and acquire polls; the poll is bounded (about a second by default), after
// which the block records where it gave up and every block returns false.  `arrivals` is the
// count one barrier waits for (the grid size; the bounded-wait self-test asks for one more).
__device__ bool gc_barrier(unsigned* bar, int* status, unsigned nb, unsigned arrivals = 0,
                           unsigned max_polls = 1u << 21) {
  __syncthreads();
  int ok = 1;
  if (threadIdx.x == 0) {
    const unsigned target = (nb + 1) * (arrivals ? arrivals : gridDim.x);
    red_release_gpu(bar, 1u);
    unsigned it = 0;
    while (ld_acquire_gpu(bar) < target) {
      if (++it > max_polls) {
        record_failure(status, DEV_ERR_TIMEOUT, 700, (int)blockIdx.x, (int)nb);
        ok = 0;
        break;
      }
      __nanosleep(32);
    }
  }
  return __syncthreads_and(ok) != 0;
}

// (S, s) += (T, t) in double-float: two-sum of the leading parts, the trailing parts added to
// the error term
__device__ __forceinline__ void df_add(float& S, float& s, float T, float t) {
  const float u = __fadd_rn(S, T);
  const float bv = __fsub_rn(u, S);
  const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(u, bv)), __fsub_rn(T, bv));
  S = u;
  s = __fadd_rn(s, __fadd_rn(err, t));
}

// a * b = p + e exactly (FMA)
__device__ __forceinline__ float2 two_prod(float a, float b) {
  const float p = __fmul_rn(a, b);
  return make_float2(p, __fmaf_rn(a, b, -p));
}

// x + y in double-float, renormalised so that |lo| stays below half an ulp of hi
__device__ __forceinline__ float2 df_sum(float2 x, float2 y) {
  float S = x.x, s = x.y;
  df_add(S, s, y.x, y.y);
  const float h = __fadd_rn(S, s);
  return make_float2(h, __fsub_rn(s, __fsub_rn(h, S)));
}

// v * (c.hi + c.lo) in double-float (v FP32)
__device__ __forceinline__ float2 df_scale(float v, float2 c) {
  const float2 p = two_prod(v, c.x);
  return make_float2(p.x, __fmaf_rn(v, c.y, p.y));
}

// (a.hi + a.lo) * (b.hi + b.lo) in double-float (the lo * lo term, 2^-48 relative, dropped)
__device__ __forceinline__ float2 df_mul(float2 a, float2 b) {
  const float2 p = two_prod(a.x, b.x);
  return make_float2(p.x, __fmaf_rn(a.x, b.y, __fmaf_rn(a.y, b.x, p.y)));
}

__device__ __forceinline__ float2 warp_sum_df(float2 v) {
  for (int o = 16; o > 0; o >>= 1)
    v = df_sum(v, make_float2(__shfl_xor_sync(0xffffffffu, v.x, o), __shfl_xor_sync(0xffffffffu, v.y, o)));
  return v;
}

// out[k] = sum over blocks of P[b * ld + k], k < cnt, in double-float: one warp per k; lane l
// adds the blocks l, l + 32, ... in order, then a fixed shuffle tree, so the sum does not
// depend on timing
__device__ void gc_sum_partials(const float2* P, int ld, int cnt, float2* out) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int k = wp; k < cnt; k += GC_WARPS) {
    float2 s = make_float2(0.0f, 0.0f);
    for (int b = lane; b < (int)gridDim.x; b += 32) s = df_sum(s, P[(size_t)b * ld + k]);
    s = warp_sum_df(s);
    if (lane == 0) out[k] = s;
  }
  __syncthreads();
}

// The block's rows of the basis live in shared memory in double-float: Vs[k * RB + r], r =
// q * 32 + lane for the block's q-th row group (global row (blockIdx.x + q * grid) * 32 + lane;
// rows past n hold 0); w likewise in ws[r], the row's preconditioner (FP32) in ds[r].
struct GcRows {
  float2* Vs;
  float2* ws;
  float* ds;
  int RB;     // 32 * gpb
  int nq;     // row groups this block owns
};

// this block's partials of iteration j's dot products, double-float, into P[blockIdx.x * ld +
// k]: k <= j: v_k . w; j < k <= 2j: v_(k-j-1) . v_j (the new column of the basis' Gram
// matrix); 2j + 1: w . w; 2j + 2: v_j . v_j
__device__ void gc_partial_dots_gram(const GcRows& R, int j, int ld, float2* P, float2* sh) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int cnt = 2 * j + 3;
  for (int k = wp; k < cnt; k += GC_WARPS) {
    float2 s = make_float2(0.0f, 0.0f);
    for (int q = 0; q < R.nq; ++q) {
      const float2 w = R.ws[q * 32 + lane];
      const float2 vj = R.Vs[(size_t)j * R.RB + q * 32 + lane];
      float2 t;
      if (k <= j) {
        t = df_mul(R.Vs[(size_t)k * R.RB + q * 32 + lane], w);
      } else if (k <= 2 * j) {
        t = df_mul(R.Vs[(size_t)(k - j - 1) * R.RB + q * 32 + lane], vj);
      } else {
        const float2 x = (k == 2 * j + 1) ? w : vj;   // x . x = hi^2 + 2 hi lo
        t = two_prod(x.x, x.x);
        t.y = __fmaf_rn(2.0f * x.x, x.y, t.y);
      }
      s = df_sum(s, t);
    }
    s = warp_sum_df(s);
    if (lane == 0) sh[k] = s;
  }
  __syncthreads();
  for (int k = threadIdx.x; k < cnt; k += GC_THREADS) P[(size_t)blockIdx.x * ld + k] = sh[k];
}

// out = G x over the first n entries (G the basis' Gram matrix, row-major with stride ldg, in
// shared memory), double-float, one warp per row in a fixed order
__device__ void gc_gram_matvec(const float2* G, int ldg, int n, const float2* x, float2* out) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  for (int k = wp; k < n; k += GC_WARPS) {
    float2 s = make_float2(0.0f, 0.0f);
    for (int l = lane; l < n; l += 32) s = df_sum(s, df_mul(G[(size_t)k * ldg + l], x[l]));
    s = warp_sum_df(s);
    if (lane == 0) out[k] = s;
  }
  __syncthreads();
}

// sum_{k <= j} V_k[r] c[k] for local row group q in double-float (warps split k, fixed-order
// sum); valid in warp 0
__device__ float2 gc_vsum(const GcRows& R, int j, int q, const float2* c, float2 (*red)[32]) {
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  float2 s = make_float2(0.0f, 0.0f);
  for (int k = wp; k <= j; k += GC_WARPS) s = df_sum(s, df_mul(R.Vs[(size_t)k * R.RB + q * 32 + lane], c[k]));
  red[wp][lane] = s;
  __syncthreads();
  float2 t = make_float2(0.0f, 0.0f);
  if (wp == 0)
    for (int p = 0; p < GC_WARPS; ++p) t = df_sum(t, red[p][lane]);
  __syncthreads();
  return t;
}

// Two columns at once (f32x2): (NS, Ns) -= a * (xh + xl) in double-float, kept negated so that
// every subtraction is an FMA by -1.  np = a * (-xh) rounded is -p, e = a * xh + np is the
// product's rounding error (exact, FMA); NS + np is split exactly by Knuth's two-sum, and the
// trailing part collects err - e - a * xl (the a * xl term, 2^-24 of the product, is rounded).
__device__ __forceinline__ void df2_acc(float2 a, float2 xh, float2 nxh, float2 nxl, float2& NS, float2& Ns) {
  const float2 m1 = make_float2(-1.0f, -1.0f);
  const float2 np = __fmul2_rn(a, nxh);
  const float2 e = __ffma2_rn(a, xh, np);
  const float2 u = __fadd2_rn(NS, np);
  const float2 bv = __ffma2_rn(NS, m1, u);                     // u - NS
  const float2 t1 = __ffma2_rn(bv, m1, u);                     // u - bv
  const float2 err = __fadd2_rn(__ffma2_rn(t1, m1, NS), __ffma2_rn(bv, m1, np));
  NS = u;
  Ns = __ffma2_rn(a, nxl, __ffma2_rn(e, m1, __fadd2_rn(Ns, err)));
}

// One restart cycle of right-preconditioned GMRES(m) with CGS2, back substitution and the
// update of x, in one cooperative launch.  Blocks own groups of 32 consecutive rows
// (column-major A: a warp reads 256 contiguous bytes of the paired hi plane per column pair)
// and keep those rows of the basis in shared memory; only the split vector Dinv v_j and the
// per-block partial sums cross between blocks.  Iteration j:
//   (1) w = A Dinv v_j on the owned rows; partials of c = V^T w, of the Gram column V^T v_j,
//       of w . w and v_j . v_j                                                      -> barrier
//   (2) the Gram matrix G = V^T V gains its column j; classical Gram-Schmidt twice with the
//       second pass from G (V^T (w - V c) = c - G c): h = 2 c - G c, ||w - V h||^2 =
//       w.w - 2 h.c + h.G h; v_{j+1} = (w - V h) / ||.|| on the owned rows; H column h -> barrier
// Two grid barriers per iteration (three with a second dot-product pass); orthogonality lost
// in forming w - V h shows in the next Gram column and is projected out one iteration later.
// The basis and the Gram-Schmidt arithmetic are double-float, as is the operator product; the
// Hessenberg matrix, the Givens rotations, g and the back substitution are FP64.  Every block
// keeps H, the rotations and g in shared memory: the rotations of column j-1 run on the last
// warp during the product of step j, as a warp scan of their recurrence (FP64 latency on this
// GPU makes a sequential chain of 2 j operations slow).  All sums over blocks run in a fixed
// order, so the result does not depend on timing.
__global__ void __launch_bounds__(GC_THREADS, 1) gmres_cycle_kernel(const GcArgs a) {
  __shared__ float2 redf[GC_WARPS][32];
  __shared__ double Hs[GC_MAXM][GC_MAXM + 1];   // Hs[j][k]: rotated column j (R factor)
  __shared__ float2 h1[GC_MAXM + 2];
  __shared__ float2 sh[2 * GC_MAXM + 3];
  __shared__ float2 gx[GC_MAXM + 1];
  __shared__ float2 wws;
  __shared__ double yv[GC_MAXM];
  __shared__ double gs[GC_MAXM + 1];
  __shared__ double css[GC_MAXM], sns[GC_MAXM];
  __shared__ float nrm_inv[2];
  __shared__ int sdone;
  extern __shared__ float dyn[];
  const unsigned FULL = 0xffffffffu;
  const int lane = threadIdx.x & 31, wp = threadIdx.x >> 5;
  const int ngroups = (a.n + 31) / 32;
  const int npairs = (a.n + 1) / 2;
  const int ld = 2 * a.m + 3;
  GcRows R;
  R.RB = 32 * a.gpb;
  R.Vs = reinterpret_cast<float2*>(dyn);
  R.ws = R.Vs + (size_t)(a.m + 1) * R.RB;
  R.ds = dyn + (size_t)2 * (a.m + 2) * R.RB;
  // the basis' Gram matrix G[k][l] = v_k . v_l (k, l <= j), double-float, symmetric
  const int ldg = a.m + 1;
  float2* gram = reinterpret_cast<float2*>(dyn + (size_t)(2 * (a.m + 2) + 1) * R.RB);
  R.nq = ((int)blockIdx.x < ngroups) ? (ngroups - 1 - (int)blockIdx.x) / (int)gridDim.x + 1 : 0;
  float2* P1 = a.P;
  // the last warp applies the Givens rotations to column j-1 while the others form A Dinv v_j
  const bool gwarp = (wp == GC_WARPS - 1);
  const int per = (npairs + GC_WARPS - 2) / (GC_WARPS - 1);
  const int p0 = gwarp ? npairs : min(npairs, wp * per), p1 = gwarp ? npairs : min(npairs, p0 + per);
  auto row = [&](int q) { return ((int)blockIdx.x + q * (int)gridDim.x) * 32 + lane; };
  // Dinv v for row i (v double-float, Dinv FP32) as hi + lo, stored with negations
  auto put_split = [&](int i, float2 v, float d) {
    const float2 z = df_scale(d, v);
    const float p = z.x, e = z.y;
    float* hp = reinterpret_cast<float*>(&a.vsp[i >> 1]);
    float* lp = reinterpret_cast<float*>(&a.vsl[i >> 1]);
    hp[i & 1] = p;
    hp[2 + (i & 1)] = -p;
    lp[i & 1] = -e;
  };
  unsigned nb = 0;
  // entries the plane cannot carry: nothing is done, and the host finishes with FP64 products
  if (*a.plane_flag & 1u) {
    if (blockIdx.x == 0 && threadIdx.x == 0) a.st->kdone = 0;
    return;
  }

  if (threadIdx.x == 0) {
    gs[0] = a.st->beta;
    sdone = a.st->done;
  }
  for (int k = 1 + threadIdx.x; k <= GC_MAXM; k += GC_THREADS) gs[k] = 0.0;
  // an odd order pads the last column pair with a zero column
  if (blockIdx.x == 0 && threadIdx.x == 0 && (a.n & 1)) {
    a.vsp[a.n >> 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    a.vsl[a.n >> 1] = make_float2(0.0f, 0.0f);
  }
  // v_0 and Dinv on the owned rows into shared memory (FP32); Dinv v_0 split for the product
  if (wp == 0)
    for (int q = 0; q < R.nq; ++q) {
      const int i = row(q);
      const double vd = (i < a.n) ? a.V0[i] : 0.0;
      const float vh = (float)vd;
      const float2 v = make_float2(vh, (float)(vd - (double)vh));
      const float d = (i < a.n) ? (float)a.dinv[i] : 0.0f;
      R.Vs[q * 32 + lane] = v;
      R.ds[q * 32 + lane] = d;
      if (i < a.n) put_split(i, v, d);
    }
  if (!gc_barrier(a.bar, a.status, nb++)) return;

  int kd = 0;
  for (int j = 0;; ++j) {
    if (gwarp && j > 0) {
      // column j-1 of H (assembled in step 3): the K = j-1 earlier rotations as the affine
      // recurrence x_{k+1} = -s_k x_k + c_k h_{k+1} (x_0 = h_0, x_k the value entering
      // rotation k), scanned over the warp (two rotations per lane); then the new rotation, g
      // and the convergence test
      const int K = j - 1;
      double* hc = Hs[K];
      const int k0 = 2 * lane, k1 = k0 + 1;
      double c0 = 1.0, s0 = 0.0, c1 = 1.0, s1 = 0.0, h0p = 0.0, h1p = 0.0;
      if (k0 < K) { c0 = css[k0]; s0 = sns[k0]; h0p = hc[k0 + 1]; }
      if (k1 < K) { c1 = css[k1]; s1 = sns[k1]; h1p = hc[k1 + 1]; }
      const double a0 = -s0, b0 = c0 * h0p, a1 = -s1, b1 = c1 * h1p;
      const double x0 = hc[0], xn = hc[K + 1];
      double Ac = a1 * a0, Bc = fma(a1, b0, b1);         // f_{k1} o f_{k0}
      for (int o = 1; o < 32; o <<= 1) {
        const double Ap = __shfl_up_sync(FULL, Ac, o), Bp = __shfl_up_sync(FULL, Bc, o);
        if (lane >= o) {
          Bc = fma(Ac, Bp, Bc);
          Ac = Ac * Ap;
        }
      }
      double Ae = __shfl_up_sync(FULL, Ac, 1), Be = __shfl_up_sync(FULL, Bc, 1);
      if (lane == 0) { Ae = 1.0; Be = 0.0; }
      const double xk0 = fma(Ae, x0, Be);                // x_{k0}
      const double xk1 = fma(a0, xk0, b0);               // x_{k1}
      const double xk2 = fma(a1, xk1, b1);               // x_{k1 + 1}
      __syncwarp();
      if (k0 < K) hc[k0] = fma(c0, xk0, s0 * h0p);
      if (k1 < K) hc[k1] = fma(c1, xk1, s1 * h1p);
      // x_K sits with element K-1: lane (K-1)/2, as xk1 (K-1 even) or xk2 (K-1 odd)
      const double cand = ((K - 1) & 1) ? xk2 : xk1;
      double xK = __shfl_sync(FULL, cand, K > 0 ? ((K - 1) >> 1) : 0);
      if (K == 0) xK = x0;
      if (lane == 0) {
        const double r = hypot(xK, xn);
        const double c = (r == 0.0) ? 1.0 : xK / r, sg = (r == 0.0) ? 0.0 : xn / r;
        css[K] = c;
        sns[K] = sg;
        hc[K] = r;
        hc[K + 1] = 0.0;
        gs[K + 1] = -sg * gs[K];
        gs[K] = c * gs[K];
        sdone = (fabs(gs[K + 1]) <= a.st->tolcyc || xn == 0.0) ? 1 : 0;
      }
    }
    const bool more = j < a.mc;
    // (1) w = A Dinv v_j on the owned rows, double-float; column pairs split over the warps,
    //     two independent f32x2 chains per lane, combined in double-float, rounded once
    for (int q = 0; q < R.nq && more; ++q) {
      const int i = row(q);
      const int ic = min(i, a.n - 1);            // rows past n compute a dummy sum, never stored
      float2 NS0 = make_float2(0.f, 0.f), Ns0 = NS0, NS1 = NS0, Ns1 = NS0;
      const float2* col = a.AH + (size_t)p0 * a.n + ic;
      int cp = p0;
#pragma unroll 4
      for (; cp + 1 < p1; cp += 2, col += 2 * (size_t)a.n) {
        const float2 A0 = __ldg(col), A1 = __ldg(col + a.n);
        const float4 H0 = a.vsp[cp], H1 = a.vsp[cp + 1];
        const float2 L0 = a.vsl[cp], L1 = a.vsl[cp + 1];
        df2_acc(A0, make_float2(H0.x, H0.y), make_float2(H0.z, H0.w), L0, NS0, Ns0);
        df2_acc(A1, make_float2(H1.x, H1.y), make_float2(H1.z, H1.w), L1, NS1, Ns1);
      }
      if (cp < p1) {
        const float4 H0 = a.vsp[cp];
        df2_acc(__ldg(col), make_float2(H0.x, H0.y), make_float2(H0.z, H0.w), a.vsl[cp], NS0, Ns0);
      }
      float S = NS0.x, s = Ns0.x;
      df_add(S, s, NS0.y, Ns0.y);
      df_add(S, s, NS1.x, Ns1.x);
      df_add(S, s, NS1.y, Ns1.y);
      redf[wp][lane] = make_float2(S, s);
      __syncthreads();
      if (wp == 0) {
        float2 t = redf[0][lane];
        for (int p = 1; p < GC_WARPS - 1; ++p) df_add(t.x, t.y, redf[p][lane].x, redf[p][lane].y);
        const float h = -__fadd_rn(t.x, t.y);   // -(S + s), renormalised
        R.ws[q * 32 + lane] = (i < a.n) ? make_float2(h, __fsub_rn(-t.y, __fadd_rn(h, t.x))) : make_float2(0.f, 0.f);
      }
      __syncthreads();
    }
    __syncthreads();
    if (sdone || !more) {   // converged at column j-1 (the last product is discarded), or m steps
      kd = j;
      break;
    }
    // (2) one pass of dot products: c = V^T w, the Gram column of v_j, w . w, v_j . v_j
    gc_partial_dots_gram(R, j, ld, P1, sh);
    if (!gc_barrier(a.bar, a.status, nb++)) return;
    gc_sum_partials(P1, ld, 2 * j + 3, sh);
    for (int k = threadIdx.x; k <= j; k += GC_THREADS) {
      const float2 g = (k < j) ? sh[j + 1 + k] : sh[2 * j + 2];
      gram[(size_t)k * ldg + j] = g;
      gram[(size_t)j * ldg + k] = g;
      h1[k] = sh[k];
    }
    if (threadIdx.x == 0) wws = sh[2 * j + 1];
    __syncthreads();
    // (3) classical Gram-Schmidt twice, the second pass from the Gram matrix G = V^T V (which
    //     equals V^T (w - V c) in exact arithmetic): h = c + (c - G c) = 2 c - G c, and
    //     ||w - V h||^2 = w.w - 2 h.c + h.G h; then v_{j+1} = (w - V h) / ||.||
    gc_gram_matvec(gram, ldg, j + 1, h1, gx);                                  // gx = G c
    for (int k = threadIdx.x; k <= j; k += GC_THREADS)
      gx[k] = df_sum(df_scale(2.0f, h1[k]), make_float2(-gx[k].x, -gx[k].y));   // gx = h
    __syncthreads();
    gc_gram_matvec(gram, ldg, j + 1, gx, sh);                                  // sh = G h
    if (wp == 0) {
      float2 hc = make_float2(0.0f, 0.0f), hgh = make_float2(0.0f, 0.0f);
      for (int k = lane; k <= j; k += 32) {
        hc = df_sum(hc, df_mul(gx[k], h1[k]));
        hgh = df_sum(hgh, df_mul(gx[k], sh[k]));
      }
      hc = warp_sum_df(hc);
      hgh = warp_sum_df(hgh);
      if (lane == 0) {
        const float2 t = df_sum(df_sum(wws, df_scale(-2.0f, hc)), hgh);
        const float nrm2 = t.x + t.y;
        const float nr = nrm2 > 0.0f ? sqrtf(nrm2) : 0.0f;
        nrm_inv[0] = nr;
        nrm_inv[1] = nr > 0.0f ? 1.0f / nr : 0.0f;
      }
    }
    __syncthreads();
    const float inv = nrm_inv[1];
    for (int q = 0; q < R.nq; ++q) {
      const float2 t = gc_vsum(R, j, q, gx, redf);
      if (wp == 0) {
        const int i = row(q);
        const float2 w2 = df_sum(R.ws[q * 32 + lane], make_float2(-t.x, -t.y));
        const float2 v = df_scale(inv, w2);       // w2 * inv; H[j+1][j] = 1 / inv, so that
                                                  // H[j+1][j] v_{j+1} = w2 to double-float
        R.Vs[(size_t)(j + 1) * R.RB + q * 32 + lane] = v;
        if (i < a.n) put_split(i, v, R.ds[q * 32 + lane]);
      }
    }
    for (int k = threadIdx.x; k <= j; k += GC_THREADS) Hs[j][k] = (double)gx[k].x + (double)gx[k].y;
    if (threadIdx.x == 0) Hs[j][j + 1] = (inv > 0.0f) ? 1.0 / (double)inv : 0.0;
    if (!gc_barrier(a.bar, a.status, nb++)) return;
  }
  // y = R^{-1} g on one warp (every block): a column sweep from the last unknown, the
  // reciprocals of the diagonal formed in parallel first; R[k][i] = Hs[i][k]
  if (wp == 0) {
    const int ia = lane, ib = lane + 32;
    double t0 = (ia < kd) ? gs[ia] : 0.0, t1 = (ib < kd) ? gs[ib] : 0.0;
    const double d0 = (ia < kd) ? 1.0 / Hs[ia][ia] : 0.0, d1 = (ib < kd) ? 1.0 / Hs[ib][ib] : 0.0;
    for (int i = kd - 1; i >= 0; --i) {
      const double ti = __shfl_sync(FULL, i < 32 ? t0 : t1, i & 31);
      const double di = __shfl_sync(FULL, i < 32 ? d0 : d1, i & 31);
      const double yi = ti * di;
      if (lane == 0) yv[i] = yi;
      if (ia < i) t0 = fma(-Hs[i][ia], yi, t0);
      if (ib < i) t1 = fma(-Hs[i][ib], yi, t1);
    }
  }
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    a.st->kdone = kd;
    a.st->done = sdone;
  }
  __syncthreads();
  // x += Dinv V y on the owned rows, in FP64: an FP32 rounding of the correction would come
  // back in the next residual amplified by the condition number of A Dinv
  double (*redd)[32] = reinterpret_cast<double (*)[32]>(redf);
  if (kd > 0)
    for (int q = 0; q < R.nq; ++q) {
      double t = 0.0;
      for (int k = wp; k < kd; k += GC_WARPS) {
        const float2 v = R.Vs[(size_t)k * R.RB + q * 32 + lane];
        t = fma((double)v.x + (double)v.y, yv[k], t);
      }
      redd[wp][lane] = t;
      __syncthreads();
      if (wp == 0) {
        double u = 0.0;
        for (int p = 0; p < GC_WARPS; ++p) u += redd[p][lane];
        const int i = row(q);
        if (i < a.n) a.x[i] += u * (double)R.ds[q * 32 + lane];
      }
      __syncthreads();
    }
}

// Bounded-wait self-tests: waits that nothing completes, so each gives up after max_polls,
// records DEV_ERR_TIMEOUT in the status block and returns (no fault, no hang).
//   which 0: an mbarrier phase with no arrival (the wait of the TMA tile pipelines)
//   which 1: a grid barrier that waits for one block more than the grid (the fused GMRES cycle)
__global__ void selftest_mbar_kernel(int* status, unsigned max_polls) {
  __shared__ __align__(8) uint64_t bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool ok = mbar_wait_bounded(&bar, 0u, max_polls);
  if (!ok && threadIdx.x == 0) record_failure(status, DEV_ERR_TIMEOUT, 901, (int)blockIdx.x, 0);
}

__global__ void selftest_grid_barrier_kernel(unsigned* bar, int* status, unsigned max_polls) {
  (void)gc_barrier(bar, status, 0, gridDim.x + 1, max_polls);
}

}  // namespace

int selftest_bounded_wait(obs_context* ctx, int which, int max_polls) {
  if (max_polls <= 0 || (which != 0 && which != 1)) return OBS_ERR_ARG;
  cudaStream_t st = ctx->stream;
  cudaError_t e;
  if (which == 0) {
    selftest_mbar_kernel<<<1, 32, 0, st>>>(ctx->d_status, (unsigned)max_polls);
    e = cudaGetLastError();
  } else {
    int s = ctx->work.ensure(256, st);
    if (s) return s;
    unsigned* bar = ctx->work.as<unsigned>();
    if ((e = cudaMemsetAsync(bar, 0, sizeof(unsigned), st)) != cudaSuccess) return cuda_status(e);
    const int grid = std::max(1, std::min(ctx->num_sms, 64));
    unsigned polls = (unsigned)max_polls;
    void* args[] = {&bar, &ctx->d_status, &polls};
    e = cudaLaunchCooperativeKernel((const void*)selftest_grid_barrier_kernel, dim3(grid), dim3(32), args, 0, st);
  }
  ctx->launches++;
  if (e != cudaSuccess) return cuda_status(e);
  return take_device_status(ctx);
}

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
  // fused cycle: co-resident grid, partials [2][grid][m+2], split vector, planes of A, counters
  int gc_occ = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&gc_occ, gmres_cycle_kernel, GC_THREADS, 0);
  if (e != cudaSuccess) return cuda_status(e);
  int coop = 0;
  cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device);
  // one block per SM (1024 threads at 64 registers fill an SM's register file); each block's
  // rows of the basis (m+1 vectors) and of w sit in dynamic shared memory
  const int ngroups = (n + 31) / 32;
  const int gc_grid = std::min(ngroups, std::max(1, gc_occ) * ctx->num_sms);
  const int gc_gpb = (ngroups + gc_grid - 1) / gc_grid;
  const size_t gc_smem = (size_t)(2 * (m + 2) + 1) * 32 * gc_gpb * sizeof(float) +
                         (size_t)(m + 1) * (m + 1) * sizeof(float2);
  bool fused = coop && gc_occ > 0 && m <= GC_MAXM && ctx->kernel_variant != OBS_VARIANT_GENERIC;
  if (fused) {
    cudaFuncAttributes fa{};
    int smem_optin = 0;
    cudaDeviceGetAttribute(&smem_optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, ctx->device);
    if ((e = cudaFuncGetAttributes(&fa, gmres_cycle_kernel)) != cudaSuccess) return cuda_status(e);
    fused = fa.sharedSizeBytes + gc_smem <= (size_t)smem_optin;
    if (fused) {
      e = cudaFuncSetAttribute(gmres_cycle_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)gc_smem);
      if (e != cudaSuccess) return cuda_status(e);
      int occ2 = 0;
      e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ2, gmres_cycle_kernel, GC_THREADS, gc_smem);
      if (e != cudaSuccess) return cuda_status(e);
      fused = occ2 * ctx->num_sms >= gc_grid;
    }
  }
  const size_t NP2 = (N + 1) / 2;                  // column pairs
  const size_t o_bp = o_n + 256;                   // block partials of the fused norms
  const size_t o_gp = o_bp + al((size_t)((n + GM_THREADS - 1) / GM_THREADS) * 8);
  const size_t o_gv = o_gp + al((size_t)2 * gc_grid * (m + 2) * 8);
  const size_t o_gl = o_gv + al(NP2 * 16);
  const size_t o_gb = o_gl + al(NP2 * 8);
  const size_t o_ap = o_gb + 256;
  const size_t total = fused ? o_ap + al(NP2 * N * 8) : o_gb + 256;
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
  float2* gpart = ctx->work.as<float2>(o_gp);
  float4* gvp = ctx->work.as<float4>(o_gv);
  float2* gvl = ctx->work.as<float2>(o_gl);
  double* bpart = ctx->work.as<double>(o_bp);
  // [0] barrier arrivals, [1] plane range flag, [2] x != 0, [3] arrivals of the fused norms
  unsigned* gbar = ctx->work.as<unsigned>(o_gb);
  float2* AH = fused ? ctx->work.as<float2>(o_ap) : nullptr;
  cudaStream_t strm = ctx->stream;
  const int gb = (n + GM_THREADS - 1) / GM_THREADS;
  const dim3 ggrid(gb, nchunk);
  auto launched = [&](int k) { ctx->launches += k; };

  // nrm[0]: the current residual norm; nrm[1]: ||b||
  if ((e = cudaMemsetAsync(gbar, 0, 4 * sizeof(unsigned), strm)) != cudaSuccess) return cuda_status(e);
  prep_kernel<<<gb, GM_THREADS, 0, strm>>>(A, b, x, n, dinv, bpart, gbar + 3, nrm + 1, gbar + 2);
  launched(1);
  if (fused) {
    {
      const int bx = std::max(1, std::min((n + 255) / 256, 16));
      const int by = std::max(1, std::min((n + 1) / 2, (8 * ctx->num_sms + bx - 1) / bx));
      split_hi_kernel<<<dim3(bx, by), 256, 0, strm>>>(A, n, AH, reinterpret_cast<int*>(gbar + 1));
    }
    launched(1);
  }

  // r = b - A x in FP64 (the true residual) into w, its norm into nrm[0]; with nz, a zero x
  // (known on the device only) gives r = b and ||b|| without the product
  auto residual = [&](const unsigned* nz) {
    gemv_part_kernel<<<ggrid, GM_THREADS, 0, strm>>>(A, n, x, nullptr, part, nullptr, nz);
    gemv_sum_norm_kernel<<<gb, GM_THREADS, 0, strm>>>(part, nchunk, n, b, w, nz, bpart, gbar + 3, nrm, nrm + 1);
    launched(2);
  };
  residual(gbar + 2);
  // The first cycle is launched without a host round trip: its start kernel forms the tolerance
  // from ||b|| and stops at once when the initial residual meets it, and the fused cycle returns
  // at once when the plane cannot carry A (the loop then continues with FP64 products).  After
  // each cycle one round trip reads the true residual norm, the cycle's start norm and
  // iteration count, ||b||, the plane's flag and the status block (a barrier that gave up
  // leaves its record there).
  int total_it = 0;
  double rel = 0.0;
  for (bool check = false;; check = true) {
    if (check) {
      double rn = 0.0, bnorm = 0.0, beta = 0.0;
      int kd = 0, flag = 0;
      unsigned range_bad = 0;
      e = cudaMemcpyAsync(&rn, nrm, 8, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&bnorm, nrm + 1, 8, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&beta, &st->beta, 8, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&kd, &st->kdone, 4, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&range_bad, gbar + 1, 4, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaMemcpyAsync(&flag, ctx->d_status, 4, cudaMemcpyDeviceToHost, strm);
      if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
      if (e != cudaSuccess) return cuda_status(e);
      if (flag) return take_device_status(ctx);
      const double bref = (bnorm == 0.0) ? 1.0 : bnorm;   // src/BEM.h:227-229 divides by 1 then
      rel = rn / bref;
      bool stalled = false;
      if (fused && (range_bad & 1u)) {
        fused = false;   // entries the FP32 plane cannot carry: FP64 products throughout
      } else {
        total_it += kd;
        stalled = kd <= 0;
        // a refinement cycle (FP32 plane) that did not halve the true residual: A is too
        // ill-conditioned for its FP32 entries, so finish with FP64 products throughout
        if (fused && kd > 0 && !(rn < 0.5 * beta)) fused = false;
      }
      if (!(rn > tol * bref) || total_it >= maxiter || stalled) break;   // converged (or NaN) / budget
    }
    cycle_start_scale_kernel<<<gb, GM_THREADS, 0, strm>>>(st, nrm, nrm + 1, tol, g, m, fused ? kRefineEta : 0.0,
                                                          gbar + 1, w, n, V, gbar);
    launched(1);
    const int mc = std::min(m, maxiter - total_it);
    if (fused) {
      GcArgs ga{AH, dinv, n, m, mc, gc_gpb, V, gvp, gvl, x, gpart, gbar, gbar + 1, st, ctx->d_status};
      void* args[] = {&ga};
      e = cudaLaunchCooperativeKernel((const void*)gmres_cycle_kernel, dim3(gc_grid), dim3(GC_THREADS), args, gc_smem,
                                      strm);
      if (e != cudaSuccess) return cuda_status(e);
      launched(1);
    } else {
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
    }
    residual(nullptr);
  }
  if (iters_out) *iters_out = total_it;
  if (rel_residual) *rel_residual = rel;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  return (rel <= tol) ? OBS_OK : OBS_ERR_NO_CONVERGENCE;
}

}  // namespace obs
