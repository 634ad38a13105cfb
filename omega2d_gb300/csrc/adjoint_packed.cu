// adjoint_packed.cu -- packed-FP32 (f32x2) VJP gathers for the Gaussian core.
//
// Same sums as adjoint.cu (the reverse mode of the finalized velocity, src/Influence.h:56-416
// with src/CoreFunc.h:111-181), organised like the packed forward kernel (p2p_packed.cuh):
// each thread owns 2*NP owners in f32x2 register pairs, elements are staged pre-duplicated by
// the TMA bulk engine, a warp owns 64*NP consecutive owners, and per 32-element block a
// warp near-mask decides between
//   far form  (every pair has d^2/s^2 > 16): K = 1/d^2 and B = 2 dK/d(d^2) = -2 K^2, the exact
//             derivative of the reference's far branch; no exponential;
//   full form : the Gaussian K and B of core_eval (series for small x, reference cut-offs),
//             with B = -2 K^2 selected wherever d^2/s^2 > 16 so both forms agree there.
// Accumulators (per owner, before the 1/(2 pi) and sign factors applied at the store):
//   ADJ_SRC  (owner = source j, element = target i with cotangent lam_i, d = x_i - x_j):
//     AX = sum K lv + B q dx,  AY = sum -K lu + B q dy,  AH = sum K q2,
//     q = dx lv - dy lu, q2 = -2 q, so dL/dG_j = -AH/2 and the far form reads
//     h = K q2 (= B q / K), AX += K (lv + h dx), AY += K (-lu + h dy)      [12 f32x2 ops + rcp]
//   ADJ_SELF (owner = particle k, element = particle j, d = x_k - x_j):
//     wu = G_j lu_k - G_k lu_j, wv = G_j lv_k - G_k lv_j, q = dx wv - dy wu,
//     AX = sum K wv + B q dx,  AY = sum -K wu + B q dy,  AE = sum K (dx lv_j - dy lu_j),
//     dL/dG_k = -AE; the far form is evaluated as moments (pa_block_self_far) [17 f32x2 ops + rcp]
// Element layout (4 float4): ADJ_SRC  (x,x,y,y) (lv,lv,-lu,-lu) (-2lv,-2lv,2lu,2lu) (z,z,0,0)
//                            ADJ_SELF (-x,-x,-y,-y) (lv,lv,-lu,-lu) (G,G,lu,lu) (z,z,0,0)
#include <algorithm>
#include <cstring>

#include "adjoint.h"
#include "obs_context.h"
#include "p2p_packed.cuh"

namespace obs {

namespace {

constexpr int PA_THREADS = 128;
constexpr int PA_TILE = 128;                      // elements per stage
constexpr int PA_ELEM = 4;                        // float4 per element
constexpr int PA_BLK = 32;
constexpr int PA_NB = PA_TILE / PA_BLK;
constexpr uint32_t PA_TILE_BYTES = PA_TILE * PA_ELEM * sizeof(float4);
enum : int { PA_SRC = 0, PA_SELF = 1 };

struct PAArgs {
  const float4* elem;
  int nst;
  const float* ox;       // owners (binned copies when binned)
  const float* oy;
  const float* orad;
  const float* og;
  const float* olu;      // ADJ_SELF: owner cotangents
  const float* olv;
  const int* operm;      // caller index of owner i (null: identity)
  int no, nob, nsplit, tiles_per_split, nitems;
  int* counter;
  const unsigned* meta;  // [0..1] element radius extrema, [2..3] owner radius extrema
  int* status;
  float* gx;
  float* gy;
  float* gg;
  double* part;          // [3][nsplit][no]
  int direct;
};

__device__ __forceinline__ void fold_radius(bool active, float r, unsigned* meta) {
  unsigned rmin = active ? __float_as_uint(r) : ~0u;
  unsigned rmax = active ? __float_as_uint(r) : 0u;
  int any = active ? 1 : 0;
  for (int o = 16; o > 0; o >>= 1) {
    rmin = min(rmin, __shfl_xor_sync(0xffffffffu, rmin, o));
    rmax = max(rmax, __shfl_xor_sync(0xffffffffu, rmax, o));
    any |= __shfl_xor_sync(0xffffffffu, any, o);
  }
  if ((threadIdx.x & 31) == 0 && any) {
    atomicMax(&meta[0], ~rmin);
    atomicMax(&meta[1], rmax);
  }
}

// elements in the (optionally permuted) order; padding: zero cotangent and strength at the
// origin with radius term 1
template <int MODE>
__global__ void pa_pack_kernel(const float* __restrict__ x, const float* __restrict__ y, const float* __restrict__ r,
                               const float* __restrict__ g, const float* __restrict__ lu,
                               const float* __restrict__ lv, const int* __restrict__ perm, int n, int n_pad,
                               float4* __restrict__ out, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = (i < n && perm) ? perm[i] : i;
  if ((unsigned)j >= (unsigned)n) j = 0;          // never taken for i < n: perm is a permutation
  const float rr = (i < n && r) ? r[j] : 0.0f;
  if (i < n) {
    const float z = r ? radius_term(CORE_GAUSS, rr) : 0.0f;
    const float X = x[j], Y = y[j], U = lu[j], V = lv[j];
    float4* o = out + (size_t)PA_ELEM * i;
    if (MODE == PA_SRC) {
      o[0] = make_float4(X, X, Y, Y);
      o[1] = make_float4(V, V, -U, -U);
      o[2] = make_float4(-2.0f * V, -2.0f * V, 2.0f * U, 2.0f * U);
    } else {
      const float G = g[j];
      o[0] = make_float4(-X, -X, -Y, -Y);
      o[1] = make_float4(V, V, -U, -U);
      o[2] = make_float4(G, G, U, U);
    }
    o[3] = make_float4(z, z, 0.0f, 0.0f);
  } else if (i < n_pad) {
    float4* o = out + (size_t)PA_ELEM * i;
    o[0] = o[1] = o[2] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    o[3] = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
  }
  fold_radius(i < n && r != nullptr, rr, meta);
}

__global__ void pa_owner_meta_kernel(const float* __restrict__ r, int n, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  fold_radius(i < n, i < n ? r[i] : 0.0f, meta + 2);
}

// owner constants of one register pair
struct PAOwn {
  float2 c0, c1;     // ADJ_SRC: -x, -y; ADJ_SELF: x, y
  float2 z;          // radius term
  float2 lvk, nluk;  // ADJ_SELF: lv_k, -lu_k
  float2 p2g, ng;    // ADJ_SELF: 2 G_k, -G_k
};

struct PAAcc {
  float2 ax, ay, ah;
};

// ADJ_SELF far form as moments (one 32-element block).  With K = 1/d^2 and B = -2 K^2,
//   K wv + B q dx = -wv P + wu Q,   -K wu + B q dy = -wu P - wv Q,
// P = (dx^2 - dy^2) K^2 = a^2 - b^2 and Q = 2 dx dy K^2 = 2 a b (a = dx K, b = dy K), and
// splitting wu, wv into their owner and element parts,
//   AX = -lv_k SP + lu_k SQ + G_k T1,   AY = -lu_k SP - lv_k SQ + G_k T2,
//   SP = sum G_j P, SQ = sum G_j Q, T1 = sum (lv_j P - lu_j Q), T2 = sum (lu_j P + lv_j Q).
// The block sums carry n = -P/2 = b^2 - K/2 (a^2 + b^2 = K) and h = Q/2 = a b:
//   sp = sum G_j n, sq = sum G_j h, t1 = sum (lv_j n + lu_j h) = -T1/2, t2 = sum (-lu_j n + lv_j h) = T2/2,
// and AE = sum K (dx lv_j - dy lu_j) = sum (a lv_j - b lu_j).  The fold once per block:
//   AX = 2 lv_k sp + 2 lu_k sq - 2 G_k t1,   AY = 2 lu_k sp - 2 lv_k sq + 2 G_k t2.
// 17 f32x2 operations per pair of pairs (the direct form: 20), no K^2 formed on its own.
// FRESH: acc[].ax, ay are zero on entry (compensated sums restart per block) and carry sp, sq.
template <int NP, bool FRESH>
__device__ __forceinline__ void pa_block_self_far(const float4* __restrict__ blk, const PAOwn (&w)[NP],
                                                  PAAcc (&acc)[NP]) {
  float2 t1[NP], t2[NP], bx[NP], by[NP];
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    if constexpr (!FRESH) {
      bx[p] = acc[p].ax;
      by[p] = acc[p].ay;
      acc[p].ax = acc[p].ay = f2(0.0f, 0.0f);
    }
    t1[p] = t2[p] = f2(0.0f, 0.0f);
  }
  const float2 mhalf = f2(-0.5f, -0.5f);
#pragma unroll 2
  for (int jj = 0; jj < PA_BLK; ++jj) {
    const float4 E0 = blk[PA_ELEM * jj];
    const float4 E1 = blk[PA_ELEM * jj + 1];
    const float4 E2 = blk[PA_ELEM * jj + 2];
    const float2 ex = f2(E0.x, E0.y), ey = f2(E0.z, E0.w);
    const float2 lv = f2(E1.x, E1.y), nlu = f2(E1.z, E1.w);
    const float2 G = f2(E2.x, E2.y), lu = f2(E2.z, E2.w);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 dx = __fadd2_rn(ex, w[p].c0);
      const float2 dy = __fadd2_rn(ey, w[p].c1);
      const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
      const float2 K = f2(rcp_a(d2.x), rcp_a(d2.y));
      const float2 a = __fmul2_rn(dx, K), b = __fmul2_rn(dy, K);
      const float2 n = __ffma2_rn(b, b, __fmul2_rn(K, mhalf));
      const float2 h = __fmul2_rn(a, b);
      acc[p].ax = __ffma2_rn(G, n, acc[p].ax);    // sp
      acc[p].ay = __ffma2_rn(G, h, acc[p].ay);    // sq
      t1[p] = __ffma2_rn(lv, n, __ffma2_rn(lu, h, t1[p]));
      t2[p] = __ffma2_rn(nlu, n, __ffma2_rn(lv, h, t2[p]));
      acc[p].ah = __ffma2_rn(a, lv, __ffma2_rn(b, nlu, acc[p].ah));
    }
  }
#pragma unroll
  for (int p = 0; p < NP; ++p) {
    // owner constants: lvk = lv_k, nluk = -lu_k, p2g = 2 G_k, ng = -G_k
    const float2 sp = acc[p].ax, sq = acc[p].ay;
    const float2 lv2 = __fmul2_rn(w[p].lvk, f2(2.0f, 2.0f)), lu2 = __fmul2_rn(w[p].nluk, f2(-2.0f, -2.0f));
    const float2 ng2 = __fmul2_rn(w[p].ng, f2(2.0f, 2.0f)), mlv2 = __fmul2_rn(w[p].lvk, f2(-2.0f, -2.0f));
    const float2 ax = __ffma2_rn(lv2, sp, __ffma2_rn(lu2, sq, __fmul2_rn(ng2, t1[p])));
    const float2 ay = __ffma2_rn(lu2, sp, __ffma2_rn(mlv2, sq, __fmul2_rn(w[p].p2g, t2[p])));
    if constexpr (FRESH) {
      acc[p].ax = ax;
      acc[p].ay = ay;
    } else {
      acc[p].ax = __fadd2_rn(bx[p], ax);
      acc[p].ay = __fadd2_rn(by[p], ay);
    }
  }
}

// one 32-element block; FAST: far form only; UNIF: uniform radii (us2, ucf); COMP: acc is zero
// on entry
template <int MODE, bool THICK, bool FAST, bool UNIF, int NP, bool COMP>
__device__ __forceinline__ void pa_block(const float4* __restrict__ blk, const PAOwn (&w)[NP], PAAcc (&acc)[NP],
                                         float us2, float ucf) {
  if constexpr (MODE == PA_SELF && FAST) {
    pa_block_self_far<NP, COMP>(blk, w, acc);
  } else {
#pragma unroll 2
    for (int jj = 0; jj < PA_BLK; ++jj) {
      const float4 E0 = blk[PA_ELEM * jj];
      const float4 E1 = blk[PA_ELEM * jj + 1];
      const float4 E2 = blk[PA_ELEM * jj + 2];
      const float2 ex = f2(E0.x, E0.y), ey = f2(E0.z, E0.w);
      const float2 P = f2(E1.x, E1.y), M = f2(E1.z, E1.w);     // lv, -lu
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2 dx = __fadd2_rn(ex, w[p].c0);
        const float2 dy = __fadd2_rn(ey, w[p].c1);
        float2 d2 = __fmul2_rn(dy, dy);
        d2 = __ffma2_rn(dx, dx, d2);
        float2 K, B;
        if constexpr (FAST) {
          K = f2(rcp_a(d2.x), rcp_a(d2.y));
          B = K;   // unused
        } else {
          const float z = blk[PA_ELEM * jj + 3].x;
          float k0, k1, b0, b1;
          if constexpr (MODE == PA_SRC) {
            core_eval<CORE_GAUSS, THICK, true, UNIF>(d2.x, w[p].z.x, z, us2, ucf, k0, b0);
            core_eval<CORE_GAUSS, THICK, true, UNIF>(d2.y, w[p].z.y, z, us2, ucf, k1, b1);
          } else {
            core_eval<CORE_GAUSS, true, true, UNIF>(d2.x, z, w[p].z.x, us2, ucf, k0, b0);
            core_eval<CORE_GAUSS, true, true, UNIF>(d2.y, z, w[p].z.y, us2, ucf, k1, b1);
          }
          if constexpr (UNIF) {
            b0 = (d2.x * ucf > 16.0f) ? -2.0f * k0 * k0 : b0;
            b1 = (d2.y * ucf > 16.0f) ? -2.0f * k1 * k1 : b1;
          }
          K = f2(k0, k1);
          // ADJ_SRC: scaled so that B * q2 = B q (q2 = -2 q from the element); ADJ_SELF forms q itself
          B = (MODE == PA_SRC) ? f2(-0.5f * b0, -0.5f * b1) : f2(b0, b1);
        }
        if constexpr (MODE == PA_SRC) {
          const float2 Q1 = f2(E2.x, E2.y), Q2 = f2(E2.z, E2.w);    // -2 lv, 2 lu
          const float2 q2 = __ffma2_rn(dx, Q1, __fmul2_rn(dy, Q2));
          if constexpr (FAST) {
            const float2 h = __fmul2_rn(K, q2);
            acc[p].ah = __fadd2_rn(acc[p].ah, h);
            acc[p].ax = __ffma2_rn(K, __ffma2_rn(h, dx, P), acc[p].ax);
            acc[p].ay = __ffma2_rn(K, __ffma2_rn(h, dy, M), acc[p].ay);
          } else {
            acc[p].ah = __ffma2_rn(K, q2, acc[p].ah);
            const float2 bq = __fmul2_rn(B, q2);
            acc[p].ax = __ffma2_rn(bq, dx, __ffma2_rn(K, P, acc[p].ax));
            acc[p].ay = __ffma2_rn(bq, dy, __ffma2_rn(K, M, acc[p].ay));
          }
        } else {
          // full form (the far blocks of ADJ_SELF run pa_block_self_far)
          const float2 G = f2(E2.x, E2.y);
          const float2 qe = __ffma2_rn(dx, P, __fmul2_rn(dy, M));             // dx lv_j - dy lu_j
          const float2 qo = __ffma2_rn(dx, w[p].lvk, __fmul2_rn(dy, w[p].nluk));
          const float2 q = __ffma2_rn(G, qo, __fmul2_rn(w[p].ng, qe));        // G_j qo - G_k qe
          acc[p].ah = __ffma2_rn(K, qe, acc[p].ah);
          const float2 wv = __ffma2_rn(G, w[p].lvk, __fmul2_rn(w[p].ng, P));
          const float2 nwu = __ffma2_rn(G, w[p].nluk, __fmul2_rn(w[p].ng, M));
          const float2 bq = __fmul2_rn(B, q);
          acc[p].ax = __ffma2_rn(bq, dx, __ffma2_rn(K, wv, acc[p].ax));
          acc[p].ay = __ffma2_rn(bq, dy, __ffma2_rn(K, nwu, acc[p].ay));
        }
      }
    }
  }
}

template <int MODE>
__device__ __forceinline__ void pa_store(const PAArgs& a, int i, double ax, double ay, double ah) {
  double sx = ax * kInv2Pi, sy = ay * kInv2Pi;
  const double sg = (MODE == PA_SRC ? -0.5 * ah : -ah) * kInv2Pi;
  if (MODE == PA_SRC) {
    const double gj = (double)a.og[i];
    sx *= -gj;
    sy *= -gj;
  }
  const int o = a.operm ? a.operm[i] : i;
  if ((unsigned)o >= (unsigned)a.no) return;      // never taken: operm is a permutation
  if (a.gx) a.gx[o] = (float)((double)a.gx[o] + sx);
  if (a.gy) a.gy[o] = (float)((double)a.gy[o] + sy);
  if (a.gg) a.gg[o] = (float)((double)a.gg[o] + sg);
}

// With one owner pair per thread the compensated self gather keeps 7 CTAs per SM (72
// registers): at 8 (64 registers) its far form spills.
template <int MODE, bool THICK, bool COMP, int NP>
__global__ void __launch_bounds__(PA_THREADS, NP == 1 ? (MODE == PA_SELF && COMP ? 7 : 8) : 4)
    pa_kernel(const PAArgs a) {
  constexpr int TPT = 2 * NP;
  constexpr int TB = PA_THREADS * TPT;
  constexpr int WT = 32 * TPT;
  __shared__ __align__(128) float4 tile[NSTAGE][PA_TILE * PA_ELEM];
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ unsigned smask[PA_THREADS / 32][PA_NB];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool thick_pair = (MODE == PA_SELF) || THICK;
  const bool owners_unif = (~a.meta[2] == a.meta[3]);
  const bool unif = thick_pair ? (owners_unif && ~a.meta[0] == a.meta[1]) : owners_unif;
  float us2 = 0.0f, ucf = 0.0f;
  if (unif) {
    us2 = radius_term(CORE_GAUSS, __uint_as_float(a.meta[3])) +
          (thick_pair ? radius_term(CORE_GAUSS, __uint_as_float(a.meta[1])) : 0.0f);
    ucf = __frcp_rn(us2);
  }
  const float lim = 16.16f * us2;                 // near test with a 1 % margin (d < 4.02 s)
  const float esign = (MODE == PA_SRC) ? 1.0f : -1.0f;   // element coordinates as staged

  uint32_t kt = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = *static_cast<volatile int*>(&s_item);
    if (item >= a.nitems) break;
    const int ob = item % a.nob;
    const int sp = item / a.nob;
    const int tile0 = sp * a.tiles_per_split;
    const int ntile = min(a.tiles_per_split, a.nst - tile0);
    if (tid == 0) {
      fence_proxy_async_smem();
      for (int s = 0; s < NSTAGE && s < ntile; ++s) {
        const int st = (kt + s) % NSTAGE;
        mbar_arrive_expect_tx(&bar[st], PA_TILE_BYTES);
        bulk_g2s(&tile[st][0], a.elem + (size_t)(tile0 + s) * PA_TILE * PA_ELEM, PA_TILE_BYTES, &bar[st]);
      }
    }
    PAOwn w[NP];
    PAAcc acc[NP], hi[NP], lo[NP];
    float bx0 = 3.0e38f, bx1 = -3.0e38f, by0 = 3.0e38f, by1 = -3.0e38f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float v[8][2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = ob * TB + warp * WT + (2 * p + h) * 32 + lane;
        const int ic = (i < a.no) ? i : (a.no - 1);
        const float x = a.ox[ic], y = a.oy[ic];
        bx0 = fminf(bx0, x); bx1 = fmaxf(bx1, x);
        by0 = fminf(by0, y); by1 = fmaxf(by1, y);
        const float G = (MODE == PA_SELF) ? a.og[ic] : 0.0f;
        v[0][h] = (MODE == PA_SRC) ? -x : x;
        v[1][h] = (MODE == PA_SRC) ? -y : y;
        v[2][h] = a.orad ? radius_term(CORE_GAUSS, a.orad[ic]) : 0.0f;
        v[3][h] = (MODE == PA_SELF) ? a.olv[ic] : 0.0f;
        v[4][h] = (MODE == PA_SELF) ? -a.olu[ic] : 0.0f;
        v[5][h] = 2.0f * G;
        v[6][h] = -G;
      }
      w[p].c0 = f2(v[0][0], v[0][1]);
      w[p].c1 = f2(v[1][0], v[1][1]);
      w[p].z = f2(v[2][0], v[2][1]);
      w[p].lvk = f2(v[3][0], v[3][1]);
      w[p].nluk = f2(v[4][0], v[4][1]);
      w[p].p2g = f2(v[5][0], v[5][1]);
      w[p].ng = f2(v[6][0], v[6][1]);
      acc[p].ax = acc[p].ay = acc[p].ah = f2(0.0f, 0.0f);
      hi[p] = acc[p];
      lo[p] = acc[p];
    }
    for (int o = 16; o > 0; o >>= 1) {
      bx0 = fminf(bx0, __shfl_xor_sync(0xffffffffu, bx0, o));
      bx1 = fmaxf(bx1, __shfl_xor_sync(0xffffffffu, bx1, o));
      by0 = fminf(by0, __shfl_xor_sync(0xffffffffu, by0, o));
      by1 = fmaxf(by1, __shfl_xor_sync(0xffffffffu, by1, o));
    }
    for (int t = 0; t < ntile; ++t, ++kt) {
      const int st = kt % NSTAGE;
      const bool ok = mbar_wait_bounded(&bar[st], (kt / NSTAGE) & 1u, WAIT_TRIES);
      if (__syncthreads_or(!ok)) {
        if (tid == 0) {
          record_failure(a.status, DEV_ERR_TIMEOUT, 520 + st, (int)kt, item);
          for (int s = 0; s < NSTAGE; ++s) (void)mbar_wait_bounded(&bar[(kt + s) % NSTAGE], ((kt + s) / NSTAGE) & 1u, WAIT_TRIES);
        }
        return;
      }
      const float4* tl = &tile[st][0];
      if (unif) {
#pragma unroll
        for (int b = 0; b < PA_NB; ++b) {
          const float4 E0 = tl[PA_ELEM * (b * PA_BLK + lane)];
          const float ex = esign * E0.x, ey = esign * E0.z;
          const float dx = fmaxf(0.0f, fmaxf(bx0 - ex, ex - bx1));
          const float dy = fmaxf(0.0f, fmaxf(by0 - ey, ey - by1));
          const unsigned m = __ballot_sync(0xffffffffu, fmaf(dx, dx, dy * dy) <= lim);
          if (lane == 0) smask[warp][b] = m;
        }
        __syncwarp();
      }
      for (int b = 0; b < PA_NB; ++b) {
        const float4* blk = tl + PA_ELEM * b * PA_BLK;
        if (unif) {
          if (smask[warp][b] == 0u) pa_block<MODE, THICK, true, true, NP, COMP>(blk, w, acc, us2, ucf);
          else pa_block<MODE, THICK, false, true, NP, COMP>(blk, w, acc, us2, ucf);
        } else {
          pa_block<MODE, THICK, false, false, NP, COMP>(blk, w, acc, us2, ucf);
        }
        if constexpr (COMP) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            two_sum2(hi[p].ax, lo[p].ax, acc[p].ax);
            two_sum2(hi[p].ay, lo[p].ay, acc[p].ay);
            two_sum2(hi[p].ah, lo[p].ah, acc[p].ah);
            acc[p].ax = acc[p].ay = acc[p].ah = f2(0.0f, 0.0f);
          }
        }
      }
      __syncthreads();
      if (tid == 0 && t + NSTAGE < ntile) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[st], PA_TILE_BYTES);
        bulk_g2s(&tile[st][0], a.elem + (size_t)(tile0 + t + NSTAGE) * PA_TILE * PA_ELEM, PA_TILE_BYTES, &bar[st]);
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = ob * TB + warp * WT + (2 * p + h) * 32 + lane;
        if (i >= a.no) continue;
        double c[3];
        if (COMP) {
          c[0] = (double)(h ? hi[p].ax.y : hi[p].ax.x) + (double)(h ? lo[p].ax.y : lo[p].ax.x);
          c[1] = (double)(h ? hi[p].ay.y : hi[p].ay.x) + (double)(h ? lo[p].ay.y : lo[p].ay.x);
          c[2] = (double)(h ? hi[p].ah.y : hi[p].ah.x) + (double)(h ? lo[p].ah.y : lo[p].ah.x);
        } else {
          c[0] = (double)(h ? acc[p].ax.y : acc[p].ax.x);
          c[1] = (double)(h ? acc[p].ay.y : acc[p].ay.x);
          c[2] = (double)(h ? acc[p].ah.y : acc[p].ah.x);
        }
        if (a.direct) {
          pa_store<MODE>(a, i, c[0], c[1], c[2]);
        } else {
#pragma unroll
          for (int q = 0; q < 3; ++q) a.part[((size_t)q * a.nsplit + sp) * a.no + i] = c[q];
        }
      }
    }
    __syncthreads();
  }
}

template <int MODE>
__global__ void pa_reduce_kernel(const PAArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.no) return;
  double c[3];
#pragma unroll
  for (int q = 0; q < 3; ++q) {
    double s = 0.0;
#pragma unroll 8
    for (int k = 0; k < a.nsplit; ++k) s += a.part[((size_t)q * a.nsplit + k) * a.no + i];
    c[q] = s;
  }
  pa_store<MODE>(a, i, c[0], c[1], c[2]);
}

// f32x2 owner pairs per thread: 2 for both gathers (about 110-127 registers, 4 CTAs per SM).
// The self gather with its moments far form: 615 ms on the 1M Gaussian patch with 2 pairs
// against 647 ms with 1 pair (72 registers, 7 CTAs per SM) and 662 ms (64 registers, 8 CTAs).
#ifndef OBS_PA_SRC_NP
#define OBS_PA_SRC_NP 2
#endif
#ifndef OBS_PA_SELF_NP
#define OBS_PA_SELF_NP 2
#endif
constexpr int pa_np(int mode) { return mode == PA_SRC ? OBS_PA_SRC_NP : OBS_PA_SELF_NP; }

cudaError_t pa_dispatch(int mode, bool thick, bool comp, const PAArgs* a, int grid, cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, PA_THREADS, 0);
    kern<<<grid, PA_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
  constexpr int NS = pa_np(PA_SRC), NF = pa_np(PA_SELF);
  if (mode == PA_SELF)
    return comp ? run(pa_kernel<PA_SELF, true, true, NF>) : run(pa_kernel<PA_SELF, true, false, NF>);
  if (thick) return comp ? run(pa_kernel<PA_SRC, true, true, NS>) : run(pa_kernel<PA_SRC, true, false, NS>);
  return comp ? run(pa_kernel<PA_SRC, false, true, NS>) : run(pa_kernel<PA_SRC, false, false, NS>);
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

bool adjoint_packed_supported(int core) { return core == CORE_GAUSS; }

int run_adjoint_packed(obs_context* ctx, int accum, int mode, int no, const float* ox, const float* oy,
                       const float* orad, const float* og, int ne, const float* ex, const float* ey, const float* er,
                       const float* eg, const float* elu, const float* elv, float* gx, float* gy, float* gg,
                       size_t off) {
  if (no == 0 || ne == 0) return OBS_OK;
  const bool comp = accum == OBS_COMPENSATED;
  const bool thick = (mode == PA_SELF) || er != nullptr;
  cudaStream_t st = ctx->stream;
  int occ = 0;
  cudaError_t e = pa_dispatch(mode, thick, comp, nullptr, 0, st, &occ);
  if (e != cudaSuccess) return cuda_status(e);
  occ = std::max(occ, 1);
  const int slots = occ * ctx->num_sms;
  const int tb = PA_THREADS * 2 * (mode == PA_SRC ? pa_np(PA_SRC) : pa_np(PA_SELF));
  const int nob = (no + tb - 1) / tb;
  const int nst = (ne + PA_TILE - 1) / PA_TILE;
  int nsplit = std::max(1, (4 * slots + nob - 1) / nob);
  nsplit = std::min(nsplit, std::max(1, nst / 4));
  const int tps = (nst + nsplit - 1) / nsplit;
  nsplit = (nst + tps - 1) / tps;

  // processing order: the owners are the gather's targets, the elements its sources
  const int order = ctx->target_order;
  const bool big = (double)no * ne >= 2e9 && no >= 4096 && ne >= 4096;
  const bool bin_o = order == OBS_ORDER_BINNED || order == OBS_ORDER_BINNED_TARGETS || (order == OBS_ORDER_AUTO && big);
  const bool bin_e = order == OBS_ORDER_BINNED || (order == OBS_ORDER_AUTO && big);
  const bool same = mode == PA_SELF;                 // owners and elements are one set

  const size_t hdr = 256;
  const size_t ebytes = (size_t)nst * PA_TILE * PA_ELEM * sizeof(float4);
  const size_t pbytes = nsplit > 1 ? al256((size_t)3 * nsplit * no * sizeof(double)) : 0;
  const size_t ovec = al256((size_t)no * sizeof(float));
  const size_t obytes = bin_o ? (same ? 7 : 5) * ovec : 0;         // perm, x, y, r, g (, lu, lv)
  const size_t evec = (bin_e && !(same && bin_o)) ? al256((size_t)ne * sizeof(int)) : 0;
  const size_t sbytes = (bin_o || bin_e) ? bin_scratch_bytes(std::max(bin_o ? no : 0, bin_e ? ne : 0)) : 0;
  int s = ctx->work.ensure(off + hdr + ebytes + pbytes + obytes + evec + sbytes, st);
  if (s) return s;
  WorkHeader* h = ctx->work.as<WorkHeader>(off);
  float4* elem = ctx->work.as<float4>(off + hdr);
  size_t q = off + hdr + ebytes + pbytes;
  int* operm = nullptr;
  float *bx = nullptr, *by = nullptr, *br = nullptr, *bg = nullptr, *blu = nullptr, *blv = nullptr;
  if (bin_o) {
    operm = ctx->work.as<int>(q);
    bx = ctx->work.as<float>(q + ovec);
    by = ctx->work.as<float>(q + 2 * ovec);
    br = ctx->work.as<float>(q + 3 * ovec);
    bg = ctx->work.as<float>(q + 4 * ovec);
    if (same) {
      blu = ctx->work.as<float>(q + 5 * ovec);
      blv = ctx->work.as<float>(q + 6 * ovec);
    }
    q += obytes;
  }
  int* eperm = nullptr;
  if (bin_e) {
    eperm = (same && bin_o) ? operm : ctx->work.as<int>(q);
    q += evec;
  }
  void* scratch = sbytes ? ctx->work.as<char>(q) : nullptr;

  e = cudaMemsetAsync(h, 0, sizeof(WorkHeader), st);
  if (e != cudaSuccess) return cuda_status(e);
  int nl = 0;
  if (bin_o) {
    e = bin_order(ox, oy, no, scratch, operm, st, &nl);
    if (e == cudaSuccess) e = bin_gather(operm, ox, oy, orad, og, no, bx, by, orad ? br : nullptr, og ? bg : nullptr, st, &nl);
    if (e == cudaSuccess && same) e = bin_gather(operm, elu, elv, nullptr, nullptr, no, blu, blv, nullptr, nullptr, st, &nl);
  }
  if (e == cudaSuccess && bin_e && !(same && bin_o)) e = bin_order(ex, ey, ne, scratch, eperm, st, &nl);
  ctx->launches += nl;
  if (e != cudaSuccess) return cuda_status(e);

  const int n_pad = nst * PA_TILE;
  if (mode == PA_SRC)
    pa_pack_kernel<PA_SRC><<<(n_pad + 255) / 256, 256, 0, st>>>(ex, ey, er, eg, elu, elv, eperm, ne, n_pad, elem, h->meta);
  else
    pa_pack_kernel<PA_SELF><<<(n_pad + 255) / 256, 256, 0, st>>>(ex, ey, er, eg, elu, elv, eperm, ne, n_pad, elem, h->meta);
  ctx->launches++;
  if (orad) {
    pa_owner_meta_kernel<<<(no + 255) / 256, 256, 0, st>>>(orad, no, h->meta);
    ctx->launches++;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);

  PAArgs a;
  std::memset(&a, 0, sizeof(a));
  a.elem = elem;
  a.nst = nst;
  a.ox = bin_o ? bx : ox;
  a.oy = bin_o ? by : oy;
  a.orad = orad ? (bin_o ? br : orad) : nullptr;
  a.og = og ? (bin_o ? bg : og) : nullptr;
  a.olu = same ? (bin_o ? blu : elu) : nullptr;
  a.olv = same ? (bin_o ? blv : elv) : nullptr;
  a.operm = operm;
  a.no = no;
  a.nob = nob;
  a.nsplit = nsplit;
  a.tiles_per_split = tps;
  a.nitems = nob * nsplit;
  a.counter = &h->counter;
  a.meta = h->meta;
  a.status = ctx->d_status;
  a.gx = gx;
  a.gy = gy;
  a.gg = gg;
  a.part = pbytes ? ctx->work.as<double>(off + hdr + ebytes) : nullptr;
  a.direct = nsplit == 1;
  timing_main_begin(ctx);
  e = pa_dispatch(mode, thick, comp, &a, std::min(a.nitems, slots), st, nullptr);
  ctx->launches++;
  timing_main_end(ctx);
  if (e == cudaSuccess && nsplit > 1) {
    if (mode == PA_SELF) pa_reduce_kernel<PA_SELF><<<(no + 255) / 256, 256, 0, st>>>(a);
    else pa_reduce_kernel<PA_SRC><<<(no + 255) / 256, 256, 0, st>>>(a);
    ctx->launches++;
    e = cudaGetLastError();
  }
  return cuda_status(e);
}

}  // namespace obs
