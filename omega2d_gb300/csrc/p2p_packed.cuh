// p2p_packed.cuh -- velocity-only particle kernels with packed FP32 (f32x2) arithmetic.
//
// Same work decomposition, TMA pipeline, bounded waits and compensated accumulation as
// p2p_kernel.cuh; what changes is the inner loop.  Each thread holds NP pairs of targets in
// 64-bit register pairs and every FP32 operation of the pair arithmetic is issued as one
// packed FADD2/FMUL2/FFMA2 for two targets.  Sources are staged pre-duplicated
// (x, x, y, y | G, G, -G, -G | z, z, -, -) so the packed operands need no broadcast moves.
// A warp owns 32*2*NP consecutive targets (consecutive in the binned order when the host
// bins targets spatially, see p2p_packed.cu).
//
// Gaussian core (src/CoreFunc.h:111-153), all radii equal (the hoisted path), per pair with
// x = d^2/s^2, exactly the reference's three branches:
//   x > 16     : G K = G * (1/d^2)                                   (fast form)
//   x < 0.001  : G K = G * (1/s^2)
//   otherwise  : G K = (1/d^2) * (G - G e),  e = 2^(d^2 * (-log2 e / s^2))
// Per tile each warp marks the 32-source blocks that have a source within 4.02 s of the
// warp's target bounding box (a conservative test); unmarked blocks only need the fast form
// and skip the exponential.  Marked blocks evaluate all three branches, so a pair gets the same
// value whichever path its warp takes.
// Rosenhead-Moore core (src/CoreFunc.h:47-59): G K = G / (d^2 + s^2).
// Vatistas n=2 (src/CoreFunc.h:238-274): G K = G / sqrt(d^4 + s^4); Winckelmans-Leonard
// (:189-229): G K = G (dd + s^2) / dd^2.  Every other core, and every core with varying radii,
// evaluates the reference forms per target (core_eval, scalar) inside the packed difference /
// accumulation arithmetic.
#pragma once

#include <type_traits>

#include "p2p_kernel.cuh"

namespace obs {

constexpr int PK_ELEM = 3;   // float4 per staged source: (x,x,y,y) (G,G,-G,-G) (z,z,|G|,|G|)
constexpr int PK_BLK = 32;   // sources per near-mask bit word / compensated block
constexpr int PK_NB = SRC_TILE / PK_BLK;

struct PackedUni {
  float us2, ucf, cfl, thr_small, thr_far;
  float2 cfl2, s22;
};

// Gaussian, uniform radii: one 32-source block; FULL evaluates all three branches
template <bool FULL, int NP>
__device__ __forceinline__ void gauss_block(const float4* __restrict__ blk, const PackedUni& q,
                                            const float2 (&ntx)[NP], const float2 (&nty)[NP],
                                            float2 (&u)[NP], float2 (&vn)[NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
    if constexpr (!FULL) {
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2 ndx = __fadd2_rn(sx2, ntx[p]);
        const float2 ndy = __fadd2_rn(sy2, nty[p]);
        float2 d2 = __fmul2_rn(ndy, ndy);
        d2 = __ffma2_rn(ndx, ndx, d2);
        const float2 ood2 = f2(rcp_a(d2.x), rcp_a(d2.y));
        const float2 r2 = __fmul2_rn(g2, ood2);
        u[p] = __ffma2_rn(r2, ndy, u[p]);
        vn[p] = __ffma2_rn(r2, ndx, vn[p]);
      }
    } else {
      const float2 ng2 = f2(B.z, B.w);
      const float gcf = B.x * q.ucf;
#pragma unroll
      for (int p = 0; p < NP; ++p) {
        const float2 ndx = __fadd2_rn(sx2, ntx[p]);
        const float2 ndy = __fadd2_rn(sy2, nty[p]);
        float2 d2 = __fmul2_rn(ndy, ndy);
        d2 = __ffma2_rn(ndx, ndx, d2);
        const float2 t = __fmul2_rn(d2, q.cfl2);
        const float2 ood2 = f2(rcp_a(d2.x), rcp_a(d2.y));
        const float2 e = f2(ex2_a(t.x), ex2_a(t.y));
        const float2 omeg = __ffma2_rn(e, ng2, g2);
        const float2 rm = __fmul2_rn(ood2, omeg);
        const float2 rf = __fmul2_rn(g2, ood2);
        float2 r2;
        r2.x = (t.x < q.thr_far) ? rf.x : ((t.x > q.thr_small) ? gcf : rm.x);
        r2.y = (t.y < q.thr_far) ? rf.y : ((t.y > q.thr_small) ? gcf : rm.y);
        u[p] = __ffma2_rn(r2, ndy, u[p]);
        vn[p] = __ffma2_rn(r2, ndx, vn[p]);
      }
    }
  }
}

// RM, uniform radii, one 32-source block
template <int NP>
__device__ __forceinline__ void rm_block(const float4* __restrict__ blk, const PackedUni& q, const float2 (&ntx)[NP],
                                         const float2 (&nty)[NP], float2 (&u)[NP], float2 (&vn)[NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 w = __ffma2_rn(ndy, ndy, q.s22);
      w = __ffma2_rn(ndx, ndx, w);
      const float2 k = f2(rcp_a(w.x), rcp_a(w.y));
      const float2 r2 = __fmul2_rn(g2, k);
      u[p] = __ffma2_rn(r2, ndy, u[p]);
      vn[p] = __ffma2_rn(r2, ndx, vn[p]);
    }
  }
}

// Vatistas n=2, uniform radii (src/CoreFunc.h:238-274): G K = G / sqrt(d^4 + s^4 (+ t^4))
template <int NP>
__device__ __forceinline__ void v2_block(const float4* __restrict__ blk, const PackedUni& q, const float2 (&ntx)[NP],
                                         const float2 (&nty)[NP], float2 (&u)[NP], float2 (&vn)[NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 d2 = __fmul2_rn(ndy, ndy);
      d2 = __ffma2_rn(ndx, ndx, d2);
      const float2 a = __ffma2_rn(d2, d2, q.s22);
      const float2 k = f2(rsqrt_a(a.x), rsqrt_a(a.y));
      const float2 r2 = __fmul2_rn(g2, k);
      u[p] = __ffma2_rn(r2, ndy, u[p]);
      vn[p] = __ffma2_rn(r2, ndx, vn[p]);
    }
  }
}

// Winckelmans-Leonard, uniform radii (src/CoreFunc.h:189-229): K = (dd + s^2) / dd^2, dd = d^2 + s^2
template <int NP>
__device__ __forceinline__ void wl_block(const float4* __restrict__ blk, const PackedUni& q, const float2 (&ntx)[NP],
                                         const float2 (&nty)[NP], float2 (&u)[NP], float2 (&vn)[NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 d2 = __fmul2_rn(ndy, ndy);
      d2 = __ffma2_rn(ndx, ndx, d2);
      const float2 dd = __fadd2_rn(d2, q.s22);
      const float2 dq = __fmul2_rn(dd, dd);
      const float2 o = f2(rcp_a(dq.x), rcp_a(dq.y));
      const float2 k = __fmul2_rn(__fadd2_rn(dd, q.s22), o);
      const float2 r2 = __fmul2_rn(g2, k);
      u[p] = __ffma2_rn(r2, ndy, u[p]);
      vn[p] = __ffma2_rn(r2, ndx, vn[p]);
    }
  }
}

// compact exponential, uniform radii, one 32-source block with some pair inside the far
// radius (blocks entirely beyond it take gauss_block<false>: both cores are exactly 1/d^2
// there): y = (d^2/s^2)^(3/2); y > 16 -> 1/d^2; y < 0.001 -> (d/s^3)(1 - y/2); else
// (1 - e^-y)/d^2, the forms of core_eval
template <int NP>
__device__ __forceinline__ void cexp_block(const float4* __restrict__ blk, const PackedUni& q,
                                           const float2 (&ntx)[NP], const float2 (&nty)[NP], float2 (&u)[NP],
                                           float2 (&vn)[NP]) {
  const float2 ucf2 = f2(q.ucf, q.ucf);
  const float2 nl2e = f2(-kLog2e, -kLog2e);
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 d2 = __fmul2_rn(ndy, ndy);
      d2 = __ffma2_rn(ndx, ndx, d2);
      const float2 x = __fmul2_rn(d2, ucf2);
      const float2 sq = f2(sqrt_a(x.x), sqrt_a(x.y));
      const float2 y = __fmul2_rn(x, sq);
      const float2 t = __fmul2_rn(y, nl2e);
      const float2 e = f2(ex2_a(t.x), ex2_a(t.y));
      const float2 ood2 = f2(rcp_a(d2.x), rcp_a(d2.y));
      float2 k = __ffma2_rn(make_float2(-ood2.x, -ood2.y), e, ood2);
      k.x = (y.x > 16.0f) ? ood2.x : k.x;
      k.y = (y.y > 16.0f) ? ood2.y : k.y;
      k.x = (y.x < 0.001f) ? sq.x * q.ucf * fmaf(-0.5f, y.x, 1.0f) : k.x;
      k.y = (y.y < 0.001f) ? sq.y * q.ucf * fmaf(-0.5f, y.y, 1.0f) : k.y;
      const float2 r2 = __fmul2_rn(g2, k);
      u[p] = __ffma2_rn(r2, ndy, u[p]);
      vn[p] = __ffma2_rn(r2, ndx, vn[p]);
    }
  }
}

// varying radii: the reference forms per target, one 32-source block
template <int CORE, bool THICK, int NP>
__device__ __forceinline__ void general_block(const float4* __restrict__ blk, const float2 (&ntx)[NP],
                                              const float2 (&nty)[NP], const float2 (&tz)[NP], float2 (&u)[NP],
                                              float2 (&vn)[NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 B = blk[PK_ELEM * jj + 1];
    const float4 C = blk[PK_ELEM * jj + 2];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(B.x, B.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 d2 = __fmul2_rn(ndy, ndy);
      d2 = __ffma2_rn(ndx, ndx, d2);
      float K0, K1, Bd;
      core_eval<CORE, THICK, false, false>(d2.x, C.x, tz[p].x, 0.0f, 0.0f, K0, Bd);
      core_eval<CORE, THICK, false, false>(d2.y, C.x, tz[p].y, 0.0f, 0.0f, K1, Bd);
      const float2 r2 = __fmul2_rn(g2, f2(K0, K1));
      u[p] = __ffma2_rn(r2, ndy, u[p]);
      vn[p] = __ffma2_rn(r2, ndx, vn[p]);
    }
  }
}

// The last split of target block tb to finish: sum the block's partials in split order (so
// the bits do not depend on which split arrived last), write the targets, then drop the
// consumed partial lines from L2 (discard.global.L2: no write-back), so the partials stay an
// L2-resident exchange instead of HBM traffic.  Compensated partials are the items' (hi, lo)
// FP32 pairs, summed with Knuth's two-sum on the FP32 pipes (FP64 once per target: this GPU
// runs a dependent chain of FP64 adds many times slower); plain partials are FP32 sums.
template <bool COMP, int TB>
__device__ __noinline__ void split_block_reduce(const P2PArgs& a, int tb, size_t pst) {
  using T = typename std::conditional<COMP, float2, float>::type;
  static_assert((TB * sizeof(T)) % 128 == 0, "a block's partial row is whole L2 lines");
  const T* part = static_cast<const T*>(a.part);
  for (int j = threadIdx.x; j < TB; j += blockDim.x) {
    const int i = tb * TB + j;
    if (i >= a.nt) break;
    double c[2];
#pragma unroll
    for (int q = 0; q < 2; ++q) {
      const T* p = part + (size_t)q * a.nsplit * pst + i;
      if constexpr (COMP) {
        float S = 0.0f, e = 0.0f;
        for (int k = 0; k < a.nsplit; ++k) {
          const float2 v = __ldcg(p + (size_t)k * pst);
          const float u = __fadd_rn(S, v.x);
          const float bv = __fsub_rn(u, S);
          const float err = __fadd_rn(__fsub_rn(S, __fsub_rn(u, bv)), __fsub_rn(v.x, bv));
          S = u;
          e = __fadd_rn(e, __fadd_rn(err, v.y));
        }
        c[q] = (double)S + (double)e;
      } else {
        float sum = 0.0f;
        for (int k = 0; k < a.nsplit; ++k) sum += __ldcg(p + (size_t)k * pst);
        c[q] = (double)sum;
      }
    }
    store_target<RES_VEL>(a, i, c);
  }
  __syncthreads();
  constexpr int LINES = (int)(TB * sizeof(T) / 128);
  const int total = 2 * a.nsplit * LINES;
  for (int l = threadIdx.x; l < total; l += blockDim.x) {
    const int seg = l / LINES, w = l - seg * LINES;
    const T* row = part + (size_t)seg * pst + (size_t)tb * TB;
    const size_t g = __cvta_generic_to_global(row) + (size_t)w * 128;
    if ((g & 127) == 0) asm volatile("discard.global.L2 [%0], 128;" ::"l"(g) : "memory");
  }
}

// NP = 2 fits 64 registers without spills: 8 CTAs (32 warps) per SM; NP = 4 keeps its 128
// registers (4 CTAs per SM).
template <int CORE, bool THICK, bool COMP, int NP>
__global__ void __launch_bounds__(P2P_THREADS, NP == 2 ? 8 : (NP == 3 ? 5 : 4))
p2p_packed_kernel(const P2PArgs a) {
  constexpr int TPT = 2 * NP;
  constexpr int TB = P2P_THREADS * TPT;
  constexpr int WT = 32 * TPT;                      // targets per warp
  constexpr uint32_t TILE_BYTES = SRC_TILE * PK_ELEM * sizeof(float4);
  __shared__ __align__(128) float4 tile[NSTAGE][SRC_TILE * PK_ELEM];
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ unsigned smask[P2P_THREADS / 32][PK_NB];
  __shared__ int s_item, s_last;

  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  const bool fused = a.blkcnt != nullptr;
  const size_t pst = fused ? (size_t)a.ntb * TB : (size_t)a.nt;   // partials' row stride
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool unif = (~a.meta[0] == a.meta[1]) && (!THICK || ~a.meta[2] == a.meta[3]);
  PackedUni q;
  q.us2 = 0.0f;
  q.ucf = 0.0f;
  if (unif) {
    q.us2 = radius_term(CORE, __uint_as_float(a.meta[1])) + (THICK ? radius_term(CORE, __uint_as_float(a.meta[3])) : 0.0f);
    q.ucf = __frcp_rn(q.us2);
  }
  q.cfl = -q.ucf * kLog2e;
  q.thr_small = -0.001f * kLog2e;                  // x < 0.001  <=>  t > thr_small
  q.thr_far = -16.0f * kLog2e;                     // x > 16     <=>  t < thr_far
  q.cfl2 = f2(q.cfl, q.cfl);
  q.s22 = f2(q.us2, q.us2);
  // near test with a 1 % margin: Gaussian far beyond d^2/s^2 = 16, compact exponential beyond
  // (d/s)^3 = 16, i.e. d^2/s^2 = 16^(2/3) = 6.3496
  const float lim = (CORE == CORE_CEXP ? 6.4131f : 16.16f) * q.us2;

  uint32_t kt = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = *static_cast<volatile int*>(&s_item);
    if (item >= a.nitems) break;
    // fused: target-block-major, so a block's splits run close together and most of its
    // partials are still in L2 when the last one reduces them; otherwise split-major
    const int tb = fused ? item / a.nsplit : item % a.ntb;
    const int sp = fused ? item - tb * a.nsplit : item / a.ntb;
    const int tile0 = sp * a.tiles_per_split;
    const int ntile = min(a.tiles_per_split, a.nst - tile0);
    if (tid == 0) {
      fence_proxy_async_smem();
      for (int s = 0; s < NSTAGE && s < ntile; ++s) {
        const int st = (kt + s) % NSTAGE;
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_g2s(&tile[st][0], a.src + (size_t)(tile0 + s) * SRC_TILE * PK_ELEM, TILE_BYTES, &bar[st]);
      }
    }
    // this warp's targets: WT consecutive ones; (pair p, half h, lane) -> (2p + h) * 32 + lane
    float2 ntx[NP], nty[NP], tz[NP], u[NP], vn[NP], hu[NP], lu[NP], hv[NP], lv[NP];
    float bx0 = 3.0e38f, bx1 = -3.0e38f, by0 = 3.0e38f, by1 = -3.0e38f;
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      float xs[2], ys[2], zs[2];
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = tb * TB + warp * WT + (2 * p + h) * 32 + lane;
        const int ic = (i < a.nt) ? i : (a.nt - 1);
        const float x = a.tx[ic], y = a.ty[ic];
        bx0 = fminf(bx0, x); bx1 = fmaxf(bx1, x);
        by0 = fminf(by0, y); by1 = fmaxf(by1, y);
        xs[h] = -x;
        ys[h] = -y;
        zs[h] = THICK ? radius_term(CORE, a.tr[ic]) : 0.0f;
      }
      ntx[p] = f2(xs[0], xs[1]);
      nty[p] = f2(ys[0], ys[1]);
      tz[p] = f2(zs[0], zs[1]);
      u[p] = vn[p] = hu[p] = lu[p] = hv[p] = lv[p] = f2(0.0f, 0.0f);
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
          record_failure(a.status, DEV_ERR_TIMEOUT, 210 + st, (int)kt, item);
          for (int s = 0; s < NSTAGE; ++s) (void)mbar_wait_bounded(&bar[(kt + s) % NSTAGE], ((kt + s) / NSTAGE) & 1u, WAIT_TRIES);
        }
        return;
      }
      const float4* tl = &tile[st][0];
      if ((CORE == CORE_GAUSS || CORE == CORE_CEXP) && unif) {
        // near-mask of this warp: bit j of word b set when source b*32+j may be within 4 s
#pragma unroll
        for (int b = 0; b < PK_NB; ++b) {
          const float4 A = tl[PK_ELEM * (b * PK_BLK + lane)];
          const float dx = fmaxf(0.0f, fmaxf(bx0 - A.x, A.x - bx1));
          const float dy = fmaxf(0.0f, fmaxf(by0 - A.z, A.z - by1));
          const unsigned m = __ballot_sync(0xffffffffu, fmaf(dx, dx, dy * dy) <= lim);
          if (lane == 0) smask[warp][b] = m;
        }
        __syncwarp();
      }
      for (int b = 0; b < PK_NB; ++b) {
        const float4* blk = tl + PK_ELEM * b * PK_BLK;
        if constexpr (CORE == CORE_GAUSS) {
          if (unif) {
            if (smask[warp][b] == 0u) gauss_block<false, NP>(blk, q, ntx, nty, u, vn);
            else gauss_block<true, NP>(blk, q, ntx, nty, u, vn);
          } else {
            general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
          }
        } else if constexpr (CORE == CORE_RM) {
          if (unif) rm_block<NP>(blk, q, ntx, nty, u, vn);
          else general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
        } else if constexpr (CORE == CORE_V2) {
          if (unif) v2_block<NP>(blk, q, ntx, nty, u, vn);
          else general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
        } else if constexpr (CORE == CORE_WL) {
          if (unif) wl_block<NP>(blk, q, ntx, nty, u, vn);
          else general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
        } else if constexpr (CORE == CORE_CEXP) {
          if (unif) {
            if (smask[warp][b] == 0u) gauss_block<false, NP>(blk, q, ntx, nty, u, vn);
            else cexp_block<NP>(blk, q, ntx, nty, u, vn);
          } else {
            general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
          }
        } else {
          general_block<CORE, THICK, NP>(blk, ntx, nty, tz, u, vn);
        }
        if constexpr (COMP) {
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            two_sum2(hu[p], lu[p], u[p]);
            two_sum2(hv[p], lv[p], vn[p]);
            u[p] = f2(0.0f, 0.0f);
            vn[p] = f2(0.0f, 0.0f);
          }
        }
      }
      __syncthreads();
      if (tid == 0 && t + NSTAGE < ntile) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_g2s(&tile[st][0], a.src + (size_t)(tile0 + t + NSTAGE) * SRC_TILE * PK_ELEM, TILE_BYTES, &bar[st]);
      }
    }
#pragma unroll
    for (int p = 0; p < NP; ++p) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int i = tb * TB + warp * WT + (2 * p + h) * 32 + lane;
        if (i >= a.nt) continue;
        if (fused && !a.direct) {
          // partials for the in-kernel reduction, no FP64 arithmetic: (hi, lo) pairs or sums
          if (COMP) {
            float2* qp = static_cast<float2*>(a.part);
            qp[((size_t)0 * a.nsplit + sp) * pst + i] = h ? make_float2(hu[p].y, lu[p].y) : make_float2(hu[p].x, lu[p].x);
            qp[((size_t)1 * a.nsplit + sp) * pst + i] =
                h ? make_float2(-hv[p].y, -lv[p].y) : make_float2(-hv[p].x, -lv[p].x);
          } else {
            float* qp = static_cast<float*>(a.part);
            qp[((size_t)0 * a.nsplit + sp) * pst + i] = h ? u[p].y : u[p].x;
            qp[((size_t)1 * a.nsplit + sp) * pst + i] = -(h ? vn[p].y : vn[p].x);
          }
          continue;
        }
        double c[2];
        if (COMP) {
          c[0] = (double)(h ? hu[p].y : hu[p].x) + (double)(h ? lu[p].y : lu[p].x);
          c[1] = -((double)(h ? hv[p].y : hv[p].x) + (double)(h ? lv[p].y : lv[p].x));
        } else {
          c[0] = (double)(h ? u[p].y : u[p].x);
          c[1] = -(double)(h ? vn[p].y : vn[p].x);
        }
        if (a.direct) {
          store_target<RES_VEL>(a, i, c);
        } else if (COMP) {
          double* qp = static_cast<double*>(a.part);
          qp[((size_t)0 * a.nsplit + sp) * pst + i] = c[0];
          qp[((size_t)1 * a.nsplit + sp) * pst + i] = c[1];
        } else {
          float* qp = static_cast<float*>(a.part);
          qp[((size_t)0 * a.nsplit + sp) * pst + i] = (float)c[0];
          qp[((size_t)1 * a.nsplit + sp) * pst + i] = (float)c[1];
        }
      }
    }
    if (fused && !a.direct) {
      // publish this split's partials, count it in; the block's last split reduces
      __threadfence();
      __syncthreads();
      if (tid == 0) s_last = atomicAdd(&a.blkcnt[tb], 1) == a.nsplit - 1;
      __syncthreads();
      if (s_last) {
        __threadfence();
        split_block_reduce<COMP, TB>(a, tb, pst);
      }
    }
    __syncthreads();
  }
}

}  // namespace obs
