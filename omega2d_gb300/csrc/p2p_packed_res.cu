// p2p_packed_res.cu -- packed-FP32 (f32x2) Gaussian kernels for the velocity-gradient,
// vorticity and shear-rate results (kernelug / kerneluw / kernelue, src/Kernels.h:112-231, with
// the Gaussian core of src/CoreFunc.h:111-181).
//
// Same organisation as the packed velocity kernel (p2p_packed.cuh): warp-contiguous targets in
// f32x2 register pairs, TMA-staged duplicated sources, per-tile warp near-masks over 32-source
// blocks.  Here a block is "far" when every pair has d^2/s^2 > 25: there the reference's
// gradient factor bbb = -2 K/d^2 + 2 s^-2 d^-2 e^{-x} equals -2 K^2 to 4e-10 relative, so the far
// form needs no exponential, and the vorticity term G (bbb d^2 + 2 K) vanishes.  Near blocks
// evaluate core_eval (series, cut-offs) per pair.
// Accumulators per target (h = -G bbb / 2):
//   U = sum G K (-dy)... (as the velocity kernel: U = sum r ndy, VN = sum r ndx, r = G K)
//   GRAD : R = sum r, PH = sum h dx dy, QH = sum h dx^2, E = sum G (bbb d^2 + 2 K) (near only);
//          S1 = -2 PH, S2 = -2 QH + R, S3 = -2 QH + R - E   (the generic kernel's S1..S3)
//   VORT : W = sum G (bbb d^2 + 2 K)                         (near only)
//   SHEAR: S = sum |G| |bbb| d^2 / 2                          (far: |G| K)
#include "obs_context.h"
#include "p2p_packed.cuh"

namespace obs {

namespace {

template <int RES> struct PRes;
template <> struct PRes<RES_GRAD> { static constexpr int NC = 6, NP = 1; };
template <> struct PRes<RES_VORT> { static constexpr int NC = 3, NP = 2; };
template <> struct PRes<RES_SHEAR> { static constexpr int NC = 3, NP = 2; };

// one 32-source block; FAR: every pair has d^2/s^2 > 25 (uniform radii)
template <int RES, bool FAR, bool THICK, bool UNIF, int NP, int NC>
__device__ __forceinline__ void res_block(const float4* __restrict__ blk, float us2, float ucf,
                                          const float2 (&ntx)[NP], const float2 (&nty)[NP],
                                          const float2 (&tz)[NP], float2 (&acc)[NC][NP]) {
#pragma unroll 2
  for (int jj = 0; jj < PK_BLK; ++jj) {
    const float4 A = blk[PK_ELEM * jj];
    const float4 Bs = blk[PK_ELEM * jj + 1];
    const float4 C = blk[PK_ELEM * jj + 2];
    const float2 sx2 = f2(A.x, A.y), sy2 = f2(A.z, A.w);
    const float2 g2 = f2(Bs.x, Bs.y);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      const float2 ndx = __fadd2_rn(sx2, ntx[p]);
      const float2 ndy = __fadd2_rn(sy2, nty[p]);
      float2 d2 = __fmul2_rn(ndy, ndy);
      d2 = __ffma2_rn(ndx, ndx, d2);
      if constexpr (FAR) {
        const float2 K = f2(rcp_a(d2.x), rcp_a(d2.y));
        const float2 r = __fmul2_rn(g2, K);
        acc[0][p] = __ffma2_rn(r, ndy, acc[0][p]);
        acc[1][p] = __ffma2_rn(r, ndx, acc[1][p]);
        if constexpr (RES == RES_GRAD) {
          acc[2][p] = __fadd2_rn(acc[2][p], r);
          const float2 hx = __fmul2_rn(__fmul2_rn(r, K), ndx);
          acc[3][p] = __ffma2_rn(hx, ndy, acc[3][p]);
          acc[4][p] = __ffma2_rn(hx, ndx, acc[4][p]);
        } else if constexpr (RES == RES_SHEAR) {
          acc[2][p] = __ffma2_rn(f2(C.z, C.w), K, acc[2][p]);   // |G| K
        }
      } else {
        float k0, k1, b0, b1;
        core_eval<CORE_GAUSS, THICK, true, UNIF>(d2.x, C.x, tz[p].x, us2, ucf, k0, b0);
        core_eval<CORE_GAUSS, THICK, true, UNIF>(d2.y, C.x, tz[p].y, us2, ucf, k1, b1);
        const float2 K = f2(k0, k1);
        const float2 r = __fmul2_rn(g2, K);
        acc[0][p] = __ffma2_rn(r, ndy, acc[0][p]);
        acc[1][p] = __ffma2_rn(r, ndx, acc[1][p]);
        const float2 gb = __fmul2_rn(g2, f2(b0, b1));
        if constexpr (RES == RES_GRAD) {
          acc[2][p] = __fadd2_rn(acc[2][p], r);
          const float2 hx = __fmul2_rn(__fmul2_rn(gb, f2(-0.5f, -0.5f)), ndx);
          acc[3][p] = __ffma2_rn(hx, ndy, acc[3][p]);
          acc[4][p] = __ffma2_rn(hx, ndx, acc[4][p]);
          acc[5][p] = __fadd2_rn(acc[5][p], __ffma2_rn(gb, d2, __fadd2_rn(r, r)));
        } else if constexpr (RES == RES_VORT) {
          acc[2][p] = __fadd2_rn(acc[2][p], __ffma2_rn(gb, d2, __fadd2_rn(r, r)));
        } else {
          acc[2][p] = __ffma2_rn(f2(0.5f * fabsf(gb.x), 0.5f * fabsf(gb.y)), d2, acc[2][p]);
        }
      }
    }
  }
}

template <bool THICK, bool COMP, int RES>
__global__ void __launch_bounds__(P2P_THREADS, 4) p2p_packed_res_kernel(const P2PArgs a) {
  constexpr int NP = PRes<RES>::NP, NC = PRes<RES>::NC;
  constexpr int TPT = 2 * NP;
  constexpr int TB = P2P_THREADS * TPT;
  constexpr int WT = 32 * TPT;
  constexpr uint32_t TILE_BYTES = SRC_TILE * PK_ELEM * sizeof(float4);
  __shared__ __align__(128) float4 tile[NSTAGE][SRC_TILE * PK_ELEM];
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ unsigned smask[P2P_THREADS / 32][PK_NB];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  const int lane = tid & 31, warp = tid >> 5;
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  const bool unif = (~a.meta[0] == a.meta[1]) && (!THICK || ~a.meta[2] == a.meta[3]);
  float us2 = 0.0f, ucf = 0.0f;
  if (unif) {
    us2 = radius_term(CORE_GAUSS, __uint_as_float(a.meta[1])) +
          (THICK ? radius_term(CORE_GAUSS, __uint_as_float(a.meta[3])) : 0.0f);
    ucf = __frcp_rn(us2);
  }
  const float lim = 25.25f * us2;                 // far test with a 1 % margin (d > 5.02 s)

  uint32_t kt = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = *static_cast<volatile int*>(&s_item);
    if (item >= a.nitems) break;
    const int tb = item % a.ntb;
    const int sp = item / a.ntb;
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
    float2 ntx[NP], nty[NP], tz[NP];
    float2 acc[NC][NP], hi[NC][NP], lo[NC][NP];
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
        zs[h] = THICK ? radius_term(CORE_GAUSS, a.tr[ic]) : 0.0f;
      }
      ntx[p] = f2(xs[0], xs[1]);
      nty[p] = f2(ys[0], ys[1]);
      tz[p] = f2(zs[0], zs[1]);
#pragma unroll
      for (int c = 0; c < NC; ++c) acc[c][p] = hi[c][p] = lo[c][p] = f2(0.0f, 0.0f);
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
          record_failure(a.status, DEV_ERR_TIMEOUT, 230 + st, (int)kt, item);
          for (int s = 0; s < NSTAGE; ++s) (void)mbar_wait_bounded(&bar[(kt + s) % NSTAGE], ((kt + s) / NSTAGE) & 1u, WAIT_TRIES);
        }
        return;
      }
      const float4* tl = &tile[st][0];
      if (unif) {
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
        if (unif) {
          if (smask[warp][b] == 0u) res_block<RES, true, THICK, true, NP, NC>(blk, us2, ucf, ntx, nty, tz, acc);
          else res_block<RES, false, THICK, true, NP, NC>(blk, us2, ucf, ntx, nty, tz, acc);
        } else {
          res_block<RES, false, THICK, false, NP, NC>(blk, us2, ucf, ntx, nty, tz, acc);
        }
        if constexpr (COMP) {
#pragma unroll
          for (int c = 0; c < NC; ++c)
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              two_sum2(hi[c][p], lo[c][p], acc[c][p]);
              acc[c][p] = f2(0.0f, 0.0f);
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
        double v[NC];
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          const float2 H = COMP ? hi[c][p] : acc[c][p];
          const float2 L = COMP ? lo[c][p] : f2(0.0f, 0.0f);
          v[c] = (double)(h ? H.y : H.x) + (double)(h ? L.y : L.x);
        }
        constexpr int NO = NComp<RES>::v;
        double c[NO];
        c[0] = v[0];
        c[1] = -v[1];
        if constexpr (RES == RES_GRAD) {
          const double Q = -2.0 * v[4];
          c[2] = -2.0 * v[3];            // S1
          c[3] = Q + v[2];               // S2
          c[4] = Q + v[2] - v[5];        // S3
        } else {
          c[2] = v[2];
        }
        if (a.direct) {
          store_target<RES>(a, i, c);
        } else if (COMP) {
          double* qp = static_cast<double*>(a.part);
#pragma unroll
          for (int q = 0; q < NO; ++q) qp[((size_t)q * a.nsplit + sp) * a.nt + i] = c[q];
        } else {
          float* qp = static_cast<float*>(a.part);
#pragma unroll
          for (int q = 0; q < NO; ++q) qp[((size_t)q * a.nsplit + sp) * a.nt + i] = (float)c[q];
        }
      }
    }
    __syncthreads();
  }
}

}  // namespace

int packed_res_np(int res) {
  if (res == RES_GRAD) return PRes<RES_GRAD>::NP;
  return res == RES_SHEAR ? PRes<RES_SHEAR>::NP : PRes<RES_VORT>::NP;
}

cudaError_t packed_res_dispatch(int res, bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st,
                                int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, P2P_THREADS, 0);
    kern<<<grid, P2P_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
#define OBS_PRES(R)                                                                                         \
  if (res == R) {                                                                                           \
    if (thick) return comp ? run(p2p_packed_res_kernel<true, true, R>) : run(p2p_packed_res_kernel<true, false, R>); \
    return comp ? run(p2p_packed_res_kernel<false, true, R>) : run(p2p_packed_res_kernel<false, false, R>);  \
  }
  OBS_PRES(RES_GRAD)
  OBS_PRES(RES_VORT)
  OBS_PRES(RES_SHEAR)
#undef OBS_PRES
  return cudaErrorInvalidValue;
}

}  // namespace obs
