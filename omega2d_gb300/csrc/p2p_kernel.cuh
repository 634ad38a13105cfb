// p2p_kernel.cuh -- particle-on-particle direct-sum kernels (points_affect_points on sm_103a).
//
// Reference: points_affect_points<S,A> (src/Influence.h:56-416) with the pair kernels of
// src/Kernels.h:52-231 and the core functions of src/CoreFunc.h.
//
// Work decomposition (one persistent CTA per resident slot):
//   item = (target block, source split); a CTA takes items from a device counter until none
//   are left.  A target block is P2P_THREADS*TPT targets (TPT per thread, in registers); a
//   split is a contiguous run of SRC_TILE-source tiles.  Source tiles (float4 x, y, z, strength)
//   are staged into shared memory by the TMA bulk-copy engine (cp.async.bulk + mbarrier,
//   double-buffered) and read by every thread as broadcast float4 loads.
// Accumulation:
//   plain       : FP32 accumulators per target (the drop-in);
//   compensated : FP32 partials over COMP_BLOCK sources, folded into a (hi, lo) two-sum pair;
//                 each item's result leaves the kernel as a double, and splits are summed in
//                 FP64 in a fixed order by p2p_reduce_kernel; or (packed velocity kernel) as
//                 (hi, lo) pairs summed in split order by the last split of each target block
//                 to finish.
#pragma once

#include "obs_device.cuh"

namespace obs {

constexpr int P2P_THREADS = 128;
constexpr int SRC_TILE = 256;        // sources per shared-memory stage (4 KiB)
constexpr int NSTAGE = 2;
constexpr int COMP_BLOCK = 32;       // sources per FP32 partial in compensated mode
constexpr uint32_t WAIT_TRIES = 1u << 22;

struct P2PArgs {
  const float4* src;     // packed sources, padded to nst*SRC_TILE
  int nst;               // number of source tiles
  const float* tx;
  const float* ty;
  const float* tr;       // null for field-point targets
  int nt;                // targets
  int ntb;               // target blocks
  int nsplit;            // source splits
  int tiles_per_split;
  int nitems;            // ntb * nsplit
  int* counter;          // work counter (zeroed before launch)
  const unsigned* meta;  // radius extrema: [0] ~min src bits, [1] max src, [2] ~min tgt, [3] max tgt
  int* status;           // DEV_ERR_* bits
  float* out[6];         // u, v, then extras (grad: ux vx uy vy; vort: w; shear: e; psi: p)
  void* part;            // split partials [ncomp][nsplit][nt] (double if compensated, else float)
  const int* perm;       // targets processed in binned order: output index of binned target i
  int direct;            // nsplit == 1: write outputs from the main kernel
  int finalize;          // apply fs + (1/2pi) in the epilogue
  double fsx, fsy;
  // Non-null (packed velocity kernel, 1 < nsplit <= 64): per target block arrival counts,
  // zeroed before launch.  Items then run target-block-major, the partials' row stride is
  // ntb * TB (compensated partials as (hi, lo) FP32 pairs), and the last split of a block to
  // finish sums the block's partials in split order and writes its targets; no reduction
  // launch follows.
  int* blkcnt;
};

template <int RES> struct NComp;
template <> struct NComp<RES_VEL>   { static constexpr int v = 2; };
template <> struct NComp<RES_GRAD>  { static constexpr int v = 5; };  // u, v, S1, S2, S3
template <> struct NComp<RES_PSI>   { static constexpr int v = 1; };
template <> struct NComp<RES_VORT>  { static constexpr int v = 3; };
template <> struct NComp<RES_SHEAR> { static constexpr int v = 3; };
template <> struct NComp<RES_BLOBVORT> { static constexpr int v = 1; };

constexpr double kInv2Pi = 0.15915494309189535;   // 0.5/pi, src/ElementBase.h:216

// Write one target's accumulated components into the caller's arrays.
//   accumulate (reference semantics, src/Influence.h:359-360): out += sum
//   finalize   (src/ElementBase.h:215-234): u = fs + (u + sum)/(2 pi); extras *= 1/(2 pi)
// GRAD components: S1 = sum G*b*dx*dy, S2 = sum G*(b dx^2 + K), S3 = -sum G*(b dy^2 + K);
// then du/dx = -S1, dv/dy = S1, dv/dx = S2, du/dy = S3 (kernelug_0v_0b, src/Kernels.h:112-133).
template <int RES>
__device__ __forceinline__ void store_target(const P2PArgs& a, int ib, const double* c) {
  const double f = a.finalize ? kInv2Pi : 1.0;
  const int i = a.perm ? a.perm[ib] : ib;
  if ((unsigned)i >= (unsigned)a.nt) return;      // never taken: perm is a permutation of 0..nt-1
  auto put = [&](int k, double add, double fs) {
    float* p = a.out[k];
    const double v = ((double)p[i] + add) * f + fs;
    p[i] = (float)v;
  };
  if constexpr (RES == RES_PSI || RES == RES_BLOBVORT) {
    put(2, c[0], 0.0);
    return;
  }
  const double fsx = a.finalize ? a.fsx : 0.0, fsy = a.finalize ? a.fsy : 0.0;
  put(0, c[0], fsx);
  put(1, c[1], fsy);
  if constexpr (RES == RES_GRAD) {
    put(2, -c[2], 0.0);   // ux
    put(3, c[3], 0.0);    // vx
    put(4, c[4], 0.0);    // uy
    put(5, c[2], 0.0);    // vy
  } else if constexpr (RES == RES_VORT || RES == RES_SHEAR) {
    put(2, c[2], 0.0);
  }
}

template <int CORE, bool THICK, int RES, bool COMP, int TPT, bool UNIF>
__device__ __forceinline__ void p2p_tile(const float4* __restrict__ tile,
                                         const float (&tx)[TPT], const float (&ty)[TPT], const float (&tz)[TPT],
                                         float us2, float ucf,
                                         float (&acc)[TPT][NComp<RES>::v],
                                         float (&hi)[TPT][NComp<RES>::v], float (&lo)[TPT][NComp<RES>::v]) {
  constexpr int NC = NComp<RES>::v;
  constexpr bool GRADCORE = (RES == RES_GRAD || RES == RES_VORT || RES == RES_SHEAR);
  constexpr int NB = COMP ? SRC_TILE / COMP_BLOCK : 1;
  constexpr int BLK = COMP ? COMP_BLOCK : SRC_TILE;
  for (int b = 0; b < NB; ++b) {
#pragma unroll 4
    for (int jj = 0; jj < BLK; ++jj) {
      const float4 s = tile[b * BLK + jj];
#pragma unroll
      for (int k = 0; k < TPT; ++k) {
        const float ndx = s.x - tx[k];    // -dx
        const float ndy = s.y - ty[k];    // -dy
        const float d2 = fmaf(ndx, ndx, ndy * ndy);
        if constexpr (RES == RES_PSI) {
          // kernelp: -strength * 0.5 * log(d^2 + sr^2 (+ tr^2)), src/Kernels.h:52-74
          const float q = d2 + (THICK ? s.z + tz[k] : s.z);
          acc[k][0] = fmaf(-s.w * (0.5f * kLn2), lg2_a(q), acc[k][0]);
        } else if constexpr (RES == RES_BLOBVORT) {
          // points_affect_points_vorticity (src/InfluenceVort.h:96-110, the non-Vc branch: no
          // cut-off): w += 2 G exp(-d^2/s^2) / s^2, s the source radius (s.z = s^2)
          const float cf = UNIF ? ucf : rcp_a(s.z);
          const float e = ex2_a(d2 * cf * -kLog2e);
          acc[k][0] = fmaf(2.0f * s.w * cf, e, acc[k][0]);
        } else {
          float K, B = 0.0f;
          core_eval<CORE, THICK, GRADCORE, UNIF>(d2, s.z, tz[k], us2, ucf, K, B);
          const float r2 = s.w * K;
          acc[k][0] = fmaf(r2, ndy, acc[k][0]);     // u -= r2*dy
          acc[k][1] = fmaf(-r2, ndx, acc[k][1]);    // v += r2*dx
          if constexpr (RES == RES_GRAD) {
            const float bb = s.w * B;
            const float bx = bb * ndx;
            acc[k][2] = fmaf(bx, ndy, acc[k][2]);             // S1 += b dx dy
            acc[k][3] = acc[k][3] + fmaf(bx, ndx, r2);        // S2 += b dx^2 + r2
            acc[k][4] = acc[k][4] - fmaf(bb * ndy, ndy, r2);  // S3 -= b dy^2 + r2
          } else if constexpr (RES == RES_VORT) {
            // kerneluw: w += dvdx - dudy = b d^2 + 2 r2 (src/Kernels.h:139-179)
            acc[k][2] = acc[k][2] + fmaf(s.w * B, d2, 2.0f * r2);
          } else if constexpr (RES == RES_SHEAR) {
            // kernelue: e += sqrt(dudx^2 + asym^2/4) = |b| d^2 / 2 (src/Kernels.h:185-231)
            acc[k][2] = fmaf(0.5f * fabsf(s.w * B), d2, acc[k][2]);
          }
        }
      }
    }
    if constexpr (COMP) {
#pragma unroll
      for (int k = 0; k < TPT; ++k)
#pragma unroll
        for (int c = 0; c < NC; ++c) {
          two_sum_acc(hi[k][c], lo[k][c], acc[k][c]);
          acc[k][c] = 0.0f;
        }
    }
  }
}

template <int CORE, bool THICK, int RES, bool COMP, int TPT>
__global__ void __launch_bounds__(P2P_THREADS)
p2p_kernel(const P2PArgs a) {
  constexpr int NC = NComp<RES>::v;
  constexpr int TB = P2P_THREADS * TPT;
  constexpr uint32_t TILE_BYTES = SRC_TILE * sizeof(float4);
  __shared__ __align__(128) float4 tile[NSTAGE][SRC_TILE];
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ int s_item;

  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();

  // All radii equal -> hoist the core's radius combination (decided per launch, no host sync).
  // meta[0] holds ~(smallest radius bits), meta[1] the largest; likewise [2], [3] for targets.
  const bool unif = (~a.meta[0] == a.meta[1]) && (!THICK || ~a.meta[2] == a.meta[3]);
  float us2 = 0.0f, ucf = 0.0f;
  if (unif) {
    const float rs = __uint_as_float(a.meta[1]);
    const float rt = THICK ? __uint_as_float(a.meta[3]) : 0.0f;
    us2 = radius_term(CORE, rs) + (THICK ? radius_term(CORE, rt) : 0.0f);
    ucf = __frcp_rn(us2);
  }

  uint32_t kt = 0;   // tiles consumed by this CTA so far (mbarrier phase bookkeeping)
  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = *static_cast<volatile int*>(&s_item);
    if (item >= a.nitems) break;
    const int tb = item % a.ntb;
    const int sp = item / a.ntb;
    const int tile0 = sp * a.tiles_per_split;
    const int ntile = min(a.tiles_per_split, a.nst - tile0);
    (void)OBS_CHECK(a.status, sp < a.nsplit && ntile >= 1, 104, item, ntile);

    if (tid == 0) {
      fence_proxy_async_smem();   // previous item's reads of these stages precede the new copies
      for (int s = 0; s < NSTAGE && s < ntile; ++s) {
        const int st = (kt + s) % NSTAGE;
        int tix = tile0 + s;
        if (!OBS_CHECK(a.status, tix >= 0 && tix < a.nst, 101, tix, item)) tix = 0;
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_g2s(&tile[st][0], a.src + (size_t)tix * SRC_TILE, TILE_BYTES, &bar[st]);
      }
    }

    float tx[TPT], ty[TPT], tz[TPT];
    float acc[TPT][NC], hi[TPT][NC], lo[TPT][NC];
#pragma unroll
    for (int k = 0; k < TPT; ++k) {
      const int i = tb * TB + k * P2P_THREADS + tid;
      int ic = (i < a.nt) ? i : (a.nt - 1);
      if (!OBS_CHECK(a.status, ic >= 0 && ic < a.nt, 102, ic, item)) ic = 0;
      tx[k] = a.tx[ic];
      ty[k] = a.ty[ic];
      tz[k] = THICK ? radius_term(RES == RES_PSI ? CORE_RM : CORE, a.tr[ic]) : 0.0f;
#pragma unroll
      for (int c = 0; c < NC; ++c) { acc[k][c] = 0.0f; hi[k][c] = 0.0f; lo[k][c] = 0.0f; }
    }

    for (int t = 0; t < ntile; ++t, ++kt) {
      const int st = kt % NSTAGE;
      const bool ok = mbar_wait_bounded(&bar[st], (kt / NSTAGE) & 1u, WAIT_TRIES);
      if (__syncthreads_or(!ok)) {
        // a tile never arrived: record where, let any copy still in flight land, and stop
        if (tid == 0) {
          record_failure(a.status, DEV_ERR_TIMEOUT, 200 + st, (int)kt, item);
          for (int s = 0; s < NSTAGE; ++s) (void)mbar_wait_bounded(&bar[(kt + s) % NSTAGE], ((kt + s) / NSTAGE) & 1u, WAIT_TRIES);
        }
        return;
      }
      if (unif)
        p2p_tile<CORE, THICK, RES, COMP, TPT, true>(&tile[st][0], tx, ty, tz, us2, ucf, acc, hi, lo);
      else
        p2p_tile<CORE, THICK, RES, COMP, TPT, false>(&tile[st][0], tx, ty, tz, us2, ucf, acc, hi, lo);
      __syncthreads();   // every thread is done with this stage
      if (tid == 0 && t + NSTAGE < ntile) {
        int tix = tile0 + t + NSTAGE;
        if (!OBS_CHECK(a.status, tix >= 0 && tix < a.nst, 101, tix, item)) tix = 0;
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[st], TILE_BYTES);
        bulk_g2s(&tile[st][0], a.src + (size_t)tix * SRC_TILE, TILE_BYTES, &bar[st]);
      }
    }

#pragma unroll
    for (int k = 0; k < TPT; ++k) {
      const int i = tb * TB + k * P2P_THREADS + tid;
      if (i >= a.nt) continue;
      double c[NC];
#pragma unroll
      for (int q = 0; q < NC; ++q)
        c[q] = COMP ? ((double)hi[k][q] + (double)lo[k][q]) : (double)acc[k][q];
      if (!OBS_CHECK(a.status, sp < a.nsplit && i < a.nt, 103, i, sp)) continue;
      if (a.direct) {
        store_target<RES>(a, i, c);
      } else if (COMP) {
        double* p = static_cast<double*>(a.part);
#pragma unroll
        for (int q = 0; q < NC; ++q) p[((size_t)q * a.nsplit + sp) * a.nt + i] = c[q];
      } else {
        float* p = static_cast<float*>(a.part);
#pragma unroll
        for (int q = 0; q < NC; ++q) p[((size_t)q * a.nsplit + sp) * a.nt + i] = acc[k][q];
      }
    }
    __syncthreads();   // the whole CTA leaves this item before thread 0 fetches the next one
  }
}

// Sum the split partials of each target in a fixed order (FP64 for compensated, FP32 for
// plain) and store like the direct epilogue.
constexpr int P2P_RED_SUB = 4;   // threads per target in the compensated split reduction
template <int RES, bool COMP>
__global__ void p2p_reduce_kernel(const P2PArgs a) {
  constexpr int NC = NComp<RES>::v;
  if (COMP) {
    // FP64 adds issue at about 2 per SM-clock on this GPU: P2P_RED_SUB consecutive threads share
    // a target, each summing every P2P_RED_SUB-th split in order, then a fixed shuffle tree
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    const int i = t / P2P_RED_SUB, sub = t % P2P_RED_SUB;
    const bool live = i < a.nt;
    const int ic = live ? i : a.nt - 1;
    double c[NC];
#pragma unroll
    for (int q = 0; q < NC; ++q) {
      const double* p = static_cast<const double*>(a.part) + (size_t)q * a.nsplit * a.nt + ic;
      double s = 0.0;
#pragma unroll 4
      for (int k = sub; k < a.nsplit; k += P2P_RED_SUB) s += p[(size_t)k * a.nt];
#pragma unroll
      for (int o = 1; o < P2P_RED_SUB; o <<= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
      c[q] = s;
    }
    if (live && sub == 0) store_target<RES>(a, i, c);
    return;
  }
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.nt) return;
  double c[NC];
#pragma unroll
  for (int q = 0; q < NC; ++q) {
    const float* p = static_cast<const float*>(a.part) + (size_t)q * a.nsplit * a.nt + i;
    float s = 0.0f;
#pragma unroll 8
    for (int k = 0; k < a.nsplit; ++k) s += p[(size_t)k * a.nt];
    c[q] = (double)s;
  }
  store_target<RES>(a, i, c);
}

}  // namespace obs
