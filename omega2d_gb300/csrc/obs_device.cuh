// obs_device.cuh -- device-side building blocks of the direct Biot-Savart engine (sm_103a).
//
// Core functions, hardware-approximation wrappers, compensated (two-sum) accumulation and the
// TMA bulk-copy / mbarrier primitives used by every pairwise kernel.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace obs {

// core-function ids (same values as OBS_CORE_* in include/omega2d_gb300.h)
enum : int { CORE_RM = 1, CORE_GAUSS = 2, CORE_V2 = 3, CORE_WL = 4, CORE_V3 = 5, CORE_SING = 6, CORE_CEXP = 7 };
// result types (same values as the reference's results_t, src/ResultsType.h:26-32)
enum : int { RES_VEL = 1, RES_GRAD = 2, RES_PSI = 3, RES_VORT = 4, RES_SHEAR = 5 };
// Gaussian blob vorticity at field points (points_affect_points_vorticity, src/InfluenceVort.h);
// internal result type of the generic kernel, not a results_t value
enum : int { RES_BLOBVORT = 6 };

// status bits written by kernels (read back by the host)
enum : int { DEV_ERR_TIMEOUT = 1, DEV_ERR_BAD_ITEM = 2, DEV_ERR_BOUNDS = 4, DEV_ERR_SINGULAR = 8 };

// Device status block: [0] DEV_ERR_* bits, [1] first check code, [2..3] its two values.
constexpr int kStatusWords = 4;

// First-failure record (kept even in normal builds for the bounded-wait timeout path).
__device__ __forceinline__ void record_failure(int* status, int bit, int code, int v1, int v2) {
  atomicOr(&status[0], bit);
  if (atomicCAS(&status[1], 0, code) == 0) {
    status[2] = v1;
    status[3] = v2;
  }
}

#ifdef OBS_DEVICE_CHECKS
// Bounds check that records the first violation and reports false so the caller skips or
// clamps the access (debug builds only).
#define OBS_CHECK(status, cond, code, v1, v2) \
  ((cond) ? true : (::obs::record_failure((status), ::obs::DEV_ERR_BOUNDS, (code), (int)(v1), (int)(v2)), false))
#else
#define OBS_CHECK(status, cond, code, v1, v2) true
#endif

constexpr float kLog2e = 1.4426950408889634f;
constexpr float kLn2 = 0.6931471805599453f;

// ---------------------------------------------------------------- PTX approximations
// Documented PTX forms; maximum errors per the PTX ISA: rcp 1 ulp, sqrt/rsqrt ~2 ulp,
// ex2 2 ulp over the full range, lg2 2^-22 absolute.
__device__ __forceinline__ float rcp_a(float x) { float r; asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }
__device__ __forceinline__ float rsqrt_a(float x) { float r; asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }
__device__ __forceinline__ float sqrt_a(float x) { float r; asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }
__device__ __forceinline__ float ex2_a(float x) { float r; asm("ex2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }
__device__ __forceinline__ float lg2_a(float x) { float r; asm("lg2.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(x)); return r; }

// ---------------------------------------------------------------- per-core source/target term
// Each source/target carries one precomputed radius term z so that the pair only combines
// them.  The forms follow the non-singular-target core functions of src/CoreFunc.h:
//   RM, Gaussian, WL, compact-exp : z = r^2          (sr*sr + tr*tr)
//   Vatistas n=2                  : z = (r^2)^2      (s2*s2 + t2*t2)
//   Vatistas n=3                  : z = (r^2)^3      (s2*s2*s2 + t2*t2*t2)
//   singular                      : unused
// The streamfunction (kernelp, src/Kernels.h:52-74) always uses z = r^2.
__host__ __device__ __forceinline__ float radius_term(int core, float r) {
  const float s2 = r * r;
  if (core == CORE_V2) return s2 * s2;
  if (core == CORE_V3) return s2 * s2 * s2;
  return s2;
}

// ---------------------------------------------------------------- Gaussian-core series
// g(x) = (1 - e^-x)/x = sum_{n>=0} (-x)^n/(n+1)!  and  g'(x) = sum_{m>=0} (m+1)(-1)^(m+1) x^m/(m+2)!
// (Taylor series of the exponential).  Truncated after the x^12 term: for 0 <= x < 1 the
// remainder is below 2e-9 relative, under FP32 rounding.
__device__ __forceinline__ float gauss_g_series(float x) {
  float p = 1.0f / 6227020800.0f;
  p = fmaf(p, x, -1.0f / 479001600.0f);
  p = fmaf(p, x, 1.0f / 39916800.0f);
  p = fmaf(p, x, -1.0f / 3628800.0f);
  p = fmaf(p, x, 1.0f / 362880.0f);
  p = fmaf(p, x, -1.0f / 40320.0f);
  p = fmaf(p, x, 1.0f / 5040.0f);
  p = fmaf(p, x, -1.0f / 720.0f);
  p = fmaf(p, x, 1.0f / 120.0f);
  p = fmaf(p, x, -1.0f / 24.0f);
  p = fmaf(p, x, 1.0f / 6.0f);
  p = fmaf(p, x, -0.5f);
  return fmaf(p, x, 1.0f);
}

__device__ __forceinline__ float gauss_gprime_series(float x) {
  float p = -1.0f / 6706022400.0f;
  p = fmaf(p, x, 1.0f / 518918400.0f);
  p = fmaf(p, x, -1.0f / 43545600.0f);
  p = fmaf(p, x, 1.0f / 3991680.0f);
  p = fmaf(p, x, -1.0f / 403200.0f);
  p = fmaf(p, x, 1.0f / 45360.0f);
  p = fmaf(p, x, -1.0f / 5760.0f);
  p = fmaf(p, x, 1.0f / 840.0f);
  p = fmaf(p, x, -1.0f / 144.0f);
  p = fmaf(p, x, 1.0f / 30.0f);
  p = fmaf(p, x, -0.125f);
  p = fmaf(p, x, 1.0f / 3.0f);
  return fmaf(p, x, -0.5f);
}

// ---------------------------------------------------------------- core functions
// K(d^2) such that one pair contributes strength*K*(-dy, dx), and (GRAD) B = 2 dK/d(d^2) as
// the reference's "bbb".  zs/zt: radius terms; THICK selects the two-radius form.  UNIF: all
// radii equal, so s2 = us2 and 1/s2 = ucf are hoisted out of the pair loop.
template <int CORE, bool THICK, bool GRAD, bool UNIF>
__device__ __forceinline__ void core_eval(float d2, float zs, float zt, float us2, float ucf,
                                          float& K, float& B) {
  if constexpr (CORE == CORE_RM) {
    // src/CoreFunc.h:47-80: 1/(d^2 + s^2), bbb = -2 K^2
    const float s2 = UNIF ? us2 : (THICK ? zs + zt : zs);
    K = rcp_a(d2 + s2);
    if constexpr (GRAD) B = -2.0f * K * K;
  } else if constexpr (CORE == CORE_GAUSS) {
    // src/CoreFunc.h:111-181 ("exponential" core): reld2 = d^2/s^2;
    // reld2 > 16 -> 1/d^2, reld2 < 0.001 -> 1/s^2, else (1 - e^-reld2)/d^2
    const float cf = UNIF ? ucf : rcp_a(THICK ? zs + zt : zs);
    const float ood2 = rcp_a(d2);
    const float x = d2 * cf;
    const float e = ex2_a(x * -kLog2e);
    float k = fmaf(-ood2, e, ood2);
    k = (x > 16.0f) ? ood2 : k;
    k = (x < 0.001f) ? cf : k;
    K = k;
    if constexpr (GRAD) {
      // bbb = 2 cf^2 g'(x) with g(x) = (1 - e^-x)/x.  The closed form (2 cf e - 2K)/d^2 cancels
      // for x < 1 (g' -> -1/2 while each term ~ 1/x), so there g and g' come from their Taylor
      // series; the x < 0.001 branch keeps the reference's cut-off value K = cf with the
      // reference's bbb there, -2 cf^2 g(x).
      if (x < 1.0f) {
        const float g = gauss_g_series(x);
        const float gp = gauss_gprime_series(x);
        K = (x < 0.001f) ? cf : cf * g;
        B = (x < 0.001f) ? -2.0f * cf * cf * g : 2.0f * cf * cf * gp;
      } else {
        B = (2.0f * cf * e - 2.0f * k) * ood2;
      }
    }
  } else if constexpr (CORE == CORE_V2) {
    // src/CoreFunc.h:238-274: 1/sqrt(d^4 + s^4 (+ t^4)), bbb = -2 K^3 d^2
    const float a = fmaf(d2, d2, THICK ? zs + zt : zs);
    K = rsqrt_a(a);
    if constexpr (GRAD) B = -2.0f * K * K * K * d2;
  } else if constexpr (CORE == CORE_WL) {
    // src/CoreFunc.h:189-229: (d2 + s2 + s2)/(d2 + s2)^2, bbb = (2 - 4 K dd)/dd^2
    const float s2 = UNIF ? us2 : (THICK ? zs + zt : zs);
    const float dd = d2 + s2;
    const float o = rcp_a(dd * dd);
    K = (dd + s2) * o;
    if constexpr (GRAD) B = (2.0f - 4.0f * K * dd) * o;
  } else if constexpr (CORE == CORE_V3) {
    // src/CoreFunc.h:283-321: (d^6 + s^6 (+ t^6))^(-1/3), bbb = -2 d^4 K / a = -2 d^4 K^4
    const float a = fmaf(d2 * d2, d2, THICK ? zs + zt : zs);
    K = ex2_a(lg2_a(a) * (-1.0f / 3.0f));
    if constexpr (GRAD) { const float k2 = K * K; B = -2.0f * d2 * d2 * k2 * k2; }
  } else if constexpr (CORE == CORE_SING) {
    // point vortex: 1/d^2, the coincident pair contributes nothing
    K = (d2 > 0.0f) ? rcp_a(d2) : 0.0f;
    if constexpr (GRAD) B = -2.0f * K * K;
  } else {  // CORE_CEXP
    // compact exponential: y = (d^2/s^2)^(3/2); y > 16 -> 1/d^2; y < 0.001 -> (d/s^3)(1 - y/2);
    // else (1 - e^-y)/d^2.  bbb = (3 y e^-y / d^2 - 2K)/d^2.
    const float cf = UNIF ? ucf : rcp_a(THICK ? zs + zt : zs);
    const float x = d2 * cf;
    const float sx = sqrt_a(x);
    const float y = x * sx;
    const float ood2 = rcp_a(d2);
    const float e = ex2_a(y * -kLog2e);
    float k = fmaf(-ood2, e, ood2);
    k = (y > 16.0f) ? ood2 : k;
    k = (y < 0.001f) ? sx * cf * fmaf(-0.5f, y, 1.0f) : k;
    K = k;
    if constexpr (GRAD) {
      float b = (3.0f * y * e * ood2 - 2.0f * k) * ood2;
      b = (y > 16.0f) ? -2.0f * ood2 * ood2 : b;
      B = (d2 == 0.0f) ? 0.0f : b;
    }
  }
}

// ---------------------------------------------------------------- compensated accumulation
// Knuth two-sum: hi + lo accumulates b exactly up to the rounding of lo itself.
__device__ __forceinline__ void two_sum_acc(float& hi, float& lo, float b) {
  const float s = hi + b;
  const float bp = s - hi;
  const float ap = s - bp;
  const float err = (hi - ap) + (b - bp);
  hi = s;
  lo += err;
}

// ---------------------------------------------------------------- packed (f32x2) helpers
__device__ __forceinline__ float2 f2(float a, float b) { return make_float2(a, b); }

// packed two-sum: hi + lo accumulates b
__device__ __forceinline__ void two_sum2(float2& hi, float2& lo, float2 b) {
  const float2 m1 = f2(-1.0f, -1.0f);
  const float2 s = __fadd2_rn(hi, b);
  const float2 bp = __ffma2_rn(hi, m1, s);        // s - hi
  const float2 ap = __ffma2_rn(bp, m1, s);        // s - bp
  const float2 da = __ffma2_rn(ap, m1, hi);       // hi - ap
  const float2 db = __ffma2_rn(bp, m1, b);        // b - bp
  lo = __fadd2_rn(lo, __fadd2_rn(da, db));
  hi = s;
}

// ---------------------------------------------------------------- TMA bulk copy + mbarrier
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" :: "r"(smem_addr(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void fence_mbar_init() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;"
               :: "r"(smem_addr(bar)), "r"(bytes) : "memory");
}

// Order this thread's earlier generic-proxy shared-memory accesses (made visible to it by a
// CTA barrier) before subsequent async-proxy (TMA) writes to the same buffer.
__device__ __forceinline__ void fence_proxy_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// one-dimensional bulk copy global -> shared (TMA engine); 16-byte aligned, size % 16 == 0
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
               :: "r"(smem_addr(dst)), "l"(src), "r"(bytes), "r"(smem_addr(bar)) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile("{\n\t.reg .pred p;\n\t"
               "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
               "selp.u32 %0, 1, 0, p;\n\t}"
               : "=r"(ok) : "r"(smem_addr(bar)), "r"(parity) : "memory");
  return ok != 0;
}

// Bounded wait: gives up after max_tries polls (each try_wait may itself suspend for a
// hardware-defined interval) and reports false so the caller can flag a timeout.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity, uint32_t max_tries) {
  for (uint32_t i = 0; i < max_tries; ++i)
    if (mbar_try_wait(bar, parity)) return true;
  return false;
}

}  // namespace obs
