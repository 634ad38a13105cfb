// p2p_packed.cu -- instances and launch helpers of the packed-FP32 velocity kernels.
#include "obs_context.h"
#include "p2p_packed.cuh"

namespace obs {

namespace {

// Sources staged for the packed kernels: (x, x, y, y), (G, G, -G, -G), (z, z, |G|, |G|); padded
// with zero-strength sources at the origin and radius term 1 (finite for both cores).  With a
// permutation, staged source i is the caller's source perm[i].
__global__ void pack_sources_dup_kernel(const float* __restrict__ sx, const float* __restrict__ sy,
                                        const float* __restrict__ sr, const float* __restrict__ ss,
                                        const int* __restrict__ perm, int ns, int ns_pad, int core,
                                        float4* __restrict__ out, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  int j = (i < ns && perm) ? perm[i] : i;
  if ((unsigned)j >= (unsigned)ns) j = i;         // never taken for i < ns: perm is a permutation
  const float r = (i < ns && sr) ? sr[j] : 0.0f;
  if (i < ns) {
    const float x = sx[j], y = sy[j], g = ss[j], z = radius_term(core, r);
    out[PK_ELEM * i] = make_float4(x, x, y, y);
    out[PK_ELEM * i + 1] = make_float4(g, g, -g, -g);
    out[PK_ELEM * i + 2] = make_float4(z, z, fabsf(g), fabsf(g));
  } else if (i < ns_pad) {
    out[PK_ELEM * i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    out[PK_ELEM * i + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
    out[PK_ELEM * i + 2] = make_float4(1.0f, 1.0f, 0.0f, 0.0f);
  }
  // radius extrema, as pack_sources_kernel does
  unsigned rmin = (i < ns) ? __float_as_uint(r) : ~0u;
  unsigned rmax = (i < ns) ? __float_as_uint(r) : 0u;
  int any = (i < ns) ? 1 : 0;
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

template <int CORE, int NP>
cudaError_t packed_dispatch_np(bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, P2P_THREADS, 0);
    kern<<<grid, P2P_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
  if (thick) return comp ? run(p2p_packed_kernel<CORE, true, true, NP>) : run(p2p_packed_kernel<CORE, true, false, NP>);
  return comp ? run(p2p_packed_kernel<CORE, false, true, NP>) : run(p2p_packed_kernel<CORE, false, false, NP>);
}

}  // namespace

bool packed_supported(int core, int res) {
  if (res == RES_VEL) return core >= CORE_RM && core <= CORE_CEXP;
  return core == CORE_GAUSS && (res == RES_GRAD || res == RES_VORT || res == RES_SHEAR);
}

int packed_np(int core, int variant, int nt) {
  if (variant == OBS_VARIANT_PACKED2) return 2;
  if (variant == OBS_VARIANT_PACKED3) return core == CORE_GAUSS ? 3 : 2;
  if (variant == OBS_VARIANT_PACKED4) return 4;
  // AUTO, from the 1M Gaussian patch (compensated, Ginter/s with 4 vs 2 target pairs):
  // Gaussian 4111 vs 3785 (Morton order), RM 4116 vs 4017, Vatistas-2 3810 vs 3776,
  // Winckelmans-Leonard 2996 vs 2762; the singular core 3694 vs 3732 and Vatistas-3 keep 2.
  // Fewer targets need the smaller target blocks to fill the GPU (uniform [-1,1]^2 clouds:
  // 20k RM 2391 vs 2136; 65k compact exponential, Morton order, 3383 vs 3190, Gaussian 3305
  // vs 3439)
  if (core == CORE_V3 || core == CORE_SING) return 2;
  if (nt < (core == CORE_CEXP ? 98304 : 49152)) return 2;
  return 4;
}

// np must come from packed_np: the host sizes the target blocks with it
cudaError_t packed_dispatch(int core, int np, bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st,
                            int* occ) {
  if (np == 3 && core != CORE_GAUSS) return cudaErrorInvalidValue;
  if (np != 2 && np != 3 && np != 4) return cudaErrorInvalidValue;
#define OBS_PACKED_NP24(C)                                                      \
  return np == 4 ? packed_dispatch_np<C, 4>(thick, comp, a, grid, st, occ)      \
                 : packed_dispatch_np<C, 2>(thick, comp, a, grid, st, occ)
  switch (core) {
    case CORE_GAUSS:
      if (np == 3) return packed_dispatch_np<CORE_GAUSS, 3>(thick, comp, a, grid, st, occ);
      OBS_PACKED_NP24(CORE_GAUSS);
    case CORE_RM: OBS_PACKED_NP24(CORE_RM);
    case CORE_V2: OBS_PACKED_NP24(CORE_V2);
    case CORE_WL: OBS_PACKED_NP24(CORE_WL);
    case CORE_V3: OBS_PACKED_NP24(CORE_V3);
    case CORE_SING: OBS_PACKED_NP24(CORE_SING);
    case CORE_CEXP: OBS_PACKED_NP24(CORE_CEXP);
    default: return cudaErrorInvalidValue;
  }
#undef OBS_PACKED_NP24
}

cudaError_t packed_launch_pack(const float* sx, const float* sy, const float* sr, const float* ss, const int* perm,
                               int ns, int ns_pad, int core, float4* out, unsigned* meta, cudaStream_t st) {
  pack_sources_dup_kernel<<<(ns_pad + 255) / 256, 256, 0, st>>>(sx, sy, sr, ss, perm, ns, ns_pad, core, out, meta);
  return cudaGetLastError();
}

}  // namespace obs
