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

cudaError_t packed_dispatch(int core, int np, bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st,
                            int* occ) {
  if (core == CORE_GAUSS) {
    if (np == 4) return packed_dispatch_np<CORE_GAUSS, 4>(thick, comp, a, grid, st, occ);
    if (np == 3) return packed_dispatch_np<CORE_GAUSS, 3>(thick, comp, a, grid, st, occ);
    return packed_dispatch_np<CORE_GAUSS, 2>(thick, comp, a, grid, st, occ);
  }
  if (core == CORE_RM) {
    return np == 4 ? packed_dispatch_np<CORE_RM, 4>(thick, comp, a, grid, st, occ)
                   : packed_dispatch_np<CORE_RM, 2>(thick, comp, a, grid, st, occ);
  }
  switch (core) {   // the other cores: 2 target pairs per thread
    case CORE_V2: return packed_dispatch_np<CORE_V2, 2>(thick, comp, a, grid, st, occ);
    case CORE_WL: return packed_dispatch_np<CORE_WL, 2>(thick, comp, a, grid, st, occ);
    case CORE_V3: return packed_dispatch_np<CORE_V3, 2>(thick, comp, a, grid, st, occ);
    case CORE_SING: return packed_dispatch_np<CORE_SING, 2>(thick, comp, a, grid, st, occ);
    case CORE_CEXP:
      return np == 4 ? packed_dispatch_np<CORE_CEXP, 4>(thick, comp, a, grid, st, occ)
                     : packed_dispatch_np<CORE_CEXP, 2>(thick, comp, a, grid, st, occ);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t packed_launch_pack(const float* sx, const float* sy, const float* sr, const float* ss, const int* perm,
                               int ns, int ns_pad, int core, float4* out, unsigned* meta, cudaStream_t st) {
  pack_sources_dup_kernel<<<(ns_pad + 255) / 256, 256, 0, st>>>(sx, sy, sr, ss, perm, ns, ns_pad, core, out, meta);
  return cudaGetLastError();
}

}  // namespace obs
