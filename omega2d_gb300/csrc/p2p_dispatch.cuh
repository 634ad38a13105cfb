// p2p_dispatch.cuh -- template dispatch for the particle-on-particle kernels of one core.
// Each core's instances live in their own translation unit (p2p_core_<name>.cu) so the build
// compiles them in parallel.
#pragma once

#include "p2p_kernel.cuh"

namespace obs {

// Targets per thread for each result type (register budget: 4 for velocity/streamfunction,
// 2 when the gradient-form core and extra accumulators are live).
__host__ __device__ constexpr int p2p_tpt(int res) {
  return (res == RES_VEL || res == RES_PSI || res == RES_BLOBVORT) ? 4 : 2;
}

// a == nullptr: report resident CTAs per SM in *occ; otherwise launch grid CTAs on st.
template <int CORE>
cudaError_t p2p_dispatch(bool thick, int res, bool comp, const P2PArgs* a, int grid,
                         cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, P2P_THREADS, 0);
    kern<<<grid, P2P_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
#define OBS_P2P_CASE(R, TPT_)                                                         \
  case R:                                                                             \
    if (thick) return comp ? run(p2p_kernel<CORE, true, R, true, TPT_>)               \
                           : run(p2p_kernel<CORE, true, R, false, TPT_>);             \
    return comp ? run(p2p_kernel<CORE, false, R, true, TPT_>)                         \
                : run(p2p_kernel<CORE, false, R, false, TPT_>);
  switch (res) {
    OBS_P2P_CASE(RES_VEL, p2p_tpt(RES_VEL))
    OBS_P2P_CASE(RES_GRAD, p2p_tpt(RES_GRAD))
    OBS_P2P_CASE(RES_VORT, p2p_tpt(RES_VORT))
    OBS_P2P_CASE(RES_SHEAR, p2p_tpt(RES_SHEAR))
    default: break;
  }
#undef OBS_P2P_CASE
  return cudaErrorInvalidValue;
}

// Instances live in p2p_core_<name>.cu; other translation units only declare them.
extern template cudaError_t p2p_dispatch<CORE_RM>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_GAUSS>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_V2>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_WL>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_V3>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_SING>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
extern template cudaError_t p2p_dispatch<CORE_CEXP>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);

// streamfunction: core-independent (kernelp), instantiated once
cudaError_t p2p_dispatch_psi(bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st, int* occ);
// Gaussian blob vorticity at field points, instantiated once
cudaError_t p2p_dispatch_blobvort(bool comp, const P2PArgs* a, int grid, cudaStream_t st, int* occ);
cudaError_t p2p_reduce(int res, bool comp, const P2PArgs& a, cudaStream_t st);

}  // namespace obs
