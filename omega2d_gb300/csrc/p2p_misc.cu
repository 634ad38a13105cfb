// Streamfunction instances and the split-reduction kernels (see p2p_kernel.cuh).
#include "p2p_dispatch.cuh"

namespace obs {

cudaError_t p2p_dispatch_psi(bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, P2P_THREADS, 0);
    kern<<<grid, P2P_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
  constexpr int T = p2p_tpt(RES_PSI);
  if (thick) return comp ? run(p2p_kernel<CORE_RM, true, RES_PSI, true, T>) : run(p2p_kernel<CORE_RM, true, RES_PSI, false, T>);
  return comp ? run(p2p_kernel<CORE_RM, false, RES_PSI, true, T>) : run(p2p_kernel<CORE_RM, false, RES_PSI, false, T>);
}

cudaError_t p2p_dispatch_blobvort(bool comp, const P2PArgs* a, int grid, cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, P2P_THREADS, 0);
    kern<<<grid, P2P_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
  constexpr int T = p2p_tpt(RES_BLOBVORT);
  return comp ? run(p2p_kernel<CORE_GAUSS, false, RES_BLOBVORT, true, T>)
              : run(p2p_kernel<CORE_GAUSS, false, RES_BLOBVORT, false, T>);
}

cudaError_t p2p_reduce(int res, bool comp, const P2PArgs& a, cudaStream_t st) {
  const int threads = 256;
  const int blocks = (a.nt + threads - 1) / threads;
  const int cblocks = (int)(((size_t)a.nt * P2P_RED_SUB + threads - 1) / threads);
#define OBS_RED(R) \
  case R: if (comp) p2p_reduce_kernel<R, true><<<cblocks, threads, 0, st>>>(a); \
          else p2p_reduce_kernel<R, false><<<blocks, threads, 0, st>>>(a); break;
  switch (res) {
    OBS_RED(RES_VEL) OBS_RED(RES_GRAD) OBS_RED(RES_PSI) OBS_RED(RES_VORT) OBS_RED(RES_SHEAR) OBS_RED(RES_BLOBVORT)
    default: return cudaErrorInvalidValue;
  }
#undef OBS_RED
  return cudaGetLastError();
}

}  // namespace obs
