// Particle-on-particle kernel instances for one core function (see p2p_kernel.cuh).
#include "p2p_dispatch.cuh"

namespace obs {
template cudaError_t p2p_dispatch<CORE_V2>(bool, int, bool, const P2PArgs*, int, cudaStream_t, int*);
}  // namespace obs
