// obs_context.h -- host-side engine state shared by the C-ABI translation units.
#pragma once

#include <cuda_runtime.h>
#include <cstddef>
#include <cstdint>

#include "omega2d_gb300.h"

namespace obs {

// Device buffer that only grows.  Growing synchronizes the owning stream first so no queued
// kernel can still be using the old allocation.
struct DevBuf {
  void* p = nullptr;
  size_t cap = 0;
  int ensure(size_t bytes, cudaStream_t st);
  void release();
  template <class T> T* as(size_t byte_offset = 0) const {
    return reinterpret_cast<T*>(static_cast<char*>(p) + byte_offset);
  }
};

// Fixed header at the start of the work buffer (zeroed before every pairwise launch).
struct WorkHeader {
  int counter;          // dynamic item counter
  unsigned meta[4];     // radius extrema (see P2PArgs::meta)
  int pad[3];
};
static_assert(sizeof(WorkHeader) == 32, "header layout");

// Checkpoints of a recorded forward time-stepping run (obs_advect_record_dev), kept for the
// backward op: ctx->tape holds r | s | checkpoints (nck x 2N floats).
struct AdvectTape {
  bool valid = false;
  int core = 0, accum = 0, order = 0, n = 0, nsteps = 0, every = 0, nck = 0;
  double fsx = 0.0, fsy = 0.0, dt = 0.0;
  bool full = false;   // every step's positions and stage positions kept (OBS_TAPE_ALL)
  bool last_seg = false;   // the last segment's positions and stage positions kept after the checkpoints
};

struct Timing {
  bool on = false;
  cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
  float main_ms = 0.0f;
  float call_ms = 0.0f;
  bool pending = false;
};

}  // namespace obs

struct obs_context {
  int device = 0;
  int num_sms = 0;
  cudaStream_t own_stream = nullptr;
  cudaStream_t stream = nullptr;
  obs::DevBuf work;      // header | packed sources | split partials | other scratch
  obs::DevBuf io;        // staging for host-pointer calls
  obs::DevBuf dense;     // BEM matrix (FP64) and its LU factors + pivots
  obs::DevBuf state;     // time stepping: stage velocities, segment positions, adjoint vectors
  obs::DevBuf tape;      // recorded forward run: radii, strengths, checkpoints
  obs::AdvectTape tape_info;
  int bem_n = 0;         // order of the BEM matrix held in `dense` (0: none)
  bool bem_lu = false;   // `dense` also holds its LU factorisation
  int* d_status = nullptr;   // device status block: DEV_ERR_* bits + first failure record
  int last_failure[4] = {0, 0, 0, 0};   // copy of the block at the last synchronize that saw one
  obs::Timing timing;
  long long launches = 0;
  int kernel_variant = 0;   // OBS_VARIANT_*
  int target_order = 0;     // OBS_ORDER_*
};

namespace obs {

// Map a CUDA error to an engine status (and clear the sticky last-error where possible).
int cuda_status(cudaError_t e);
// Bind the context's device on the calling thread.
int bind(obs_context* ctx);
// Read and clear the device error bits (synchronizes the stream).
int take_device_status(obs_context* ctx);
// runs a wait that nothing completes (which 0: mbarrier, 1: grid barrier) and returns the
// status the host reads afterwards (OBS_ERR_TIMEOUT when the bounded wait gave up as designed)
int selftest_bounded_wait(obs_context* ctx, int which, int max_polls);
// Event helpers around the main kernel of a call.
void timing_begin(obs_context* ctx);
void timing_main_begin(obs_context* ctx);
void timing_main_end(obs_context* ctx);
void timing_end(obs_context* ctx);

// One particle-on-particle request on device arrays (see obs_points_affect_points_dev).
struct P2PRequest {
  int core, result, accum, flags;
  double fsx, fsy;
  int ns;
  const float *sx, *sy, *sr, *ss;
  int nt;
  const float *tx, *ty, *tr;
  float *tu, *tv;
  float* extra[4];
};
int run_p2p(obs_context* ctx, const P2PRequest& rq);
double p2p_flops(int core, int result, bool thick, long long ns, long long nt);

// Launch helpers over the same kernels for callers that supply their own scratch.
struct P2PArgs;
cudaError_t p2p_launch_pack(const float* sx, const float* sy, const float* sr, const float* ss,
                            int ns, int ns_pad, int core, float4* out, unsigned* meta, cudaStream_t st);
cudaError_t p2p_launch_target_meta(const float* tr, int nt, unsigned* meta, cudaStream_t st);
cudaError_t p2p_dispatch_any(int core, bool thick, int res, bool comp, const P2PArgs* a, int grid,
                             cudaStream_t st, int* occ);
int p2p_ncomp(int res);

// packed-FP32 velocity kernels (p2p_packed.cu)
bool packed_supported(int core, int res);
// target pairs per thread of the packed velocity kernel for a core, OBS_VARIANT_* and target count
int packed_np(int core, int variant, int nt);
cudaError_t packed_dispatch(int core, int np, bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st,
                            int* occ);
// packed Gaussian kernels for the gradient, vorticity and shear results (p2p_packed_res.cu):
// target pairs per thread and the launcher
int packed_res_np(int res);
cudaError_t packed_res_dispatch(int res, bool thick, bool comp, const P2PArgs* a, int grid, cudaStream_t st,
                                int* occ);
cudaError_t packed_launch_pack(const float* sx, const float* sy, const float* sr, const float* ss, const int* perm,
                               int ns, int ns_pad, int core, float4* out, unsigned* meta, cudaStream_t st);
// Spatial (Morton) order of n points (bin_order.cu).  `scratch` holds bin_scratch_bytes(n)
// bytes, 256-aligned.  On return perm[k] is the caller's index of the k-th point in the order;
// the order is stable, so it depends on the input alone.  bin_gather writes x, y (and r, g when
// given) in that order.
size_t bin_scratch_bytes(int n);
cudaError_t bin_order(const float* x, const float* y, int n, void* scratch, int* perm, cudaStream_t st, int* launches);
cudaError_t bin_gather(const int* perm, const float* x, const float* y, const float* r, const float* g, int n,
                       float* bx, float* by, float* br, float* bg, cudaStream_t st, int* launches);

}  // namespace obs
