// adjoint.h -- host-side declarations for the VJP gathers and the time stepping.
#pragma once

#include "obs_context.h"

namespace obs {

// VJP gather (see adjoint.cu).  mode 0: owners are sources, elements are targets (er NULL for
// field points); mode 1: owners and elements are the same particles (self-interaction).
int run_adjoint(obs_context* ctx, int core, int accum, int mode,
                int no, const float* ox, const float* oy, const float* orad, const float* og,
                int ne, const float* ex, const float* ey, const float* er, const float* eg,
                const float* elu, const float* elv,
                float* gx, float* gy, float* gg, size_t off);

// Packed-FP32 variant for the Gaussian core (adjoint_packed.cu), same arguments and results;
// run_adjoint dispatches to it unless the generic kernels are forced.
bool adjoint_packed_supported(int core);
int run_adjoint_packed(obs_context* ctx, int accum, int mode, int no, const float* ox, const float* oy,
                       const float* orad, const float* og, int ne, const float* ex, const float* ey, const float* er,
                       const float* eg, const float* elu, const float* elv, float* gx, float* gy, float* gg,
                       size_t off);

// Euler (order 1) or Ralston RK2 (order 2) steps of the self-induced velocity, in place on
// device positions (Convection::advect_1st / advect_2nd_ralston, src/Convection.h:274-466).
int run_advect(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y,
               const float* r, const float* s, double fsx, double fsy, double dt, int nsteps);

// Schemes: 1 Euler, 2 Ralston RK2, 3 RK3, 4 Heun RK2 (src/Convection.h:274-598).
bool advect_order_ok(int order);
// run_advect that also records checkpoints every `every` steps into ctx->tape for
// run_advect_vjp_tape (0: ceil(sqrt(nsteps))).
int run_advect_record(obs_context* ctx, int core, int accum, int order, int n, float* x, float* y, const float* r,
                      const float* s, double fsx, double fsy, double dt, int nsteps, int every);
// Backward of the recorded run: dL/d(final positions) in (lx, ly); accumulates dL/ds and
// dL/d(initial positions).  The tape stays valid for further cotangents.
int run_advect_vjp_tape(obs_context* ctx, const float* lx, const float* ly, float* gs, float* gx0, float* gy0,
                        long long* peak_bytes);

// Reverse of run_advect from the initial positions: given dL/d(final positions), accumulate
// dL/ds and dL/d(initial positions); the trajectory is recomputed from checkpoints every
// `every` steps.  peak_bytes (optional) receives the engine's device memory high-water mark.
int run_advect_vjp(obs_context* ctx, int core, int accum, int order, int n, const float* x0, const float* y0,
                   const float* r, const float* s, double fsx, double fsy, double dt, int nsteps, int every,
                   const float* lx, const float* ly, float* gs, float* gx0, float* gy0, long long* peak_bytes);

}  // namespace obs
