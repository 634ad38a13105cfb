// panels_pap.cu -- panels_affect_panels (src/Influence.h:774-795) on the device.
//
// The reference evaluates panel-on-panel velocities through temporary collocation points:
// Surfaces::represent_as_particles(1e-4, -1) (src/Surfaces.h:830-876) puts
// nshed_i = 1 + max(0, (int)(len_i / (1.2 len_0))) points on panel i at weights (1+2j)/(2 nshed_i)
// from node 0 to node 1, pushed 1e-4 along the panel normal into the fluid (the bases of
// compute_bases, src/Surfaces.h:682-724); panels_affect_points then runs on those points and
// the first npan point velocities are added to the npan panel velocities, index by index.
// Here one block builds the first npan points (a block-wide scan of the per-panel counts) and
// the panel kernel of panels.cu accumulates straight into the panel velocities.
#include "obs_context.h"
#include "obs_device.cuh"
#include "panels.h"

namespace obs {

namespace {

struct PanelGeom {
  float x0, y0, x1, y1, len, nx, ny;
};

__device__ __forceinline__ PanelGeom panel_geom(const float* __restrict__ nx, const float* __restrict__ ny,
                                                const unsigned* __restrict__ idx, int nnodes, int i, int* status) {
  unsigned i0 = idx[2 * i], i1 = idx[2 * i + 1];
  if (i0 >= (unsigned)nnodes || i1 >= (unsigned)nnodes) {
    record_failure(status, DEV_ERR_BOUNDS, 601, i, (int)(i0 >= (unsigned)nnodes ? i0 : i1));
    i0 = i1 = 0;
  }
  PanelGeom g;
  g.x0 = nx[i0]; g.y0 = ny[i0]; g.x1 = nx[i1]; g.y1 = ny[i1];
  float tx = g.x1 - g.x0, ty = g.y1 - g.y0;
  g.len = sqrtf(tx * tx + ty * ty);
  const double inv = 1.0 / (double)g.len;
  tx = (float)((double)tx * inv);
  ty = (float)((double)ty * inv);
  g.nx = -ty;   // normal into the fluid: left of node 0 -> node 1
  g.ny = tx;
  return g;
}

__device__ __forceinline__ long long shed_count(float len, float len0) {
  const double q = (double)len / (1.2 * (double)len0);
  const long long c = (q >= 1.0) ? (long long)fmin(q, 4.0e9) : 0;   // (int) truncation, clamped
  return 1 + c;
}

__global__ void __launch_bounds__(1024) collocation_kernel(const float* __restrict__ nx, const float* __restrict__ ny,
                                                           int nnodes, const unsigned* __restrict__ idx, int npan,
                                                           float* __restrict__ px, float* __restrict__ py,
                                                           int* status) {
  __shared__ long long wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (npan + 1023) / 1024;
  const int lo = min(npan, t * per), hi = min(npan, lo + per);
  const float len0 = panel_geom(nx, ny, idx, nnodes, 0, status).len;
  long long cnt = 0;
  for (int i = lo; i < hi; ++i) cnt += shed_count(panel_geom(nx, ny, idx, nnodes, i, status).len, len0);
  long long incl = cnt;
  for (int o = 1; o < 32; o <<= 1) {
    const long long q = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += q;
  }
  if (lane == 31) wsum[w] = incl;
  __syncthreads();
  if (w == 0) {
    long long x = wsum[lane];
    for (int o = 1; o < 32; o <<= 1) {
      const long long q = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += q;
    }
    wsum[lane] = x;
  }
  __syncthreads();
  long long m = incl - cnt + (w ? wsum[w - 1] : 0);
  const float off = 0.0001f;
  for (int i = lo; i < hi && m < npan; ++i) {
    const PanelGeom g = panel_geom(nx, ny, idx, nnodes, i, status);
    const long long ns = shed_count(g.len, len0);
    for (long long j = 0; j < ns && m < npan; ++j, ++m) {
      const float wt = (float)(1 + 2 * j) / (float)(2 * ns);
      px[m] = (float)((double)(wt * g.x1) + (1.0 - (double)wt) * (double)g.x0 + (double)(off * g.nx));
      py[m] = (float)((double)(wt * g.y1) + (1.0 - (double)wt) * (double)g.y0 + (double)(off * g.ny));
    }
  }
}

}  // namespace

int run_panels_affect_panels(obs_context* ctx, const PanelSet& src, const float* vs, const float* ss, int accum,
                             int flags, double fsx, double fsy, const PanelSet& targ, float* pu, float* pv) {
  if (src.npan == 0 || targ.npan == 0) return OBS_OK;
  const size_t T = (size_t)targ.npan;
  int s = ctx->state.ensure(2 * T * sizeof(float) + 256, ctx->stream);
  if (s) return s;
  float* px = ctx->state.as<float>();
  float* py = px + T;
  collocation_kernel<<<1, 1024, 0, ctx->stream>>>(targ.nx, targ.ny, targ.nnodes, targ.idx, targ.npan, px, py,
                                                  ctx->d_status);
  ctx->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  return run_panels_affect_points(ctx, src, vs, ss, accum, flags, fsx, fsy, targ.npan, px, py, pu, pv);
}

}  // namespace obs
