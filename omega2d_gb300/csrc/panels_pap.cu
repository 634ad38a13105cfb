// panels_pap.cu -- panels_affect_panels (src/Influence.h:774-795) on the device, and the
// rotation augmentation of the BEM self block that uses it (src/Coefficients.h:429-572).
//
// The reference evaluates panel-on-panel velocities through temporary collocation points:
// Surfaces::represent_as_particles(1e-4, -1) (src/Surfaces.h:830-876) puts
// nshed_i = 1 + max(0, (int)(len_i / (1.2 len_0))) points on panel i at weights (1+2j)/(2 nshed_i)
// from node 0 to node 1, pushed 1e-4 along the panel normal into the fluid (the bases of
// compute_bases, src/Surfaces.h:682-724); panels_affect_points then runs on those points and
// the first npan point velocities are added to the npan panel velocities, index by index.
// Here the first npan points are built on the device (per-panel counts, one scan, per-panel
// emission) and the panel kernel of panels.cu accumulates straight into the panel velocities.
#include <cmath>

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

// Collocation points in three grid-wide steps (FP64 runs slowly on this GPU, so each panel's
// FP64 divisions happen once, on many SMs): per-panel geometry and shed count; a one-block
// exclusive scan of the counts; per-panel emission of its points below index npan.
__global__ void shed_kernel(const float* __restrict__ nx, const float* __restrict__ ny, int nnodes,
                            const unsigned* __restrict__ idx, int npan, float4* __restrict__ geo,
                            float2* __restrict__ nrm, long long* __restrict__ cnt, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npan) return;
  const float len0 = panel_geom(nx, ny, idx, nnodes, 0, status).len;
  const PanelGeom g = panel_geom(nx, ny, idx, nnodes, i, status);
  geo[i] = make_float4(g.x0, g.y0, g.x1, g.y1);
  nrm[i] = make_float2(g.nx, g.ny);
  cnt[i] = shed_count(g.len, len0);
}

__global__ void __launch_bounds__(1024) shed_scan_kernel(const long long* __restrict__ cnt, int npan,
                                                         long long* __restrict__ off) {
  __shared__ long long wsum[32];
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  const int per = (npan + 1023) / 1024;
  const int lo = min(npan, t * per), hi = min(npan, lo + per);
  long long c = 0;
  for (int i = lo; i < hi; ++i) c += cnt[i];
  long long incl = c;
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
  long long m = incl - c + (w ? wsum[w - 1] : 0);
  for (int i = lo; i < hi; ++i) {
    off[i] = m;
    m += cnt[i];
  }
}

// nshed points per panel at weights (1+2j)/(2 nshed) from node 0, pushed 1e-4 along the normal
__global__ void emit_kernel(const float4* __restrict__ geo, const float2* __restrict__ nrm,
                            const long long* __restrict__ cnt, const long long* __restrict__ off, int npan,
                            float* __restrict__ px, float* __restrict__ py) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npan) return;
  long long m = off[i];
  const long long ns = cnt[i];
  if (m >= npan) return;
  const float4 g = geo[i];
  const float2 n = nrm[i];
  const float offd = 0.0001f;
  for (long long j = 0; j < ns && m < npan; ++j, ++m) {
    const float wt = (float)(1 + 2 * j) / (float)(2 * ns);
    px[m] = (float)((double)(wt * g.z) + (1.0 - (double)wt) * (double)g.x + (double)(offd * n.x));
    py[m] = (float)((double)(wt * g.w) + (1.0 - (double)wt) * (double)g.y + (double)(offd * n.y));
  }
}

// Surfaces::add_rot_strengths_base with unit rotation (src/Surfaces.h:566-605): per panel, the
// vortex and source strengths whose sheet reproduces solid-body rotation about (cx, cy)
__global__ void unit_rot_strengths_kernel(const float* __restrict__ nx, const float* __restrict__ ny, int nnodes,
                                          const unsigned* __restrict__ idx, int npan, float cx, float cy,
                                          float* __restrict__ vs, float* __restrict__ ss, int* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npan) return;
  const PanelGeom g = panel_geom(nx, ny, idx, nnodes, i, status);
  const float dx = (float)(0.5 * (double)(g.x0 + g.x1) - (double)cx);
  const float dy = (float)(0.5 * (double)(g.y0 + g.y1) - (double)cy);
  const float ui = -dy, vi = dx;
  const float oop = (float)(1.0 / (double)g.len);
  const float px = (g.x1 - g.x0) * oop, py = (g.y1 - g.y0) * oop;
  vs[i] = (float)(-1.0 * (double)(ui * px + vi * py));
  ss[i] = (float)(-1.0 * (double)(ui * py - vi * px));
}

// (n+1) x (n+1) column-major augmented block from the n x n block An (src/Coefficients.h:429-572):
// bottom row = panel lengths under the vortex unknowns, right column = the unit-rotation panel
// velocity along each target panel's tangent (and normal for the source unknowns), corner 2 vol
__global__ void augment_kernel(const double* __restrict__ An, int n, int nunk, const float* __restrict__ nx,
                               const float* __restrict__ ny, int nnodes, const unsigned* __restrict__ idx,
                               const float* __restrict__ pu, const float* __restrict__ pv, double vol,
                               double* __restrict__ Aa, int* status) {
  const int np1 = n + 1;
  const size_t total = (size_t)np1 * np1;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / np1), i = (int)(k % np1);
    double v;
    if (i < n && j < n) {
      v = An[(size_t)j * n + i];
    } else if (i == n && j < n) {
      const int pj = (nunk == 1) ? j : j / 2;
      v = (nunk == 1 || (j % 2) == 0) ? (double)panel_geom(nx, ny, idx, nnodes, pj, status).len : 0.0;
    } else if (j == n && i < n) {
      const int pi = (nunk == 1) ? i : i / 2;
      const PanelGeom g = panel_geom(nx, ny, idx, nnodes, pi, status);
      const float tx = g.ny, ty = -g.nx;   // tangent from the normal (n = (-t_y, t_x))
      const bool tang = (nunk == 1) || (i % 2) == 0;
      v = tang ? (double)(pu[pi] * tx + pv[pi] * ty) : (double)(pu[pi] * g.nx + pv[pi] * g.ny);
    } else {
      v = 2.0 * vol;
    }
    Aa[k] = v;
  }
}

}  // namespace

// state layout of panels_affect_panels: px, py (T floats each) | geo (T float4) | nrm (T float2)
// | cnt, off (T long long each)
size_t pap_scratch_bytes(int T) { return (size_t)T * (2 * 4 + 16 + 8 + 2 * 8) + 256; }

// Surfaces::set_geom_center (src/Surfaces.h:623-678) on the host: signed triangle areas from the
// origin accumulated in double; returns the enclosed area and its centroid
void geom_center_host(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, double* vol,
                      double* cx, double* cy) {
  double asum = 0.0, xsum = 0.0, ysum = 0.0;
  for (int i = 0; i < npan; ++i) {
    const unsigned j = idx[2 * i], jp1 = idx[2 * i + 1];
    if (j >= (unsigned)nnodes || jp1 >= (unsigned)nnodes) continue;
    const double xj = nx[j], yj = ny[j], xk = nx[jp1], yk = ny[jp1];
    const double xc = (0.0 + xj + xk) / 3.0, yc = (0.0 + yj + yk) / 3.0;
    const double px = xk - xj, py = yk - yj;
    const double a = std::sqrt(xj * xj + yj * yj), b = std::sqrt(px * px + py * py), c = std::sqrt(xk * xk + yk * yk);
    const double hs = 0.5 * (a + b + c);
    const double a2 = hs * (hs - a) * (hs - b) * (hs - c);
    double ar = a2 > 0.0 ? std::sqrt(a2) : 0.0;
    if (yj * px - xj * py < 0.0) ar = -ar;
    asum += ar;
    xsum += xc * ar;
    ysum += yc * ar;
  }
  *vol = (double)(float)asum;
  *cx = (double)(float)(xsum / asum);
  *cy = (double)(float)(ysum / asum);
}

int run_panels_on_panels_coeff_augmented(obs_context* ctx, const PanelSet& ps, int nunk, int accum, double vol,
                                         double cx, double cy, double* Aa) {
  const int n = ps.npan * nunk;
  const size_t N = (size_t)ps.npan;
  const size_t nn = (size_t)n * n;
  // state: the collocation scratch of panels_affect_panels | An (n^2 doubles) | unit strengths
  // vs, ss | induced pu, pv
  const size_t base = (pap_scratch_bytes(ps.npan) + 255) & ~(size_t)255;
  int s = ctx->state.ensure(base + nn * 8 + 4 * N * 4 + 1024, ctx->stream);
  if (s) return s;
  double* An = reinterpret_cast<double*>(ctx->state.as<char>() + base);
  float* vs = reinterpret_cast<float*>(An + nn);
  float* ss = vs + N;
  float* pu = ss + N;
  float* pv = pu + N;
  cudaStream_t st = ctx->stream;
  unit_rot_strengths_kernel<<<(ps.npan + 255) / 256, 256, 0, st>>>(ps.nx, ps.ny, ps.nnodes, ps.idx, ps.npan,
                                                                  (float)cx, (float)cy, vs, ss, ctx->d_status);
  ctx->launches++;
  cudaError_t e = cudaMemsetAsync(pu, 0, 2 * N * 4, st);
  if (e != cudaSuccess) return cuda_status(e);
  // the unit-rotation velocity at the body's own panels, finalized with zero freestream
  if ((s = run_panels_affect_panels(ctx, ps, vs, ss, accum, OBS_FLAG_FINALIZE, 0.0, 0.0, ps, pu, pv))) return s;
  if ((s = run_panels_on_panels_coeff(ctx, ps, ps, nunk, 1, nullptr, An))) return s;
  augment_kernel<<<2 * ctx->num_sms, 256, 0, st>>>(An, n, nunk, ps.nx, ps.ny, ps.nnodes, ps.idx, pu, pv, vol, Aa,
                                                   ctx->d_status);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

// Several bodies in one system, some of them rotating (the reference's block assembly,
// src/BEMHelper.h:166-221 with src/Coefficients.h:429-572 per block): the panel unknowns of the
// joined panel set first (An, nunk * npan), then one rotation unknown per augmented body a --
//   row a   : the panel lengths of body a in its vortex-strength columns, 0 in every other
//             panel column; 2 * area(a) on the diagonal, 0 for the other rotation columns;
//   column a: the velocity of body a's unit-rotation sheet at every panel of the joined set
//             (panels_affect_panels, finalized with zero freestream), along each panel's
//             tangent (and normal for the source unknowns).
__global__ void augment_bodies_kernel(const double* __restrict__ An, int np, int nunk, const float* __restrict__ nx,
                                      const float* __restrict__ ny, int nnodes, const unsigned* __restrict__ idx,
                                      int npan, const float* __restrict__ pu, const float* __restrict__ pv,
                                      const AugBodies ab, double* __restrict__ Aa, int* status) {
  const int n = np + ab.naug;
  const size_t total = (size_t)n * n;
  for (size_t k = (size_t)blockIdx.x * blockDim.x + threadIdx.x; k < total; k += (size_t)gridDim.x * blockDim.x) {
    const int j = (int)(k / n), i = (int)(k % n);
    double v;
    if (i < np && j < np) {
      v = An[(size_t)j * np + i];
    } else if (j < np) {
      const int a = i - np;
      const int pj = (nunk == 1) ? j : j / 2;
      const bool mine = pj >= ab.p0[a] && pj < ab.p1[a] && (nunk == 1 || (j % 2) == 0);
      v = mine ? (double)panel_geom(nx, ny, idx, nnodes, pj, status).len : 0.0;
    } else if (i < np) {
      const int a = j - np;
      const int pi = (nunk == 1) ? i : i / 2;
      const PanelGeom g = panel_geom(nx, ny, idx, nnodes, pi, status);
      const float tx = g.ny, ty = -g.nx;   // tangent from the normal (n = (-t_y, t_x))
      const bool tang = (nunk == 1) || (i % 2) == 0;
      const float u = pu[(size_t)a * npan + pi], w = pv[(size_t)a * npan + pi];
      v = tang ? (double)(u * tx + w * ty) : (double)(u * g.nx + w * g.ny);
    } else {
      v = (i == j) ? ab.vol2[i - np] : 0.0;
    }
    Aa[k] = v;
  }
}

int run_panels_on_panels_coeff_bodies_augmented(obs_context* ctx, const PanelSet& ps, int nunk, int accum,
                                                const AugBodies& ab, const float* cx, const float* cy,
                                                int nbodies, const int* panel_off, double* Aa) {
  const int np = ps.npan * nunk;
  const size_t N = (size_t)ps.npan;
  const size_t nn = (size_t)np * np;
  // state: the collocation scratch of panels_affect_panels | An (np^2 doubles) | unit strengths
  // vs, ss | induced pu, pv per augmented body
  const size_t base = (pap_scratch_bytes(ps.npan) + 255) & ~(size_t)255;
  int s = ctx->state.ensure(base + nn * 8 + (2 * N + 2 * N * (size_t)ab.naug) * 4 + 1024, ctx->stream);
  if (s) return s;
  double* An = reinterpret_cast<double*>(ctx->state.as<char>() + base);
  float* vs = reinterpret_cast<float*>(An + nn);
  float* ss = vs + N;
  float* pu = ss + N;
  float* pv = pu + N * ab.naug;
  cudaStream_t st = ctx->stream;
  cudaError_t e = cudaMemsetAsync(pu, 0, 2 * N * ab.naug * 4, st);
  if (e != cudaSuccess) return cuda_status(e);
  for (int a = 0; a < ab.naug; ++a) {
    const int nb = ab.p1[a] - ab.p0[a];
    const PanelSet body{ps.nnodes, ps.nx, ps.ny, nb, ps.idx + 2 * (size_t)ab.p0[a]};
    unit_rot_strengths_kernel<<<(nb + 255) / 256, 256, 0, st>>>(body.nx, body.ny, body.nnodes, body.idx, nb, cx[a],
                                                               cy[a], vs, ss, ctx->d_status);
    ctx->launches++;
    // the unit-rotation velocity of body a at every panel, finalized with zero freestream, one
    // target body at a time: a body's collocation points are spaced by its own first panel
    // (src/Surfaces.h:846-865 through src/Influence.h:783)
    for (int t = 0; t < nbodies; ++t) {
      const int q0 = panel_off[t], q1 = panel_off[t + 1];
      if (q1 <= q0) continue;
      const PanelSet targ{ps.nnodes, ps.nx, ps.ny, q1 - q0, ps.idx + 2 * (size_t)q0};
      if ((s = run_panels_affect_panels(ctx, body, vs, ss, accum, OBS_FLAG_FINALIZE, 0.0, 0.0, targ,
                                        pu + N * a + q0, pv + N * a + q0)))
        return s;
    }
  }
  if ((s = run_panels_on_panels_coeff(ctx, ps, ps, nunk, 1, nullptr, An))) return s;
  augment_bodies_kernel<<<2 * ctx->num_sms, 256, 0, st>>>(An, np, nunk, ps.nx, ps.ny, ps.nnodes, ps.idx, ps.npan, pu,
                                                          pv, ab, Aa, ctx->d_status);
  ctx->launches++;
  return cuda_status(cudaGetLastError());
}

int run_panels_affect_panels(obs_context* ctx, const PanelSet& src, const float* vs, const float* ss, int accum,
                             int flags, double fsx, double fsy, const PanelSet& targ, float* pu, float* pv) {
  if (src.npan == 0 || targ.npan == 0) return OBS_OK;
  const int T = targ.npan;
  int s = ctx->state.ensure(pap_scratch_bytes(T), ctx->stream);
  if (s) return s;
  float* px = ctx->state.as<float>();
  float* py = px + T;
  float4* geo = reinterpret_cast<float4*>(ctx->state.as<char>() + (((size_t)T * 8 + 15) & ~(size_t)15));
  float2* nrm = reinterpret_cast<float2*>(geo + T);
  long long* cnt = reinterpret_cast<long long*>(nrm + T);
  long long* off = cnt + T;
  const int nb = (T + 255) / 256;
  shed_kernel<<<nb, 256, 0, ctx->stream>>>(targ.nx, targ.ny, targ.nnodes, targ.idx, T, geo, nrm, cnt, ctx->d_status);
  shed_scan_kernel<<<1, 1024, 0, ctx->stream>>>(cnt, T, off);
  emit_kernel<<<nb, 256, 0, ctx->stream>>>(geo, nrm, cnt, off, T, px, py);
  ctx->launches += 3;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return cuda_status(e);
  return run_panels_affect_points(ctx, src, vs, ss, accum, flags, fsx, fsy, T, px, py, pu, pv);
}

}  // namespace obs
