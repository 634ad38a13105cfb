// clear_inner.cu -- clear_inner_layer on the GPU (src/Reflect.h:733-760 over clear_inner_panp2,
// :491-729): the particles (or field points) that lie inside a body's cutoff layer are cropped
// with the cut tables or pushed onto the layer.
//
// Layout: a parallel prep forms each panel's normal (Surfaces::compute_bases) and a 32-byte
// record (nodes, 1/length^2, normal) and sums the node normals; then one thread per point runs
// the per-point logic of clear_inner.cuh against panel tiles staged in shared memory (all
// threads of a block read the same panel record at the same time: a broadcast).  Each panel is
// bounded from below in FP32 (clear::seg_lower_bound) and evaluated exactly (the reference's
// float/double arithmetic) only when it may be the closest or tie it, so the common case costs
// two passes of about twenty FP32 operations per (point, panel) pair and no FP64.  The removed
// circulation is summed in FP64 in a fixed order by one block.  The same clear_inner.cuh
// compiles for the host, which the CPU tests use to check this logic against the oracle.  This
// file is compiled without fused multiply-adds (-fmad=false), like the oracle.
#include <cmath>
#include <cstring>
#include <mutex>
#include <vector>

#include "clear_inner.cuh"
#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {
namespace {

constexpr int kClearThreads = 256;
constexpr int kClearSumThreads = 1024;
constexpr int kMaxSweeps = 64;
constexpr int kClearTile = 1536;          // panels per shared-memory tile (48 KB of records)

// one thread per panel: index and length checks, the panel normal (clear::normals' formula),
// the panel's record for the point kernel, and the node normals (atomic sums; exact for nodes
// of one or two panels, since 0 + a + b rounds the same in either order)
__global__ void clear_panels_kernel(int nnodes, const float* __restrict__ nx, const float* __restrict__ ny, int npan,
                                    const unsigned* __restrict__ idx, float* pnx, float* pny, float4* geo,
                                    float4* nrm, float* nnx, float* nny, int* deg, int* first_bad) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= npan) return;
  const unsigned a = idx[2 * j], b = idx[2 * j + 1];
  if (a >= (unsigned)nnodes || b >= (unsigned)nnodes) {
    atomicMin(first_bad, j);
    return;
  }
  const float x0 = nx[a], y0 = ny[a], x1 = nx[b], y1 = ny[b];
  float tx = x1 - x0, ty = y1 - y0;
  const float blensq = tx * tx + ty * ty;
  const float base = sqrtf(blensq);
  if (!(base > 0.0f)) {
    atomicMin(first_bad, j);
    return;
  }
  tx = (float)((double)tx * (1.0 / (double)base));
  ty = (float)((double)ty * (1.0 / (double)base));
  pnx[j] = -ty;
  pny[j] = tx;
  geo[j] = make_float4(x0, y0, x1, y1);
  nrm[j] = make_float4(1.0f / blensq, -ty, tx, __uint_as_float(a));
  atomicAdd(&nnx[a], -ty); atomicAdd(&nny[a], tx);
  atomicAdd(&nnx[b], -ty); atomicAdd(&nny[b], tx);
  atomicAdd(&deg[a], 1);
  atomicAdd(&deg[b], 1);
}

// a node shared by three or more panels: its normal summed again in panel order (the
// reference's order, src/Reflect.h:521-533); also records a bad panel
__global__ void clear_nodes_kernel(int nnodes, int npan, const unsigned* __restrict__ idx, const float* __restrict__ pnx,
                                   const float* __restrict__ pny, float* nnx, float* nny, const int* __restrict__ deg,
                                   const int* __restrict__ first_bad, int* bad, int* status) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k == 0) {
    const int fb = *first_bad;
    *bad = fb < npan ? 1 : 0;
    if (fb < npan) record_failure(status, DEV_ERR_BOUNDS, 900, fb, 0);   // bad node index or zero-length panel
  }
  if (k >= nnodes || deg[k] <= 2 || *first_bad < npan) return;
  float sx = 0.0f, sy = 0.0f;
  for (int j = 0; j < npan; ++j) {
    const unsigned a = idx[2 * j], b = idx[2 * j + 1];
    if (a == (unsigned)k) { sx += pnx[j]; sy += pny[j]; }
    if (b == (unsigned)k) { sx += pnx[j]; sy += pny[j]; }
  }
  nnx[k] = sx;
  nny[k] = sy;
}

// One thread per point; the block sweeps until all its points pass.  Per sweep, the panel
// records stream through shared memory tile by tile (once for the whole kernel when one tile
// holds them) in two passes, as clear::clear_point does: the smallest lower bound names a
// candidate whose exact distance T bounds the minimum, then the panels whose bound does not
// exceed T are evaluated exactly (clear::closest_add) and the point is cropped or pushed
// (clear::clear_apply).
__global__ void __launch_bounds__(kClearThreads) clear_points_kernel(const clear::Geo g, const float4* __restrict__ geo,
                                                                     const float4* __restrict__ nrm,
                                                                     const int* __restrict__ bad, int method,
                                                                     float cutoff_mult, float ips, int n, float* x,
                                                                     float* y, float* s, const float* __restrict__ r,
                                                                     double* lost, int* crops) {
  __shared__ float4 tg[kClearTile];
  __shared__ float4 tn[kClearTile];
  if (*bad) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const bool mine = i < n;
  float xi = mine ? x[i] : 0.0f, yi = mine ? y[i] : 0.0f, si = (mine && s) ? s[i] : 0.0f;
  const float rad = (mine && r) ? r[i] : ips;
  double l = 0.0;
  int c = 0;
  bool active = mine;
  const int ntile = (g.npan + kClearTile - 1) / kClearTile;
  int loaded = -1;
  auto stage = [&](int t) {                   // uniform over the block
    if (loaded == t) return;
    __syncthreads();
    const int j0 = t * kClearTile, cnt = min(kClearTile, g.npan - j0);
    for (int k = threadIdx.x; k < cnt; k += blockDim.x) {
      tg[k] = geo[j0 + k];
      tn[k] = nrm[j0 + k];
    }
    __syncthreads();
    loaded = t;
  };
  while (__syncthreads_or(active)) {
    // pass 1: the candidate with the smallest lower bound
    float lbmin = 3.4028234663852886e38f;
    int jstar = -1;
    for (int t = 0; t < ntile; ++t) {
      stage(t);
      const int j0 = t * kClearTile, cnt = min(kClearTile, g.npan - j0);
      if (active)
        for (int k = 0; k < cnt; ++k) {
          const float4 pg = tg[k];
          const float lb = clear::seg_lower_bound(pg.x, pg.y, pg.z, pg.w, tn[k].x, xi, yi);
          if (lb < lbmin) { lbmin = lb; jstar = j0 + k; }
        }
    }
    float T = INFINITY;
    if (active && jstar >= 0) {
      const float4 pg = geo[jstar];
      float cx, cy;
      int kind, which;
      clear::seg_closest(pg.x, pg.y, pg.z, pg.w, xi, yi, T, cx, cy, kind, which);
    }
    // pass 2: exact evaluation of every panel that may be the closest or tie it
    clear::Closest cl;
    clear::closest_init(cl);
    for (int t = 0; t < ntile; ++t) {
      stage(t);
      const int cnt = min(kClearTile, g.npan - t * kClearTile);
      if (active)
        for (int k = 0; k < cnt; ++k) {
          const float4 pg = tg[k], pn = tn[k];
          if (clear::beyond(clear::seg_lower_bound(pg.x, pg.y, pg.z, pg.w, pn.x, xi, yi), T)) continue;
          const unsigned a = __float_as_uint(pn.w), b = g.idx[2 * (t * kClearTile + k) + 1];
          clear::closest_add(g, cl, a, b, pg.x, pg.y, pg.z, pg.w, pn.y, pn.z, xi, yi);
        }
    }
    if (active) {
      const int rc = clear::clear_apply(g, cl, method, cutoff_mult, ips, rad, xi, yi, si, l);
      if (rc == 1) {
        if (++c >= kMaxSweeps) {      // sweep limit: reported as no convergence
          c = -1;
          active = false;
        }
      } else {
        active = false;
      }
    }
  }
  if (!mine) return;
  x[i] = xi;
  y[i] = yi;
  if (s) s[i] = si;
  lost[i] = l;
  crops[i] = c;
}

// fixed-order sums: each thread a strided run, then a shared-memory tree
__global__ void __launch_bounds__(kClearSumThreads) clear_sum_kernel(const int* __restrict__ bad, int n,
                                                                     const double* __restrict__ lost,
                                                                     const int* __restrict__ crops, double* out) {
  __shared__ double sl[kClearSumThreads];
  __shared__ double sc[kClearSumThreads];
  __shared__ double sf[kClearSumThreads];
  const int t = threadIdx.x;
  double a = 0.0, c = 0.0, f = 0.0;
  if (!*bad) {
    for (int i = t; i < n; i += kClearSumThreads) {
      a += lost[i];
      if (crops[i] < 0) f += 1.0;
      else c += (double)crops[i];
    }
  }
  sl[t] = a; sc[t] = c; sf[t] = f;
  __syncthreads();
  for (int o = kClearSumThreads / 2; o > 0; o >>= 1) {
    if (t < o) { sl[t] += sl[t + o]; sc[t] += sc[t + o]; sf[t] += sf[t + o]; }
    __syncthreads();
  }
  if (t == 0) { out[0] = sl[0]; out[1] = sc[0]; out[2] = sf[0]; }
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

// Device arrays in, updated in place; results (circulation removed, modifications) to the host.
int run_clear_inner(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes, const float* nx,
                    const float* ny, int npan, const unsigned* idx, int n, float* x, float* y, float* s,
                    const float* r, double* circ_removed, long long* ncropped) {
  static float table[3 * clear::CUT_N];
  static std::once_flag table_once;       // callers on several host threads share the table
  std::call_once(table_once, [] { clear::cut_table(table, table + clear::CUT_N, table + 2 * clear::CUT_N); });
  const size_t P = (size_t)npan, M = (size_t)nnodes;
  const size_t off_pn = 0;
  const size_t off_geo = off_pn + al256(2 * P * sizeof(float));
  const size_t off_nrm = off_geo + al256(P * sizeof(float4));
  const size_t off_nn = off_nrm + al256(P * sizeof(float4));
  const size_t off_deg = off_nn + al256(2 * M * sizeof(float));
  const size_t off_ct = off_deg + al256(M * sizeof(int) + 256);
  const size_t off_lost = off_ct + al256(sizeof(table));
  const size_t off_crops = off_lost + al256((size_t)n * sizeof(double));
  const size_t off_out = off_crops + al256((size_t)n * sizeof(int));
  const size_t off_bad = off_out + al256(3 * sizeof(double));
  int st = ctx->work.ensure(off_bad + 256, ctx->stream);
  if (st) return st;
  float* pn = ctx->work.as<float>(off_pn);
  float4* geo = ctx->work.as<float4>(off_geo);
  float4* nrm = ctx->work.as<float4>(off_nrm);
  float* nn = ctx->work.as<float>(off_nn);
  int* deg = ctx->work.as<int>(off_deg);
  int* first_bad = deg + M;                     // in the same cleared run as the degrees
  float* ct = ctx->work.as<float>(off_ct);
  double* lost = ctx->work.as<double>(off_lost);
  int* crops = ctx->work.as<int>(off_crops);
  double* out = ctx->work.as<double>(off_out);
  int* bad = ctx->work.as<int>(off_bad);
  cudaStream_t strm = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(ct, table, sizeof(table), cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemsetAsync(nn, 0, 2 * M * sizeof(float), strm);
  if (e == cudaSuccess) e = cudaMemsetAsync(deg, 0, M * sizeof(int), strm);
  if (e == cudaSuccess) e = cudaMemsetAsync(first_bad, 0x7f, sizeof(int), strm);   // 0x7f7f7f7f: no bad panel
  if (e != cudaSuccess) return cuda_status(e);
  clear_panels_kernel<<<(npan + 255) / 256, 256, 0, strm>>>(nnodes, nx, ny, npan, idx, pn, pn + npan, geo, nrm, nn,
                                                            nn + nnodes, deg, first_bad);
  clear_nodes_kernel<<<(nnodes + 255) / 256, 256, 0, strm>>>(nnodes, npan, idx, pn, pn + npan, nn, nn + nnodes, deg,
                                                             first_bad, bad, ctx->d_status);
  const clear::Geo g{nx, ny, idx, npan, pn, pn + npan, nn, nn + nnodes, ct, ct + clear::CUT_N,
                     ct + 2 * clear::CUT_N};
  clear_points_kernel<<<(n + kClearThreads - 1) / kClearThreads, kClearThreads, 0, strm>>>(
      g, geo, nrm, bad, method, cutoff_mult, ips, n, x, y, s, r, lost, crops);
  clear_sum_kernel<<<1, kClearSumThreads, 0, strm>>>(bad, n, lost, crops, out);
  ctx->launches += 4;
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  double h[3] = {0.0, 0.0, 0.0};
  e = cudaMemcpyAsync(h, out, sizeof(h), cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
  if (e != cudaSuccess) return cuda_status(e);
  if ((st = take_device_status(ctx))) return st;
  if (circ_removed) *circ_removed = h[0];
  if (ncropped) *ncropped = (long long)h[1];
  return h[2] > 0.0 ? OBS_ERR_NO_CONVERGENCE : OBS_OK;
}

}  // namespace obs

namespace {

int check_clear(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes, const float* nx,
                const float* ny, int npan, const unsigned* idx, int n, const float* x, const float* y,
                const float* s, const float* r) {
  if (!ctx || (method != 0 && method != 1) || nnodes < 0 || npan < 0 || n < 0) return OBS_ERR_ARG;
  if (!(ips > 0.0f) || !std::isfinite(ips) || !std::isfinite(cutoff_mult)) return OBS_ERR_ARG;
  if (npan > 0 && (!nx || !ny || !idx || nnodes < 2)) return OBS_ERR_ARG;
  if (n > 0 && (!x || !y)) return OBS_ERR_ARG;
  if (method == 0 && n > 0 && (!s || !r)) return OBS_ERR_ARG;   // cropping needs particles
  return OBS_OK;
}

}  // namespace

extern "C" {

int obs_clear_inner_layer_dev(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes,
                              const float* nx, const float* ny, int npan, const unsigned* idx, int n, float* x,
                              float* y, float* s, const float* r, double* circ_removed, long long* ncropped) {
  int st = check_clear(ctx, method, cutoff_mult, ips, nnodes, nx, ny, npan, idx, n, x, y, s, r);
  if (st) return st;
  if (circ_removed) *circ_removed = 0.0;
  if (ncropped) *ncropped = 0;
  if (n == 0 || npan == 0) return OBS_OK;
  if ((st = obs::bind(ctx))) return st;
  return obs::run_clear_inner(ctx, method, cutoff_mult, ips, nnodes, nx, ny, npan, idx, n, x, y,
                              method == 0 ? s : nullptr, r, circ_removed, ncropped);
}

int obs_clear_inner_layer(obs_context* ctx, int method, float cutoff_mult, float ips, int nnodes, const float* nx,
                          const float* ny, int npan, const unsigned* idx, int n, float* x, float* y, float* s,
                          const float* r, double* circ_removed, long long* ncropped) {
  int st = check_clear(ctx, method, cutoff_mult, ips, nnodes, nx, ny, npan, idx, n, x, y, s, r);
  if (st) return st;
  if (circ_removed) *circ_removed = 0.0;
  if (ncropped) *ncropped = 0;
  if (n == 0 || npan == 0) return OBS_OK;
  for (size_t k = 0; k < 2 * (size_t)npan; ++k)
    if (idx[k] >= (unsigned)nnodes) return OBS_ERR_ARG;
  if ((st = obs::bind(ctx))) return st;
  const size_t N = (size_t)n, P = (size_t)npan, M = (size_t)nnodes;
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t o_nx = 0, o_ny = o_nx + al(M * 4), o_idx = o_ny + al(M * 4), o_x = o_idx + al(P * 8);
  const size_t o_y = o_x + al(N * 4), o_s = o_y + al(N * 4), o_r = o_s + al(N * 4), tot = o_r + al(N * 4);
  if ((st = ctx->io.ensure(tot, ctx->stream))) return st;
  float* dnx = ctx->io.as<float>(o_nx);
  float* dny = ctx->io.as<float>(o_ny);
  unsigned* didx = ctx->io.as<unsigned>(o_idx);
  float* dx = ctx->io.as<float>(o_x);
  float* dy = ctx->io.as<float>(o_y);
  float* ds = (method == 0) ? ctx->io.as<float>(o_s) : nullptr;
  float* dr = r ? ctx->io.as<float>(o_r) : nullptr;
  cudaStream_t strm = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(dnx, nx, M * 4, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dny, ny, M * 4, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(didx, idx, P * 8, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, x, N * 4, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, y, N * 4, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess && ds) e = cudaMemcpyAsync(ds, s, N * 4, cudaMemcpyHostToDevice, strm);
  if (e == cudaSuccess && dr) e = cudaMemcpyAsync(dr, r, N * 4, cudaMemcpyHostToDevice, strm);
  if (e != cudaSuccess) return obs::cuda_status(e);
  double circ = 0.0;
  long long nc = 0;
  st = obs::run_clear_inner(ctx, method, cutoff_mult, ips, nnodes, dnx, dny, npan, didx, n, dx, dy, ds, dr, &circ,
                            &nc);
  if (st && st != OBS_ERR_NO_CONVERGENCE) return st;
  // device -> temporaries -> caller, so a failed copy leaves the caller's arrays untouched
  std::vector<float> hx(N), hy(N), hs(ds ? N : 0);
  e = cudaMemcpyAsync(hx.data(), dx, N * 4, cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess) e = cudaMemcpyAsync(hy.data(), dy, N * 4, cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess && ds) e = cudaMemcpyAsync(hs.data(), ds, N * 4, cudaMemcpyDeviceToHost, strm);
  if (e == cudaSuccess) e = cudaStreamSynchronize(strm);
  if (e != cudaSuccess) return obs::cuda_status(e);
  std::memcpy(x, hx.data(), N * 4);
  std::memcpy(y, hy.data(), N * 4);
  if (ds) std::memcpy(s, hs.data(), N * 4);
  if (circ_removed) *circ_removed = circ;
  if (ncropped) *ncropped = nc;
  return st;
}

}  // extern "C"
