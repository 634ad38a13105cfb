// clear_inner.cu -- clear_inner_layer on the GPU (src/Reflect.h:733-760 over clear_inner_panp2,
// :491-729): the particles (or field points) that lie inside a body's cutoff layer are cropped
// with the cut tables or pushed onto the layer.
//
// Layout: one thread per point runs clear::clear_point (clear_inner.cuh) against every panel;
// all threads of a warp read the same panel at the same time, so the node and normal arrays
// are served as broadcasts from L1.  A one-thread prep kernel validates the node indices and
// forms the panel normals and node normals in panel order (the reference's summation order);
// the cut table (63 entries) is built on the host once.  The removed circulation is summed in
// FP64 in a fixed order by one block.  The same clear_inner.cuh compiles for the host, which
// the CPU tests use to check this logic against the oracle.
#include <cmath>
#include <cstring>
#include <vector>

#include "clear_inner.cuh"
#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {
namespace {

constexpr int kClearThreads = 256;
constexpr int kClearSumThreads = 1024;
constexpr int kMaxSweeps = 64;

// one thread: index check, panel normals and node normals in panel order (clear::normals)
__global__ void clear_prep_kernel(int nnodes, const float* __restrict__ nx, const float* __restrict__ ny, int npan,
                                  const unsigned* __restrict__ idx, float* pnx, float* pny, float* nnx, float* nny,
                                  int* bad, int* status) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int r = clear::normals(nnodes, nx, ny, npan, idx, pnx, pny, nnx, nny);
  if (r) record_failure(status, DEV_ERR_BOUNDS, 900, r - 1, 0);   // bad node index or zero-length panel
  *bad = r ? 1 : 0;
}

__global__ void __launch_bounds__(kClearThreads) clear_points_kernel(const clear::Geo g, const int* __restrict__ bad,
                                                                     int method, float cutoff_mult, float ips, int n,
                                                                     float* x, float* y, float* s,
                                                                     const float* __restrict__ r, double* lost,
                                                                     int* crops) {
  if (*bad) return;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  float xi = x[i], yi = y[i], si = s ? s[i] : 0.0f;
  const float rad = r ? r[i] : ips;
  double l = 0.0;
  const int c = clear::clear_point(g, method, cutoff_mult, ips, rad, xi, yi, si, l, kMaxSweeps);
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
  static bool table_ready = false;
  if (!table_ready) {
    clear::cut_table(table, table + clear::CUT_N, table + 2 * clear::CUT_N);
    table_ready = true;
  }
  const size_t off_pn = 0;
  const size_t off_nn = off_pn + al256((size_t)2 * npan * sizeof(float));
  const size_t off_ct = off_nn + al256((size_t)2 * nnodes * sizeof(float));
  const size_t off_lost = off_ct + al256(sizeof(table));
  const size_t off_crops = off_lost + al256((size_t)n * sizeof(double));
  const size_t off_out = off_crops + al256((size_t)n * sizeof(int));
  const size_t off_bad = off_out + al256(3 * sizeof(double));
  int st = ctx->work.ensure(off_bad + 256, ctx->stream);
  if (st) return st;
  float* pn = ctx->work.as<float>(off_pn);
  float* nn = ctx->work.as<float>(off_nn);
  float* ct = ctx->work.as<float>(off_ct);
  double* lost = ctx->work.as<double>(off_lost);
  int* crops = ctx->work.as<int>(off_crops);
  double* out = ctx->work.as<double>(off_out);
  int* bad = ctx->work.as<int>(off_bad);
  cudaStream_t strm = ctx->stream;
  cudaError_t e = cudaMemcpyAsync(ct, table, sizeof(table), cudaMemcpyHostToDevice, strm);
  if (e != cudaSuccess) return cuda_status(e);
  clear_prep_kernel<<<1, 1, 0, strm>>>(nnodes, nx, ny, npan, idx, pn, pn + npan, nn, nn + nnodes, bad, ctx->d_status);
  const clear::Geo g{nx, ny, idx, npan, pn, pn + npan, nn, nn + nnodes, ct, ct + clear::CUT_N,
                     ct + 2 * clear::CUT_N};
  clear_points_kernel<<<(n + kClearThreads - 1) / kClearThreads, kClearThreads, 0, strm>>>(
      g, bad, method, cutoff_mult, ips, n, x, y, s, r, lost, crops);
  clear_sum_kernel<<<1, kClearSumThreads, 0, strm>>>(bad, n, lost, crops, out);
  ctx->launches += 3;
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
