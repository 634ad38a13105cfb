// adjoint.cu -- hand-written reverse mode (VJP) of the particle velocity sums.
//
// The reference has no adjoint.  Forward map (finalized, src/Influence.h:56-416 +
// src/ElementBase.h:215-234):  u_i = fs + c sum_j G_j K(|d_ij|^2) J(d_ij),  d_ij = x_i - x_j,
// J(d) = (-dy, dx), c = 1/(2 pi).  With b = 2 dK/d(d^2) the pair Jacobian is
//   M(d) = d(K J)/dd = [[-b dx dy, -K - b dy^2], [K + b dx^2, b dx dy]]   (even in d),
// and for cotangents lam_i on u_i:
//   dL/dG_j  = c sum_i lam_i . K J(d_ij)
//   dL/dx_j -= c G_j sum_i M(d_ij)^T lam_i          (source side)
//   dL/dx_i += c (sum_j G_j M(d_ij))^T lam_i        (target side = velocity-gradient tensor)
// Two gather kernels:
//   ADJ_SRC  : one thread per source j, tiles of targets (x, y, radius term, lam) -- distinct
//              targets such as probes (0p) or a separate particle set (thick);
//   ADJ_SELF : targets are the sources; one pass per particle k over all j accumulates
//              c sum_j M(d_kj)^T (G_j lam_k - G_k lam_j)  and  -c sum_j lam_j . K J(d_kj),
//              so the core function is evaluated once per pair and no atomics are needed.
// Pipeline, work items, bounded waits and compensated accumulation follow p2p_kernel.cuh.
#include <algorithm>
#include <cstring>

#include "adjoint.h"
#include "obs_context.h"
#include "p2p_kernel.cuh"

namespace obs {

namespace {

constexpr int ADJ_THREADS = 128;
constexpr int ADJ_TILE = 256;                  // elements per stage
constexpr int ADJ_TPT = 2;                     // owners (sources / particles) per thread
constexpr int ADJ_NC = 3;                      // (gx, gy, gG)
constexpr uint32_t ADJ_TILE_BYTES = ADJ_TILE * 2 * sizeof(float4);

enum : int { ADJ_SRC = 0, ADJ_SELF = 1 };

struct AdjArgs {
  const float4* elem;    // 2 float4 per element: (x, y, z, G) | (lam_u, lam_v, 0, 0)
  int nst;               // element tiles
  const float* ox;       // owners (sources for ADJ_SRC, particles for ADJ_SELF)
  const float* oy;
  const float* orad;
  const float* og;
  const float* olu;      // ADJ_SELF: owners' cotangents
  const float* olv;
  int no;
  int nob;               // owner blocks
  int nsplit, tiles_per_split, nitems;
  int* counter;
  const unsigned* meta;
  int* status;
  float* gx;             // accumulated outputs
  float* gy;
  float* gg;
  void* part;
  int direct;
};

// fold radius extrema as in p2p_host.cu
__device__ __forceinline__ void fold_extrema2(bool active, float r, unsigned* meta) {
  unsigned rmin = active ? __float_as_uint(r) : ~0u;
  unsigned rmax = active ? __float_as_uint(r) : 0u;
  int any = active ? 1 : 0;
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

// elements: (x, y, radius term, G) | (lam_u, lam_v, 0, 0); padded with zero cotangent and zero
// strength at the origin with radius term 1 (finite for every core)
__global__ void pack_adj_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                const float* __restrict__ r, const float* __restrict__ g,
                                const float* __restrict__ lu, const float* __restrict__ lv,
                                int n, int n_pad, int core, float4* __restrict__ out, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float rr = (i < n && r) ? r[i] : 0.0f;
  if (i < n) {
    out[2 * i] = make_float4(x[i], y[i], r ? radius_term(core, rr) : 0.0f, g ? g[i] : 0.0f);
    out[2 * i + 1] = make_float4(lu[i], lv[i], 0.0f, 0.0f);
  } else if (i < n_pad) {
    out[2 * i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
    out[2 * i + 1] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
  }
  fold_extrema2(i < n && r != nullptr, rr, meta);
}

__global__ void owner_meta_kernel(const float* __restrict__ r, int n, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  fold_extrema2(i < n, i < n ? r[i] : 0.0f, meta + 2);
}

template <int CORE, int MODE, bool THICK, bool UNIF>
__device__ __forceinline__ void adj_tile(const float4* __restrict__ tile, const float (&ox)[ADJ_TPT],
                                         const float (&oy)[ADJ_TPT], const float (&oz)[ADJ_TPT],
                                         const float (&og)[ADJ_TPT], const float (&olu)[ADJ_TPT],
                                         const float (&olv)[ADJ_TPT], float us2, float ucf,
                                         float (&acc)[ADJ_TPT][ADJ_NC], float (&hi)[ADJ_TPT][ADJ_NC],
                                         float (&lo)[ADJ_TPT][ADJ_NC], bool comp) {
  for (int b = 0; b < ADJ_TILE / COMP_BLOCK; ++b) {
#pragma unroll 2
    for (int jj = 0; jj < COMP_BLOCK; ++jj) {
      const float4 e = tile[2 * (b * COMP_BLOCK + jj)];
      const float4 l = tile[2 * (b * COMP_BLOCK + jj) + 1];
#pragma unroll
      for (int k = 0; k < ADJ_TPT; ++k) {
        float K, B;
        if constexpr (MODE == ADJ_SRC) {
          // d = target - source (the element is the target)
          const float dx = e.x - ox[k], dy = e.y - oy[k];
          const float d2 = fmaf(dx, dx, dy * dy);
          core_eval<CORE, THICK, true, UNIF>(d2, oz[k], e.z, us2, ucf, K, B);
          acc[k][2] = fmaf(fmaf(l.y, dx, -l.x * dy), K, acc[k][2]);      // lam . K J(d)
          const float q = fmaf(dx, l.y, -dy * l.x);
          const float bq = B * q;
          acc[k][0] = acc[k][0] + fmaf(K, l.y, bq * dx);                 // (M^T lam)_x
          acc[k][1] = acc[k][1] + fmaf(-K, l.x, bq * dy);                // (M^T lam)_y
        } else {
          // d = owner - element (the owner is the target side)
          const float dx = ox[k] - e.x, dy = oy[k] - e.y;
          const float d2 = fmaf(dx, dx, dy * dy);
          core_eval<CORE, true, true, UNIF>(d2, e.z, oz[k], us2, ucf, K, B);
          const float wu = fmaf(e.w, olu[k], -og[k] * l.x);
          const float wv = fmaf(e.w, olv[k], -og[k] * l.y);
          const float q = fmaf(dx, wv, -dy * wu);
          const float bq = B * q;
          acc[k][0] = acc[k][0] + fmaf(K, wv, bq * dx);
          acc[k][1] = acc[k][1] + fmaf(-K, wu, bq * dy);
          acc[k][2] = fmaf(-fmaf(l.y, dx, -l.x * dy), K, acc[k][2]);
        }
      }
    }
    if (comp) {
#pragma unroll
      for (int k = 0; k < ADJ_TPT; ++k)
#pragma unroll
        for (int c = 0; c < ADJ_NC; ++c) {
          two_sum_acc(hi[k][c], lo[k][c], acc[k][c]);
          acc[k][c] = 0.0f;
        }
    }
  }
}

__device__ __forceinline__ void adj_store(const AdjArgs& a, int MODE, int i, const double (&c)[ADJ_NC]) {
  // scale by 1/(2 pi); source side of ADJ_SRC also by -G_j
  double sx = c[0] * kInv2Pi, sy = c[1] * kInv2Pi;
  const double sg = c[2] * kInv2Pi;
  if (MODE == ADJ_SRC) {
    const double gj = (double)a.og[i];
    sx *= -gj;
    sy *= -gj;
  }
  if (a.gx) a.gx[i] = (float)((double)a.gx[i] + sx);
  if (a.gy) a.gy[i] = (float)((double)a.gy[i] + sy);
  if (a.gg) a.gg[i] = (float)((double)a.gg[i] + sg);
}

template <int CORE, int MODE, bool THICK, bool COMP>
__global__ void __launch_bounds__(ADJ_THREADS) adj_kernel(const AdjArgs a) {
  constexpr int TB = ADJ_THREADS * ADJ_TPT;
  __shared__ __align__(128) float4 tile[NSTAGE][2 * ADJ_TILE];
  __shared__ __align__(8) uint64_t bar[NSTAGE];
  __shared__ int s_item;
  const int tid = threadIdx.x;
  if (tid == 0) {
    for (int s = 0; s < NSTAGE; ++s) mbar_init(&bar[s], 1);
    fence_mbar_init();
  }
  __syncthreads();
  // meta[0..1]: element radius extrema, meta[2..3]: owner radius extrema.  Field-point targets
  // (ADJ_SRC, !THICK) carry no radius: only the owners' (sources') radii enter the core.
  const bool thick_pair = (MODE == ADJ_SELF) || THICK;
  const bool owners_unif = (~a.meta[2] == a.meta[3]);
  const bool unif = thick_pair ? (owners_unif && ~a.meta[0] == a.meta[1]) : owners_unif;
  float us2 = 0.0f, ucf = 0.0f;
  if (unif) {
    us2 = radius_term(CORE, __uint_as_float(a.meta[3])) +
          (thick_pair ? radius_term(CORE, __uint_as_float(a.meta[1])) : 0.0f);
    ucf = __frcp_rn(us2);
  }
  uint32_t kt = 0;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(a.counter, 1);
    __syncthreads();
    const int item = *static_cast<volatile int*>(&s_item);
    if (item >= a.nitems) break;
    const int ob = item % a.nob;
    const int sp = item / a.nob;
    const int tile0 = sp * a.tiles_per_split;
    const int ntile = min(a.tiles_per_split, a.nst - tile0);
    if (tid == 0) {
      fence_proxy_async_smem();
      for (int s = 0; s < NSTAGE && s < ntile; ++s) {
        const int st = (kt + s) % NSTAGE;
        mbar_arrive_expect_tx(&bar[st], ADJ_TILE_BYTES);
        bulk_g2s(&tile[st][0], a.elem + (size_t)(tile0 + s) * 2 * ADJ_TILE, ADJ_TILE_BYTES, &bar[st]);
      }
    }
    float ox[ADJ_TPT], oy[ADJ_TPT], oz[ADJ_TPT], og[ADJ_TPT], olu[ADJ_TPT], olv[ADJ_TPT];
    float acc[ADJ_TPT][ADJ_NC], hi[ADJ_TPT][ADJ_NC], lo[ADJ_TPT][ADJ_NC];
#pragma unroll
    for (int k = 0; k < ADJ_TPT; ++k) {
      const int i = ob * TB + k * ADJ_THREADS + tid;
      const int ic = i < a.no ? i : a.no - 1;
      ox[k] = a.ox[ic];
      oy[k] = a.oy[ic];
      oz[k] = a.orad ? radius_term(CORE, a.orad[ic]) : 0.0f;
      og[k] = a.og ? a.og[ic] : 0.0f;
      olu[k] = MODE == ADJ_SELF ? a.olu[ic] : 0.0f;
      olv[k] = MODE == ADJ_SELF ? a.olv[ic] : 0.0f;
#pragma unroll
      for (int c = 0; c < ADJ_NC; ++c) { acc[k][c] = 0.0f; hi[k][c] = 0.0f; lo[k][c] = 0.0f; }
    }
    for (int t = 0; t < ntile; ++t, ++kt) {
      const int st = kt % NSTAGE;
      const bool ok = mbar_wait_bounded(&bar[st], (kt / NSTAGE) & 1u, WAIT_TRIES);
      if (__syncthreads_or(!ok)) {
        if (tid == 0) {
          record_failure(a.status, DEV_ERR_TIMEOUT, 500 + st, (int)kt, item);
          for (int s = 0; s < NSTAGE; ++s) (void)mbar_wait_bounded(&bar[(kt + s) % NSTAGE], ((kt + s) / NSTAGE) & 1u, WAIT_TRIES);
        }
        return;
      }
      if (unif)
        adj_tile<CORE, MODE, THICK, true>(&tile[st][0], ox, oy, oz, og, olu, olv, us2, ucf, acc, hi, lo, COMP);
      else
        adj_tile<CORE, MODE, THICK, false>(&tile[st][0], ox, oy, oz, og, olu, olv, us2, ucf, acc, hi, lo, COMP);
      __syncthreads();
      if (tid == 0 && t + NSTAGE < ntile) {
        fence_proxy_async_smem();
        mbar_arrive_expect_tx(&bar[st], ADJ_TILE_BYTES);
        bulk_g2s(&tile[st][0], a.elem + (size_t)(tile0 + t + NSTAGE) * 2 * ADJ_TILE, ADJ_TILE_BYTES, &bar[st]);
      }
    }
#pragma unroll
    for (int k = 0; k < ADJ_TPT; ++k) {
      const int i = ob * TB + k * ADJ_THREADS + tid;
      if (i >= a.no) continue;
      double c[ADJ_NC];
#pragma unroll
      for (int q = 0; q < ADJ_NC; ++q) c[q] = COMP ? ((double)hi[k][q] + (double)lo[k][q]) : (double)acc[k][q];
      if (a.direct) {
        adj_store(a, MODE, i, c);
      } else {
        double* p = static_cast<double*>(a.part);
#pragma unroll
        for (int q = 0; q < ADJ_NC; ++q) p[((size_t)q * a.nsplit + sp) * a.no + i] = c[q];
      }
    }
    __syncthreads();
  }
}

template <int MODE>
__global__ void adj_reduce_kernel(const AdjArgs a) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= a.no) return;
  double c[ADJ_NC];
  const double* p = static_cast<const double*>(a.part);
#pragma unroll
  for (int q = 0; q < ADJ_NC; ++q) {
    double s = 0.0;
    for (int k = 0; k < a.nsplit; ++k) s += p[((size_t)q * a.nsplit + k) * a.no + i];
    c[q] = s;
  }
  adj_store(a, MODE, i, c);
}

template <int CORE>
cudaError_t adj_dispatch(int mode, bool thick, bool comp, const AdjArgs* a, int grid, cudaStream_t st, int* occ) {
  auto run = [&](auto kern) -> cudaError_t {
    if (!a) return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, kern, ADJ_THREADS, 0);
    kern<<<grid, ADJ_THREADS, 0, st>>>(*a);
    return cudaGetLastError();
  };
  if (mode == ADJ_SELF)
    return comp ? run(adj_kernel<CORE, ADJ_SELF, true, true>) : run(adj_kernel<CORE, ADJ_SELF, true, false>);
  if (thick)
    return comp ? run(adj_kernel<CORE, ADJ_SRC, true, true>) : run(adj_kernel<CORE, ADJ_SRC, true, false>);
  return comp ? run(adj_kernel<CORE, ADJ_SRC, false, true>) : run(adj_kernel<CORE, ADJ_SRC, false, false>);
}

cudaError_t adj_dispatch_any(int core, int mode, bool thick, bool comp, const AdjArgs* a, int grid, cudaStream_t st,
                             int* occ) {
  switch (core) {
    case CORE_RM: return adj_dispatch<CORE_RM>(mode, thick, comp, a, grid, st, occ);
    case CORE_GAUSS: return adj_dispatch<CORE_GAUSS>(mode, thick, comp, a, grid, st, occ);
    case CORE_V2: return adj_dispatch<CORE_V2>(mode, thick, comp, a, grid, st, occ);
    case CORE_WL: return adj_dispatch<CORE_WL>(mode, thick, comp, a, grid, st, occ);
    case CORE_V3: return adj_dispatch<CORE_V3>(mode, thick, comp, a, grid, st, occ);
    case CORE_SING: return adj_dispatch<CORE_SING>(mode, thick, comp, a, grid, st, occ);
    case CORE_CEXP: return adj_dispatch<CORE_CEXP>(mode, thick, comp, a, grid, st, occ);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// One VJP gather.  mode ADJ_SRC: owners = sources (ox.. = sx, sy, sr, sg), elements = targets
// (ex, ey, er (NULL: field points), cotangents elu, elv); ADJ_SELF: owners = elements = the
// particles (ox = ex, ...), owner cotangents = element cotangents.  Work buffer from `off`.
int run_adjoint(obs_context* ctx, int core, int accum, int mode,
                int no, const float* ox, const float* oy, const float* orad, const float* og,
                int ne, const float* ex, const float* ey, const float* er, const float* eg,
                const float* elu, const float* elv,
                float* gx, float* gy, float* gg, size_t off) {
  if (no == 0 || ne == 0) return OBS_OK;
  if (ctx->kernel_variant != OBS_VARIANT_GENERIC && adjoint_packed_supported(core))
    return run_adjoint_packed(ctx, accum, mode, no, ox, oy, orad, og, ne, ex, ey, er, eg, elu, elv, gx, gy, gg, off);
  const bool comp = accum == OBS_COMPENSATED;
  const bool thick = (mode == ADJ_SELF) || er != nullptr;
  cudaStream_t st = ctx->stream;
  int occ = 0;
  cudaError_t e = adj_dispatch_any(core, mode, thick, comp, nullptr, 0, st, &occ);
  if (e != cudaSuccess) return cuda_status(e);
  occ = std::max(occ, 1);
  const int slots = occ * ctx->num_sms;
  const int tb = ADJ_THREADS * ADJ_TPT;
  const int nob = (no + tb - 1) / tb;
  const int nst = (ne + ADJ_TILE - 1) / ADJ_TILE;
  int nsplit = std::max(1, (24 * slots + nob - 1) / nob);
  nsplit = std::min(nsplit, std::max(1, nst / 4));
  const int tps = (nst + nsplit - 1) / nsplit;
  nsplit = (nst + tps - 1) / tps;
  const size_t hdr = 256;
  const size_t ebytes = (size_t)nst * ADJ_TILE * 2 * sizeof(float4);
  const size_t pbytes = nsplit > 1 ? (size_t)ADJ_NC * nsplit * no * sizeof(double) : 0;
  int s = ctx->work.ensure(off + hdr + ebytes + pbytes, st);
  if (s) return s;
  WorkHeader* h = ctx->work.as<WorkHeader>(off);
  float4* elem = ctx->work.as<float4>(off + hdr);
  e = cudaMemsetAsync(h, 0, sizeof(WorkHeader), st);
  if (e != cudaSuccess) return cuda_status(e);
  const int n_pad = nst * ADJ_TILE;
  pack_adj_kernel<<<(n_pad + 255) / 256, 256, 0, st>>>(ex, ey, er, eg, elu, elv, ne, n_pad, core, elem, h->meta);
  ctx->launches++;
  if (orad) {
    owner_meta_kernel<<<(no + 255) / 256, 256, 0, st>>>(orad, no, h->meta);
    ctx->launches++;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  AdjArgs a;
  std::memset(&a, 0, sizeof(a));
  a.elem = elem; a.nst = nst;
  a.ox = ox; a.oy = oy; a.orad = orad; a.og = og;
  a.olu = elu; a.olv = elv;   // ADJ_SELF: the owners are the elements
  a.no = no; a.nob = nob;
  a.nsplit = nsplit; a.tiles_per_split = tps; a.nitems = nob * nsplit;
  a.counter = &h->counter; a.meta = h->meta; a.status = ctx->d_status;
  a.gx = gx; a.gy = gy; a.gg = gg;
  a.part = pbytes ? ctx->work.as<char>(off + hdr + ebytes) : nullptr;
  a.direct = nsplit == 1;
  timing_main_begin(ctx);
  e = adj_dispatch_any(core, mode, thick, comp, &a, std::min(a.nitems, slots), st, nullptr);
  ctx->launches++;
  timing_main_end(ctx);
  if (e == cudaSuccess && nsplit > 1) {
    if (mode == ADJ_SELF) adj_reduce_kernel<ADJ_SELF><<<(no + 255) / 256, 256, 0, st>>>(a);
    else adj_reduce_kernel<ADJ_SRC><<<(no + 255) / 256, 256, 0, st>>>(a);
    ctx->launches++;
    e = cudaGetLastError();
  }
  return cuda_status(e);
}

}  // namespace obs
