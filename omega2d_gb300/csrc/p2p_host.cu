// p2p_host.cu -- launch planning for the particle-on-particle kernels (points_affect_points).
#include <algorithm>
#include <cstring>

#include "obs_context.h"
#include "p2p_dispatch.cuh"
#include "p2p_packed.cuh"

namespace obs {

namespace {

// Warp-reduce radius extrema (as bit patterns; radii are non-negative) and fold them into
// meta[k] = ~min, meta[k+1] = max with one atomic per warp.
__device__ __forceinline__ void fold_extrema(bool active, float r, unsigned* meta) {
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

// Pack the caller's SoA sources into float4 (x, y, radius term, strength), padded to whole
// tiles with zero-strength sources at the origin (radius term 1 keeps every core and every
// gradient form finite there, so 0 * K stays 0), and record the radius extrema in meta[0..1].
__global__ void pack_sources_kernel(const float* __restrict__ sx, const float* __restrict__ sy,
                                    const float* __restrict__ sr, const float* __restrict__ ss,
                                    int ns, int ns_pad, int core, float4* __restrict__ out,
                                    unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const float r = (i < ns && sr) ? sr[i] : 0.0f;
  if (i < ns) {
    out[i] = make_float4(sx[i], sy[i], radius_term(core, r), ss[i]);
  } else if (i < ns_pad) {
    out[i] = make_float4(0.0f, 0.0f, 1.0f, 0.0f);
  }
  fold_extrema(i < ns, r, meta);
}

__global__ void target_meta_kernel(const float* __restrict__ tr, int nt, unsigned* __restrict__ meta) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  fold_extrema(i < nt, i < nt ? tr[i] : 0.0f, meta + 2);
}

int ncomp_of(int res) {
  switch (res) {
    case RES_VEL: return 2;
    case RES_GRAD: return 5;
    case RES_PSI: return 1;
    case RES_BLOBVORT: return 1;
    default: return 3;
  }
}

cudaError_t dispatch(int core, bool thick, int res, bool comp, const P2PArgs* a, int grid,
                     cudaStream_t st, int* occ) {
  if (res == RES_PSI) return p2p_dispatch_psi(thick, comp, a, grid, st, occ);
  if (res == RES_BLOBVORT) return thick ? cudaErrorInvalidValue : p2p_dispatch_blobvort(comp, a, grid, st, occ);
  switch (core) {
    case CORE_RM: return p2p_dispatch<CORE_RM>(thick, res, comp, a, grid, st, occ);
    case CORE_GAUSS: return p2p_dispatch<CORE_GAUSS>(thick, res, comp, a, grid, st, occ);
    case CORE_V2: return p2p_dispatch<CORE_V2>(thick, res, comp, a, grid, st, occ);
    case CORE_WL: return p2p_dispatch<CORE_WL>(thick, res, comp, a, grid, st, occ);
    case CORE_V3: return p2p_dispatch<CORE_V3>(thick, res, comp, a, grid, st, occ);
    case CORE_SING: return p2p_dispatch<CORE_SING>(thick, res, comp, a, grid, st, occ);
    case CORE_CEXP: return p2p_dispatch<CORE_CEXP>(thick, res, comp, a, grid, st, occ);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

// Launch helpers for callers that manage their own scratch (the no-allocation entry point).
cudaError_t p2p_launch_pack(const float* sx, const float* sy, const float* sr, const float* ss,
                            int ns, int ns_pad, int core, float4* out, unsigned* meta, cudaStream_t st) {
  const int threads = 256;
  pack_sources_kernel<<<(ns_pad + threads - 1) / threads, threads, 0, st>>>(sx, sy, sr, ss, ns, ns_pad,
                                                                            core, out, meta);
  return cudaGetLastError();
}

cudaError_t p2p_launch_target_meta(const float* tr, int nt, unsigned* meta, cudaStream_t st) {
  const int threads = 256;
  target_meta_kernel<<<(nt + threads - 1) / threads, threads, 0, st>>>(tr, nt, meta);
  return cudaGetLastError();
}

cudaError_t p2p_dispatch_any(int core, bool thick, int res, bool comp, const P2PArgs* a, int grid,
                             cudaStream_t st, int* occ) {
  return dispatch(core, thick, res, comp, a, grid, st, occ);
}

int p2p_ncomp(int res) { return ncomp_of(res); }

// Reference flop counts: flopsu_0v_0b = 10 + flops_tv_nograds, flopsu_0v_0p = 10 +
// flops_tp_nograds, flopsug_0v_0b = 25 + flops_tv_grads, flopsuw = 19 + .._grads, flopsue = 23
// + .._grads, flopsp = 10 + .._nograds (src/Kernels.h:50-190; src/CoreFunc.h flops_*).
// Cores the reference lacks reuse the nearest reference form (singular: RM, compact exp:
// Gaussian); the field-point gradient uses the thick-target rule with the 0p core count.
double p2p_flops(int core, int result, bool thick, long long ns, long long nt) {
  //                       RM  GAUSS V2  WL  V3  SING CEXP
  static const int tvn[8] = {0, 5, 9, 9, 7, 12, 5, 9};
  static const int tpn[8] = {0, 3, 7, 6, 5, 8, 3, 7};
  static const int tvg[8] = {0, 9, 16, 13, 12, 16, 9, 16};
  static const int tpg[8] = {0, 9, 14, 10, 10, 12, 9, 14};
  if (core < 1 || core > 7) return -1.0;
  int per = 0, extra_per_target = 2;
  switch (result) {
    case RES_VEL: per = 10 + (thick ? tvn[core] : tpn[core]); break;
    case RES_GRAD: per = 25 + (thick ? tvg[core] : tpg[core]); break;
    case RES_PSI: per = 10 + (thick ? tvn[core] : tpn[core]); extra_per_target = 1; break;
    case RES_VORT: per = 19 + (thick ? tvg[core] : tpg[core]); extra_per_target = 3; break;
    case RES_SHEAR: per = 23 + (thick ? tvg[core] : tpg[core]); extra_per_target = 3; break;
    case RES_BLOBVORT: per = 13; extra_per_target = 1; break;   // src/InfluenceVort.h:112
    default: return -1.0;
  }
  return (double)nt * ((double)extra_per_target + (double)per * (double)ns);
}

int run_p2p(obs_context* ctx, const P2PRequest& rq) {
  const bool thick = rq.tr != nullptr;
  const bool comp = rq.accum == OBS_COMPENSATED;
  if (rq.ns == 0 || rq.nt == 0) return OBS_OK;
  const int res = rq.result;
  const int kcore = (res == RES_PSI) ? CORE_RM : rq.core;
  cudaStream_t st = ctx->stream;

  // ---- kernel choice: the packed-FP32 kernels serve velocity sums of every core and the
  // Gaussian gradient-type results
  const int variant = ctx->kernel_variant;
  const bool packed = variant != OBS_VARIANT_GENERIC && packed_supported(rq.core, res);
  // target pairs per thread: one table (packed_np) sizes the target blocks here and picks the
  // kernel instantiation in packed_dispatch
  const bool masked_core = rq.core == CORE_GAUSS || rq.core == CORE_CEXP;
  int np = packed_np(rq.core, variant, rq.nt);
  if (packed && res != RES_VEL) np = packed_res_np(res);
  auto launch = [&](const P2PArgs* args, int g, int* occ_out) -> cudaError_t {
    if (!packed) return dispatch(rq.core, thick, res, comp, args, g, st, occ_out);
    if (res != RES_VEL) return packed_res_dispatch(res, thick, comp, args, g, st, occ_out);
    return packed_dispatch(rq.core, np, thick, comp, args, g, st, occ_out);
  };

  // ---- plan the split
  int occ = 0;
  cudaError_t e = launch(nullptr, 0, &occ);
  if (e != cudaSuccess) return cuda_status(e);
  occ = std::max(occ, 1);
  const int slots = occ * ctx->num_sms;
  const int tb = P2P_THREADS * (packed ? 2 * np : p2p_tpt(res));
  const int ntb = (rq.nt + tb - 1) / tb;
  const int nst = (rq.ns + SRC_TILE - 1) / SRC_TILE;
  const int want_items = 24 * slots;
  int nsplit = std::max(1, (want_items + ntb - 1) / ntb);
  // at least two source tiles per split (20k sources: 39 splits, 0.156 ms per sum against
  // 0.165 ms with four tiles per split, which left a third of the CTA slots idle), and at most
  // 512 splits: few targets against many sources (10k probes, 500k sources) otherwise make
  // over a thousand splits whose partials and reduction chains cost more than they balance
  nsplit = std::min(nsplit, std::max(1, std::min(nst / 2, 512)));
  const int tps = (nst + nsplit - 1) / nsplit;
  nsplit = (nst + tps - 1) / tps;
  const int nitems = ntb * nsplit;
  const int grid = std::min(nitems, slots);
  const int nc = ncomp_of(res);
  // spatial (Morton) order lets the packed Gaussian and compact-exponential kernels skip the
  // exponential for far (warp, block) pairs
  const int order = ctx->target_order;
  const bool gauss_packed = packed && masked_core;
  // Morton order pays from ~3e8 pairs (uniform [-1,1]^2, s = 0.01, Gaussian / compact
  // exponential: 20k +2 % / +25 %, 33k +20 % / +56 %; 8k loses 28 % to the sort)
  const bool big = (double)rq.ns * rq.nt >= 3e8 && rq.nt >= 4096 && rq.ns >= 4096;
  const bool bin_t = gauss_packed && (order == OBS_ORDER_BINNED || order == OBS_ORDER_BINNED_TARGETS ||
                                      (order == OBS_ORDER_AUTO && big));
  const bool bin_s = gauss_packed && (order == OBS_ORDER_BINNED || (order == OBS_ORDER_AUTO && big));
  const bool same_pts = bin_t && bin_s && rq.sx == rq.tx && rq.sy == rq.ty && rq.ns == rq.nt;

  // the packed velocity kernel reduces its splits itself (P2PArgs::blkcnt: partial rows padded
  // to whole target blocks, one arrival count per block) when the partials would not stay in
  // L2 (over 64 MB): that is when the in-kernel reduction saves HBM traffic (1M targets: 274
  // -> 241 MB per launch); below it the separate reduction launch is as fast or faster (20k
  // targets: 0.166 vs 0.185 ms), and beyond 64 splits (few targets, many sources) the last
  // split of a block would sum a long chain on one CTA
  const size_t part_all = (size_t)nc * nsplit * rq.nt * (comp ? sizeof(double) : sizeof(float));
  const bool fused = packed && res == RES_VEL && nsplit > 1 && nsplit <= 64 && part_all > ((size_t)64 << 20);
  const size_t pst = fused ? (size_t)ntb * tb : (size_t)rq.nt;

  // ---- work buffer: header | block counts | packed sources | partials | target order
  //      (perm, x, y, r) | source order (perm) | sort scratch
  auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
  const size_t hdr = 256;
  const size_t cnt_bytes = fused ? al((size_t)ntb * sizeof(int)) : 0;
  const size_t src_bytes = (size_t)nst * SRC_TILE * sizeof(float4) * (packed ? PK_ELEM : 1);
  const size_t part_bytes = nsplit > 1 ? al((size_t)nc * nsplit * pst * (comp ? sizeof(double) : sizeof(float))) : 0;
  const size_t tvec = al((size_t)rq.nt * sizeof(float));
  const size_t svec = (bin_s && !same_pts) ? al((size_t)rq.ns * sizeof(int)) : 0;
  const size_t sort_bytes = (bin_t || bin_s) ? bin_scratch_bytes(std::max(bin_t ? rq.nt : 0, bin_s ? rq.ns : 0)) : 0;
  const size_t bin_bytes = (bin_t ? 4 * tvec : 0) + svec + sort_bytes;
  int s = ctx->work.ensure(hdr + cnt_bytes + src_bytes + part_bytes + bin_bytes, st);
  if (s) return s;
  WorkHeader* h = ctx->work.as<WorkHeader>(0);
  int* blkcnt = fused ? ctx->work.as<int>(hdr) : nullptr;
  float4* src = ctx->work.as<float4>(hdr + cnt_bytes);
  void* part = part_bytes ? ctx->work.as<char>(hdr + cnt_bytes + src_bytes) : nullptr;
  size_t off = hdr + cnt_bytes + src_bytes + part_bytes;
  int* tperm = nullptr;
  float *bx = nullptr, *by = nullptr, *br = nullptr;
  if (bin_t) {
    tperm = ctx->work.as<int>(off);
    bx = ctx->work.as<float>(off + tvec);
    by = ctx->work.as<float>(off + 2 * tvec);
    if (thick) br = ctx->work.as<float>(off + 3 * tvec);
    off += 4 * tvec;
  }
  int* sperm = nullptr;
  if (bin_s) {
    sperm = same_pts ? tperm : ctx->work.as<int>(off);
    off += svec;
  }
  void* sort_scratch = sort_bytes ? ctx->work.as<char>(off) : nullptr;

  timing_begin(ctx);
  e = cudaMemsetAsync(h, 0, fused ? hdr + cnt_bytes : sizeof(WorkHeader), st);
  if (e != cudaSuccess) return cuda_status(e);
  {
    int nl = 0;
    if (bin_t) {
      e = bin_order(rq.tx, rq.ty, rq.nt, sort_scratch, tperm, st, &nl);
      if (e == cudaSuccess) e = bin_gather(tperm, rq.tx, rq.ty, rq.tr, nullptr, rq.nt, bx, by, br, nullptr, st, &nl);
    }
    if (e == cudaSuccess && bin_s && !same_pts) e = bin_order(rq.sx, rq.sy, rq.ns, sort_scratch, sperm, st, &nl);
    ctx->launches += nl;
    if (e != cudaSuccess) return cuda_status(e);
  }
  {
    const int threads = 256;
    const int ns_pad = nst * SRC_TILE;
    if (packed) {
      e = packed_launch_pack(rq.sx, rq.sy, rq.sr, rq.ss, sperm, rq.ns, ns_pad, kcore, src, h->meta, st);
      if (e != cudaSuccess) return cuda_status(e);
    } else {
      pack_sources_kernel<<<(ns_pad + threads - 1) / threads, threads, 0, st>>>(
          rq.sx, rq.sy, rq.sr, rq.ss, rq.ns, ns_pad, kcore, src, h->meta);
    }
    ctx->launches++;
    if (thick) {
      target_meta_kernel<<<(rq.nt + threads - 1) / threads, threads, 0, st>>>(rq.tr, rq.nt, h->meta);
      ctx->launches++;
    }
    e = cudaGetLastError();
    if (e != cudaSuccess) return cuda_status(e);
  }

  P2PArgs a;
  std::memset(&a, 0, sizeof(a));
  a.src = src;
  a.nst = nst;
  a.tx = rq.tx; a.ty = rq.ty; a.tr = rq.tr;
  if (bin_t) {
    a.tx = bx; a.ty = by; a.tr = br;
    a.perm = tperm;
  }
  a.nt = rq.nt; a.ntb = ntb;
  a.nsplit = nsplit; a.tiles_per_split = tps; a.nitems = nitems;
  a.counter = &h->counter;
  a.meta = h->meta;
  a.status = ctx->d_status;
  a.out[0] = rq.tu; a.out[1] = rq.tv;
  for (int k = 0; k < 4; ++k) a.out[2 + k] = rq.extra[k];
  a.part = part;
  a.direct = nsplit == 1;
  a.finalize = (rq.flags & OBS_FLAG_FINALIZE) ? 1 : 0;
  a.fsx = rq.fsx; a.fsy = rq.fsy;
  a.blkcnt = blkcnt;

  timing_main_begin(ctx);
  e = launch(&a, grid, nullptr);
  ctx->launches++;
  timing_main_end(ctx);
  if (e != cudaSuccess) return cuda_status(e);
  if (nsplit > 1 && !fused) {
    e = p2p_reduce(res, comp, a, st);
    ctx->launches++;
    if (e != cudaSuccess) return cuda_status(e);
  }
  timing_end(ctx);
  return OBS_OK;
}

}  // namespace obs
