// tree.cu -- O(N log N) velocity of vortex particles: a treecode over Morton-ordered sources.
//
// The reference's execution environment names a Barnes-Hut summation (summation_t barneshut,
// src/ExecEnv.h:26-31) that it never runs internally; an external build reaches onbody's
// treecode through external_vel_solver_* (src/Influence.h:31-38, 74-98).  This is that
// summation on the GPU, for the velocity (results_t velonly) of every core:
//
//   * sources are put in Morton order (bin_order.cu); a leaf is a run of 32 consecutive sources
//     (one warp), a node at level L+1 groups 4 consecutive nodes of level L, up to one root;
//   * each node keeps its bounding box, a centre c (the box centre), a radius rho bounding
//     |z_j - c| over its sources, the largest radius term of its sources, and P multipole
//     coefficients b_k = sum_j G_j ((z_j - c)/rho)^k (complex; normalised by rho so that every
//     power lies in the unit disc) -- formed by warp reductions at the leaves and shifted up the
//     levels with the binomial theorem ((z - c')/rho' = s (z - c)/rho + t, |s| + |t| <= 1);
//   * one warp takes 32 Morton-consecutive targets and walks the tree with a warp-uniform stack:
//     a node is evaluated through its expansion,
//        sum_j G_j / (z - z_j) = (1/(z - c)) sum_k b_k w^k,   w = rho/(z - c),
//     when rho <= theta (|z - c| - r) for the warp's target box (r its half diagonal), so |w|
//     <= theta and the truncation after P terms is below theta^P/(1 - theta) of the node's
//     sum |G_j|/|z - z_j|; and only when every (target, source) pair of the node lies in the
//     core's far regime, where the core is 1/d^2: for the Gaussian and the compact exponential
//     that is the reference's own cut-off (d^2/s^2 > 16, (d/s)^3 > 16: the far branch IS 1/d^2,
//     src/CoreFunc.h:119-131), for the singular core always, and for Rosenhead-Moore,
//     Winckelmans-Leonard and the Vatistas cores where the core differs from 1/d^2 by less
//     than 2^-24 relative.  Other nodes open; at a leaf the pairs are summed directly with the
//     core (core_eval, as the direct kernels).
//
// With u + i v = i conj(F), F = sum_j G_j / (z - z_j): u = Im F, v = Re F (unscaled, as the
// direct sums; finalize_vels semantics optional).  Per-node contributions are accumulated with
// two-sums.  Results are deterministic: the traversal order is a function of the inputs.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {

namespace {

constexpr int TREE_LEAF = 32;        // sources per leaf: one warp
constexpr int TREE_FAN = 4;          // children per node
constexpr int TREE_PMAX = 32;        // coefficient stride per node (largest order)
constexpr int TREE_MAXLEV = 16;      // 32 * 4^15 sources
constexpr int TREE_WARPS = 4;        // warps per block (leaf, up and evaluation kernels)
constexpr int TREE_STACK = 96;       // > 1 + 3 * TREE_MAXLEV: the depth-first stack never overflows
constexpr int TREE_LEVBITS = 26;     // stack entry: level << 26 | index within the level
constexpr double kTreeInv2Pi = 0.15915494309189535;   // 0.5/pi, finalize_vels (src/ElementBase.h:216)

__constant__ float c_binom[TREE_PMAX][TREE_PMAX];

struct TreeNodes {
  float4* geo;       // (cx, cy, rho, zmax)
  float4* box;       // (xmin, ymin, xmax, ymax)
  float2* coef;      // [node][TREE_PMAX]
};

struct TreeArgs {
  const float4* sp4; // sources in Morton order: (x, y, radius term, strength)
  int ns;
  const float* tx;   // targets in Morton order (tr: radius, null for field points)
  const float* ty;
  const float* tr;
  const int* tperm;  // caller's index of the k-th sorted target
  int nt;
  float* tu;
  float* tv;
  TreeNodes nodes;
  int nlev;
  int lev_off[TREE_MAXLEV];
  int lev_cnt[TREE_MAXLEV];
  int P;
  float theta;
  int finalize;
  double fsx, fsy;
  int* status;
  const unsigned* meta;   // radius extrema: [2] ~min, [3] max of the sources; [4], [5] of the targets
};

__device__ __forceinline__ float warp_min(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_max(float v) {
  for (int o = 16; o > 0; o >>= 1) v = fmaxf(v, __shfl_xor_sync(0xffffffffu, v, o));
  return v;
}
__device__ __forceinline__ float warp_add(float v) {
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// leaves: one warp per 32 sorted sources; also packs each source as (x, y, radius term, G)
__global__ void __launch_bounds__(TREE_WARPS * 32) tree_leaf_kernel(const float* __restrict__ sx,
                                                                    const float* __restrict__ sy,
                                                                    const float* __restrict__ sr,
                                                                    const float* __restrict__ sg, int ns, int core,
                                                                    float4* __restrict__ sp4, TreeNodes nd, int nleaf,
                                                                    int P) {
  const int leaf = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (leaf >= nleaf) return;                        // warp-uniform
  const int i = leaf * TREE_LEAF + lane;
  const bool v = i < ns;
  const float inf = __int_as_float(0x7f800000);
  const float x = v ? sx[i] : 0.0f, y = v ? sy[i] : 0.0f;
  const float z = (v && sr) ? radius_term(core, sr[i]) : 0.0f;
  const float g = v ? sg[i] : 0.0f;
  if (v) sp4[i] = make_float4(x, y, z, g);
  const float x0 = warp_min(v ? x : inf), x1 = warp_max(v ? x : -inf);
  const float y0 = warp_min(v ? y : inf), y1 = warp_max(v ? y : -inf);
  const float zmax = warp_max(z);
  const float cx = 0.5f * (x0 + x1), cy = 0.5f * (y0 + y1);
  const float dx = x - cx, dy = y - cy;
  const float rho = warp_max(v ? sqrtf(dx * dx + dy * dy) : 0.0f);
  const float rn = rho > 0.0f ? rho : 1.0f;
  const float wr = v ? dx / rn : 0.0f, wi = v ? dy / rn : 0.0f;
  float pr = g, pi = 0.0f;                          // G w^k
  float2* cf = nd.coef + (size_t)leaf * TREE_PMAX;
  for (int k = 0; k < P; ++k) {
    const float sr_ = warp_add(pr), si_ = warp_add(pi);
    if (lane == 0) cf[k] = make_float2(sr_, si_);
    const float t = pr * wr - pi * wi;
    pi = pr * wi + pi * wr;
    pr = t;
  }
  if (lane == 0) {
    nd.geo[leaf] = make_float4(cx, cy, rho, zmax);
    nd.box[leaf] = make_float4(x0, y0, x1, y1);
  }
}

// one level up: one warp per parent (children 4q .. 4q+3 of the level below)
__global__ void __launch_bounds__(TREE_WARPS * 32) tree_up_kernel(TreeNodes nd, int off_c, int cnt_c, int off_p,
                                                                  int cnt_p, int P) {
  __shared__ float sp[TREE_WARPS][TREE_PMAX];
  __shared__ float2 tp[TREE_WARPS][TREE_PMAX];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int q = blockIdx.x * TREE_WARPS + w;
  if (q >= cnt_p) return;                           // warp-uniform
  const int c0 = q * TREE_FAN, c1 = min(c0 + TREE_FAN, cnt_c);
  float x0 = __int_as_float(0x7f800000), y0 = x0, x1 = -x0, y1 = -x0, zmax = 0.0f;
  for (int c = c0; c < c1; ++c) {
    const float4 b = nd.box[off_c + c];
    x0 = fminf(x0, b.x); y0 = fminf(y0, b.y); x1 = fmaxf(x1, b.z); y1 = fmaxf(y1, b.w);
    zmax = fmaxf(zmax, nd.geo[off_c + c].w);
  }
  const float cx = 0.5f * (x0 + x1), cy = 0.5f * (y0 + y1);
  float rho = 0.0f;
  for (int c = c0; c < c1; ++c) {
    const float4 gc = nd.geo[off_c + c];
    const float ex = gc.x - cx, ey = gc.y - cy;
    rho = fmaxf(rho, sqrtf(ex * ex + ey * ey) + gc.z);
  }
  const float rn = rho > 0.0f ? rho : 1.0f;
  float ar = 0.0f, ai = 0.0f;
  for (int c = c0; c < c1; ++c) {
    const float4 gc = nd.geo[off_c + c];
    const float rnc = gc.z > 0.0f ? gc.z : 1.0f;
    // (z - c)/rn = s (z - c_child)/rnc + t
    const float s = rnc / rn, tr = (gc.x - cx) / rn, ti = (gc.y - cy) / rn;
    float pws = 1.0f, pwr = 1.0f, pwi = 0.0f;
    for (int m = 0; m < lane; ++m) {                // lane m: s^m and t^m
      pws *= s;
      const float t = pwr * tr - pwi * ti;
      pwi = pwr * ti + pwi * tr;
      pwr = t;
    }
    sp[w][lane] = pws;
    tp[w][lane] = make_float2(pwr, pwi);
    __syncwarp();
    if (lane < P) {
      const float2* cf = nd.coef + (size_t)(off_c + c) * TREE_PMAX;
      for (int m = 0; m <= lane; ++m) {
        const float2 b = cf[m];
        const float2 t = tp[w][lane - m];
        const float f = c_binom[lane][m] * sp[w][m];
        ar += f * (b.x * t.x - b.y * t.y);
        ai += f * (b.x * t.y + b.y * t.x);
      }
    }
    __syncwarp();
  }
  const int node = off_p + q;
  if (lane < P) nd.coef[(size_t)node * TREE_PMAX + lane] = make_float2(ar, ai);
  if (lane == 0) {
    nd.geo[node] = make_float4(cx, cy, rho, zmax);
    nd.box[node] = make_float4(x0, y0, x1, y1);
  }
}

// Every (target, source) pair with squared distance >= d2 and radius terms summing to at most
// zsum lies where the core is 1/d^2: exactly (the reference's far branches of the Gaussian and
// compact exponential cores, the singular core), or within 2^-24 relative.
template <int CORE>
__device__ __forceinline__ bool tree_far(float d2, float zsum) {
  if constexpr (CORE == CORE_SING) return d2 > 0.0f;
  else if constexpr (CORE == CORE_GAUSS) return d2 > 0.0f && d2 > 16.05f * zsum;          // d^2/s^2 > 16
  else if constexpr (CORE == CORE_CEXP) return d2 > 0.0f && d2 > 6.36f * zsum;            // (d/s)^3 > 16
  else if constexpr (CORE == CORE_RM) return d2 > 0.0f && d2 > 16777216.0f * zsum;        // s^2/d^2 < 2^-24
  else if constexpr (CORE == CORE_WL) return d2 > 0.0f && d2 > 4096.0f * zsum;            // (s^2/d^2)^2 < 2^-24
  else if constexpr (CORE == CORE_V2) return d2 > 0.0f && d2 * d2 > 8388608.0f * zsum;    // s^4/(2 d^4) < 2^-24
  else return d2 > 0.0f && d2 * d2 * d2 > 8388608.0f * zsum;                              // s^6/(3 d^6) < 2^-24
}

template <int CORE, bool THICK>
__global__ void __launch_bounds__(TREE_WARPS * 32) tree_eval_kernel(const TreeArgs a) {
  __shared__ int stk[TREE_WARPS][TREE_STACK];
  __shared__ float4 leafs[TREE_WARPS][TREE_LEAF];
  const int w = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int wg = blockIdx.x * TREE_WARPS + w;
  if (wg * 32 >= a.nt) return;                      // warp-uniform
  const int i = wg * 32 + lane;
  const bool v = i < a.nt;
  const float inf = __int_as_float(0x7f800000);
  const float tx = v ? a.tx[i] : 0.0f, ty = v ? a.ty[i] : 0.0f;
  const float tz = (THICK && v) ? radius_term(CORE, a.tr[i]) : 0.0f;
  // Gaussian with one radius for every source (and every target): the near leaf sums take the
  // packed form below, with the core's cut-offs on t = -x log2(e), x = d^2 / s^2
  bool gunif = false;
  float gcf = 0.0f, gcfl = 0.0f;
  if constexpr (CORE == CORE_GAUSS) {
    gunif = (~a.meta[2] == a.meta[3]) && (!THICK || ~a.meta[4] == a.meta[5]);
    if (gunif) {
      const float us2 = radius_term(CORE, __uint_as_float(a.meta[3])) +
                        (THICK ? radius_term(CORE, __uint_as_float(a.meta[5])) : 0.0f);
      gcf = __frcp_rn(us2);
      gcfl = -gcf * kLog2e;
    }
  }
  const float bx0 = warp_min(v ? tx : inf), bx1 = warp_max(v ? tx : -inf);
  const float by0 = warp_min(v ? ty : inf), by1 = warp_max(v ? ty : -inf);
  const float ztmax = warp_max(tz);
  const float ctx_ = 0.5f * (bx0 + bx1), cty = 0.5f * (by0 + by1);
  const float rt = 0.5f * sqrtf((bx1 - bx0) * (bx1 - bx0) + (by1 - by0) * (by1 - by0));
  float hu = 0.0f, lu = 0.0f, hv = 0.0f, lv = 0.0f;
  const int top = a.nlev - 1;
  if (lane == 0)
    for (int q = 0; q < a.lev_cnt[top]; ++q) stk[w][q] = (top << TREE_LEVBITS) | q;
  int sp = a.lev_cnt[top];                          // 1 by construction
  __syncwarp();
  while (sp > 0) {
    const int e = stk[w][--sp];
    __syncwarp();
    const int lev = e >> TREE_LEVBITS, q = e & ((1 << TREE_LEVBITS) - 1);
    const int node = a.lev_off[lev] + q;
    const float4 gn = a.nodes.geo[node];
    const float4 bn = a.nodes.box[node];
    const float gx = fmaxf(0.0f, fmaxf(bn.x - bx1, bx0 - bn.z));
    const float gy = fmaxf(0.0f, fmaxf(bn.y - by1, by0 - bn.w));
    const float dmin2 = gx * gx + gy * gy;
    const float ex = gn.x - ctx_, ey = gn.y - cty;
    const float sep = sqrtf(ex * ex + ey * ey) - rt;
    const bool accept = sep > 0.0f && gn.z <= a.theta * sep && tree_far<CORE>(dmin2, gn.w + ztmax);
    if (accept) {
      // F = (1/(z - c)) sum_k b_k w^k, w = rn/(z - c); u += Im F, v += Re F
      const float2* cf = a.nodes.coef + (size_t)node * TREE_PMAX;
      const float rn = gn.z > 0.0f ? gn.z : 1.0f;
      const float dx = tx - gn.x, dy = ty - gn.y;
      const float inv = rcp_a(dx * dx + dy * dy);
      const float wr = rn * dx * inv, wi = -rn * dy * inv;
      float2 h = cf[a.P - 1];
      for (int k = a.P - 2; k >= 0; --k) {
        const float2 b = cf[k];
        const float t = fmaf(h.x, wr, fmaf(-h.y, wi, b.x));
        h.y = fmaf(h.x, wi, fmaf(h.y, wr, b.y));
        h.x = t;
      }
      const float fr = (dx * h.x + dy * h.y) * inv, fi = (dx * h.y - dy * h.x) * inv;
      if (v) {
        two_sum_acc(hu, lu, fi);
        two_sum_acc(hv, lv, fr);
      }
    } else if (lev == 0) {
      // direct sum over the leaf's sources (warp-broadcast loads): with the core, or -- when every
      // pair lies in the core's far regime, the leaf being too close for its expansion -- with
      // the far form 1/d^2 the core takes there.  Two sources per f32x2 operation: the leaf is
      // staged as pairs, ps[2 kp] = (-x, -x', -y, -y'), ps[2 kp + 1] = (z, z', -G, -G') for
      // sources 2 kp and 2 kp + 1 (one load per lane; padding past the leaf's end has G = 0)
      const int cnt = min(TREE_LEAF, a.ns - q * TREE_LEAF);
      __syncwarp();
      {
        const float4 p = a.sp4[q * TREE_LEAF + min(lane, cnt - 1)];
        float* st = reinterpret_cast<float*>(&leafs[w][0]) + (lane >> 1) * 8 + (lane & 1);
        st[0] = -p.x;
        st[2] = -p.y;
        st[4] = p.z;
        st[6] = (lane < cnt) ? -p.w : 0.0f;
      }
      __syncwarp();
      const float4* ps = leafs[w];
      const int np2 = (cnt + 1) >> 1;
      const float2 tx2 = f2(tx, tx), ty2 = f2(ty, ty);
      float2 au = f2(0.0f, 0.0f), av = f2(0.0f, 0.0f);   // sum -G K dy (= u), sum -G K dx (= -v)
      if (tree_far<CORE>(dmin2, gn.w + ztmax)) {
#pragma unroll 4
        for (int kp = 0; kp < np2; ++kp) {
          const float4 P = ps[2 * kp], Q = ps[2 * kp + 1];
          const float2 dx = __fadd2_rn(tx2, f2(P.x, P.y)), dy = __fadd2_rn(ty2, f2(P.z, P.w));
          const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
          const float2 fn = __fmul2_rn(f2(Q.z, Q.w), f2(rcp_a(d2.x), rcp_a(d2.y)));
          au = __ffma2_rn(fn, dy, au);
          av = __ffma2_rn(fn, dx, av);
        }
      } else if (CORE == CORE_GAUSS && gunif) {
        // (1 - e^-x)/d^2; x > 16 -> 1/d^2; x < 0.001 -> 1/s^2 (src/CoreFunc.h:111-181)
        const float thr_far = -16.0f * kLog2e, thr_small = -0.001f * kLog2e;
        const float2 cfl2 = f2(gcfl, gcfl), m1 = f2(-1.0f, -1.0f), one = f2(1.0f, 1.0f);
#pragma unroll 2
        for (int kp = 0; kp < np2; ++kp) {
          const float4 P = ps[2 * kp], Q = ps[2 * kp + 1];
          const float2 dx = __fadd2_rn(tx2, f2(P.x, P.y)), dy = __fadd2_rn(ty2, f2(P.z, P.w));
          const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
          const float2 t = __fmul2_rn(d2, cfl2);
          const float2 ood2 = f2(rcp_a(d2.x), rcp_a(d2.y));
          const float2 ome = __ffma2_rn(f2(ex2_a(t.x), ex2_a(t.y)), m1, one);
          float2 k = __fmul2_rn(ood2, ome);
          k.x = (t.x < thr_far) ? ood2.x : ((t.x > thr_small) ? gcf : k.x);
          k.y = (t.y < thr_far) ? ood2.y : ((t.y > thr_small) ? gcf : k.y);
          const float2 fn = __fmul2_rn(f2(Q.z, Q.w), k);
          au = __ffma2_rn(fn, dy, au);
          av = __ffma2_rn(fn, dx, av);
        }
      } else {
#pragma unroll 2
        for (int kp = 0; kp < np2; ++kp) {
          const float4 P = ps[2 * kp], Q = ps[2 * kp + 1];
          const float2 dx = __fadd2_rn(tx2, f2(P.x, P.y)), dy = __fadd2_rn(ty2, f2(P.z, P.w));
          const float2 d2 = __ffma2_rn(dx, dx, __fmul2_rn(dy, dy));
          float K0, K1, B;
          core_eval<CORE, THICK, false, false>(d2.x, Q.x, tz, 0.0f, 0.0f, K0, B);
          core_eval<CORE, THICK, false, false>(d2.y, Q.y, tz, 0.0f, 0.0f, K1, B);
          const float2 fn = __fmul2_rn(f2(Q.z, Q.w), f2(K0, K1));
          au = __ffma2_rn(fn, dy, au);
          av = __ffma2_rn(fn, dx, av);
        }
      }
      const float su = au.x + au.y, sv = -(av.x + av.y);
      if (v) {
        two_sum_acc(hu, lu, su);
        two_sum_acc(hv, lv, sv);
      }
    } else {
      const int c0 = q * TREE_FAN, c1 = min(c0 + TREE_FAN, a.lev_cnt[lev - 1]);
      if (sp + (c1 - c0) > TREE_STACK) {            // cannot happen (depth bound); recorded, not taken
        if (lane == 0) record_failure(a.status, DEV_ERR_BOUNDS, 1100, wg, sp);
        break;
      }
      if (lane == 0)
        for (int c = c1 - 1; c >= c0; --c) stk[w][sp + (c1 - 1 - c)] = ((lev - 1) << TREE_LEVBITS) | c;
      sp += c1 - c0;
      __syncwarp();
    }
  }
  if (!v) return;
  const int o = a.tperm ? a.tperm[i] : i;
  if ((unsigned)o >= (unsigned)a.nt) return;        // never taken: tperm is a permutation
  const double f = a.finalize ? kTreeInv2Pi : 1.0;
  const double su = (double)hu + (double)lu, sv = (double)hv + (double)lv;
  a.tu[o] = (float)(((double)a.tu[o] + su) * f + (a.finalize ? a.fsx : 0.0));
  a.tv[o] = (float)(((double)a.tv[o] + sv) * f + (a.finalize ? a.fsy : 0.0));
}

template <int CORE>
cudaError_t tree_eval_core(bool thick, const TreeArgs& a, int grid, cudaStream_t st) {
  if (thick) tree_eval_kernel<CORE, true><<<grid, TREE_WARPS * 32, 0, st>>>(a);
  else tree_eval_kernel<CORE, false><<<grid, TREE_WARPS * 32, 0, st>>>(a);
  return cudaGetLastError();
}

cudaError_t tree_eval(int core, bool thick, const TreeArgs& a, int grid, cudaStream_t st) {
  switch (core) {
    case CORE_RM: return tree_eval_core<CORE_RM>(thick, a, grid, st);
    case CORE_GAUSS: return tree_eval_core<CORE_GAUSS>(thick, a, grid, st);
    case CORE_V2: return tree_eval_core<CORE_V2>(thick, a, grid, st);
    case CORE_WL: return tree_eval_core<CORE_WL>(thick, a, grid, st);
    case CORE_V3: return tree_eval_core<CORE_V3>(thick, a, grid, st);
    case CORE_SING: return tree_eval_core<CORE_SING>(thick, a, grid, st);
    default: return tree_eval_core<CORE_CEXP>(thick, a, grid, st);
  }
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

// Device arrays in; accumulates into tu, tv (finalize_vels semantics with OBS_FLAG_FINALIZE).
int run_tree(obs_context* ctx, int core, int flags, double fsx, double fsy, double theta, int order, int ns,
             const float* sx, const float* sy, const float* sr, const float* ss, int nt, const float* tx,
             const float* ty, const float* tr, float* tu, float* tv) {
  if (ns == 0 || nt == 0) return OBS_OK;
  const int P = std::min(order, TREE_PMAX);
  // levels: leaves, then groups of four up to one root
  int lev_cnt[TREE_MAXLEV], lev_off[TREE_MAXLEV], nlev = 0, total = 0;
  int cnt = (ns + TREE_LEAF - 1) / TREE_LEAF;
  for (;;) {
    if (nlev == TREE_MAXLEV) return OBS_ERR_UNSUPPORTED;
    lev_cnt[nlev] = cnt;
    lev_off[nlev] = total;
    total += cnt;
    ++nlev;
    if (cnt == 1) break;
    cnt = (cnt + TREE_FAN - 1) / TREE_FAN;
  }
  const bool same = (tx == sx && ty == sy && tr == sr);
  const int nmax = std::max(ns, nt);
  const size_t S = (size_t)ns, T = (size_t)nt;
  const size_t o_bin = 0;
  const size_t o_sperm = o_bin + al256(bin_scratch_bytes(nmax));
  const size_t o_s = o_sperm + al256(S * 4);               // x y r g (4 S floats), then (x, y, z, g)
  const size_t o_p4 = o_s + 4 * al256(S * 4);
  const size_t o_tperm = o_p4 + al256(S * 16);
  const size_t o_t = o_tperm + al256(T * 4);               // x y r (3 T floats)
  const size_t o_geo = o_t + 3 * al256(T * 4);
  const size_t o_box = o_geo + al256((size_t)total * sizeof(float4));
  const size_t o_coef = o_box + al256((size_t)total * sizeof(float4));
  const size_t o_meta = o_coef + al256((size_t)total * TREE_PMAX * sizeof(float2));
  const size_t bytes = o_meta + 256;
  int s = ctx->work.ensure(bytes, ctx->stream);
  if (s) return s;
  char* W = ctx->work.as<char>();
  int* sperm = reinterpret_cast<int*>(W + o_sperm);
  float* bs[4];
  for (int k = 0; k < 4; ++k) bs[k] = reinterpret_cast<float*>(W + o_s + k * al256(S * 4));
  float4* sp4 = reinterpret_cast<float4*>(W + o_p4);
  int* tperm = reinterpret_cast<int*>(W + o_tperm);
  float* bt[3];
  for (int k = 0; k < 3; ++k) bt[k] = reinterpret_cast<float*>(W + o_t + k * al256(T * 4));
  TreeNodes nd{reinterpret_cast<float4*>(W + o_geo), reinterpret_cast<float4*>(W + o_box),
               reinterpret_cast<float2*>(W + o_coef)};
  cudaStream_t st = ctx->stream;
  // binomial coefficients for the upward shifts (exact in double, rounded once)
  float binom[TREE_PMAX][TREE_PMAX];
  for (int k = 0; k < TREE_PMAX; ++k) {
    double c = 1.0;
    for (int m = 0; m < TREE_PMAX; ++m) {
      binom[k][m] = m <= k ? (float)c : 0.0f;
      c = c * (double)(k - m) / (double)(m + 1);
    }
  }
  cudaError_t e = cudaMemcpyToSymbolAsync(c_binom, binom, sizeof(binom), 0, cudaMemcpyHostToDevice, st);
  int launches = 0;
  if (e == cudaSuccess) e = bin_order(sx, sy, ns, W + o_bin, sperm, st, &launches);
  if (e == cudaSuccess) e = bin_gather(sperm, sx, sy, sr, ss, ns, bs[0], bs[1], sr ? bs[2] : nullptr, bs[3], st,
                                       &launches);
  if (e != cudaSuccess) return cuda_status(e);
  const float *ttx = bs[0], *tty = bs[1], *ttr = tr ? bs[2] : nullptr;
  const int* tp = sperm;
  if (!same) {
    e = bin_order(tx, ty, nt, W + o_bin, tperm, st, &launches);
    if (e == cudaSuccess) e = bin_gather(tperm, tx, ty, tr, nullptr, nt, bt[0], bt[1], tr ? bt[2] : nullptr, nullptr, st,
                                         &launches);
    if (e != cudaSuccess) return cuda_status(e);
    ttx = bt[0]; tty = bt[1]; ttr = tr ? bt[2] : nullptr;
    tp = tperm;
  }
  const int tb = TREE_WARPS * 32;
  tree_leaf_kernel<<<(lev_cnt[0] + TREE_WARPS - 1) / TREE_WARPS, tb, 0, st>>>(bs[0], bs[1], sr ? bs[2] : nullptr, bs[3],
                                                                            ns, core, sp4, nd, lev_cnt[0], P);
  ++launches;
  for (int l = 0; l + 1 < nlev; ++l) {
    tree_up_kernel<<<(lev_cnt[l + 1] + TREE_WARPS - 1) / TREE_WARPS, tb, 0, st>>>(nd, lev_off[l], lev_cnt[l],
                                                                                lev_off[l + 1], lev_cnt[l + 1], P);
    ++launches;
  }
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_status(e);
  TreeArgs a;
  std::memset(&a, 0, sizeof(a));
  a.sp4 = sp4; a.ns = ns;
  a.tx = ttx; a.ty = tty; a.tr = ttr; a.tperm = tp; a.nt = nt;
  a.tu = tu; a.tv = tv;
  a.nodes = nd;
  a.nlev = nlev;
  for (int l = 0; l < nlev; ++l) { a.lev_off[l] = lev_off[l]; a.lev_cnt[l] = lev_cnt[l]; }
  a.P = P;
  a.theta = (float)theta;
  a.finalize = (flags & OBS_FLAG_FINALIZE) ? 1 : 0;
  a.fsx = fsx; a.fsy = fsy;
  a.status = ctx->d_status;
  // radius extrema for the Gaussian's uniform-radius leaf sums (zeroed: "not uniform")
  unsigned* meta = reinterpret_cast<unsigned*>(W + o_meta);
  if ((e = cudaMemsetAsync(meta, 0, 6 * sizeof(unsigned), st)) != cudaSuccess) return cuda_status(e);
  if (core == CORE_GAUSS && sr) {
    if ((e = p2p_launch_target_meta(sr, ns, meta, st)) != cudaSuccess) return cuda_status(e);
    ++launches;
    if (tr) {
      if ((e = p2p_launch_target_meta(tr, nt, meta + 2, st)) != cudaSuccess) return cuda_status(e);
      ++launches;
    }
  }
  a.meta = meta;
  const int nwarps = (nt + 31) / 32;
  e = tree_eval(core, tr != nullptr, a, (nwarps + TREE_WARPS - 1) / TREE_WARPS, st);
  ++launches;
  ctx->launches += launches;
  return cuda_status(e);
}

}  // namespace obs
