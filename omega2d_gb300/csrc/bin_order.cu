// bin_order.cu -- spatial (Morton) order of a point set on the device.
//
// The packed Gaussian kernel is fastest when the targets of one warp lie close together and
// the 32 sources of one block lie close together: then most (warp, block) pairs are farther
// apart than 4 core radii and take the reference's far-field form G/d^2 without an
// exponential.  This file produces that order:
//   1. bounding box of the points (order-preserving float keys, atomic max);
//   2. 16-bit Morton key of each point's cell in a 256 x 256 grid over the box;
//   3. stable LSD radix sort of (key, index) in two 8-bit passes: per-tile digit counts (and
//      digit totals), per-digit offsets over the tiles (one warp per digit), and a stable
//      scatter whose in-tile ranks
//      come from warp match + per-warp digit counts, so the order is a function of the input
//      alone (points of one cell keep the caller's relative order);
//   4. optional gather of x, y, r, g into the sorted order.
// Everything runs on the caller's stream; nothing is synchronized.
#include "obs_context.h"
#include "obs_device.cuh"

namespace obs {

namespace {

constexpr int BIN_BITS = 8;                       // cells per axis: 256
constexpr int RS_THREADS = 256;                   // = number of digits per pass
constexpr int RS_CHUNKS = 4;
constexpr int RS_TILE = RS_THREADS * RS_CHUNKS;   // points per radix tile
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int HDR_BYTES = 4096;                   // bb | digit totals of pass 1 | of pass 2

// order-preserving map of a float to an unsigned key (and back)
__device__ __forceinline__ unsigned ord_key(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord_val(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7fffffffu) : ~k);
}

// bb[0] = ~min key x, bb[1] = max key x, bb[2] = ~min key y, bb[3] = max key y (zeroed first);
// one set of atomics per block
__global__ void __launch_bounds__(256) bin_bbox_kernel(const float* __restrict__ x, const float* __restrict__ y,
                                                       int n, unsigned* __restrict__ bb) {
  __shared__ unsigned red[4][8];
  unsigned v[4] = {0u, 0u, 0u, 0u};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const unsigned kx = ord_key(x[i]), ky = ord_key(y[i]);
    v[0] = max(v[0], ~kx); v[1] = max(v[1], kx);
    v[2] = max(v[2], ~ky); v[3] = max(v[3], ky);
  }
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
  for (int c = 0; c < 4; ++c) {
    for (int o = 16; o > 0; o >>= 1) v[c] = max(v[c], __shfl_xor_sync(0xffffffffu, v[c], o));
    if (lane == 0) red[c][w] = v[c];
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    unsigned m = 0u;
    for (int q = 0; q < 8; ++q) m = max(m, red[threadIdx.x][q]);
    atomicMax(&bb[threadIdx.x], m);
  }
}

__device__ __forceinline__ unsigned spread8(unsigned v) {
  v = (v | (v << 4)) & 0x0F0Fu;
  v = (v | (v << 2)) & 0x3333u;
  v = (v | (v << 1)) & 0x5555u;
  return v;
}

__device__ __forceinline__ unsigned cell_of(float v, float lo, float scale) {
  const float c = fminf(fmaxf((v - lo) * scale, 0.0f), (float)((1 << BIN_BITS) - 1));   // NaN -> 0
  return (unsigned)c;
}

__global__ void bin_key_kernel(const float* __restrict__ x, const float* __restrict__ y, int n,
                               const unsigned* __restrict__ bb, unsigned* __restrict__ keys) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float x0 = ord_val(~bb[0]), x1 = ord_val(bb[1]);
  const float y0 = ord_val(~bb[2]), y1 = ord_val(bb[3]);
  const float wx = x1 - x0, wy = y1 - y0;
  const float sx = (wx > 0.0f) ? (float)(1 << BIN_BITS) / wx : 0.0f;
  const float sy = (wy > 0.0f) ? (float)(1 << BIN_BITS) / wy : 0.0f;
  keys[i] = spread8(cell_of(x[i], x0, sx)) | (spread8(cell_of(y[i], y0, sy)) << 1);
}

// digit counts of one tile: table[digit * ntiles + tile]; digit totals into tot[256] (zeroed)
__global__ void __launch_bounds__(RS_THREADS) rs_count_kernel(const unsigned* __restrict__ keys, int n, int shift,
                                                             unsigned* __restrict__ table, int ntiles,
                                                             unsigned* __restrict__ tot) {
  __shared__ unsigned cnt[RS_THREADS];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const int base = blockIdx.x * RS_TILE;
#pragma unroll
  for (int k = 0; k < RS_CHUNKS; ++k) {
    const int i = base + k * RS_THREADS + threadIdx.x;
    if (i < n) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  }
  __syncthreads();
  const unsigned c = cnt[threadIdx.x];
  table[(size_t)threadIdx.x * ntiles + blockIdx.x] = c;
  if (c) atomicAdd(&tot[threadIdx.x], c);
}

// exclusive offsets in place: table[d][t] <- sum of all counts of digits < d + counts of digit d
// in tiles < t.  One warp per digit; the row is scanned 32 tiles at a time (coalesced).
__global__ void __launch_bounds__(256) rs_offsets_kernel(unsigned* __restrict__ table, int ntiles,
                                                         const unsigned* __restrict__ tot) {
  const int lane = threadIdx.x & 31;
  const int d = blockIdx.x * 8 + (threadIdx.x >> 5);
  if (d >= RS_THREADS) return;
  unsigned base = 0;
  for (int q = lane; q < d; q += 32) base += tot[q];
  for (int o = 16; o > 0; o >>= 1) base += __shfl_xor_sync(0xffffffffu, base, o);
  unsigned* row = table + (size_t)d * ntiles;
  for (int t0 = 0; t0 < ntiles; t0 += 32) {
    const int t = t0 + lane;
    const unsigned c = (t < ntiles) ? row[t] : 0u;
    unsigned incl = c;
    for (int o = 1; o < 32; o <<= 1) {
      const unsigned q = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += q;
    }
    if (t < ntiles) row[t] = base + incl - c;
    base += __shfl_sync(0xffffffffu, incl, 31);
  }
}

// stable scatter of one tile; vin == nullptr means the identity payload (the point's index)
__global__ void __launch_bounds__(RS_THREADS) rs_scatter_kernel(const unsigned* __restrict__ kin,
                                                               const int* __restrict__ vin, int n, int shift,
                                                               const unsigned* __restrict__ table, int ntiles,
                                                               unsigned* __restrict__ kout, int* __restrict__ vout) {
  __shared__ unsigned run[RS_THREADS];            // next output slot per digit for this tile
  __shared__ unsigned wcnt[RS_WARPS][RS_THREADS]; // per-warp counts of the chunk, then their prefix
  const int t = threadIdx.x, lane = t & 31, w = t >> 5;
  run[t] = table[(size_t)t * ntiles + blockIdx.x];
  const int base = blockIdx.x * RS_TILE;
  for (int k = 0; k < RS_CHUNKS; ++k) {
#pragma unroll
    for (int q = 0; q < RS_WARPS; ++q) wcnt[q][t] = 0;
    __syncthreads();
    const int i = base + k * RS_THREADS + t;
    const bool valid = i < n;
    const unsigned key = valid ? kin[i] : 0u;
    const int val = valid ? (vin ? vin[i] : i) : 0;
    const unsigned d = (key >> shift) & 255u;
    const unsigned peers = __match_any_sync(0xffffffffu, valid ? d : 0x100u);
    const unsigned below = peers & ((1u << lane) - 1u);
    if (valid && below == 0u) wcnt[w][d] = __popc(peers);
    __syncthreads();
    unsigned acc = 0;                              // thread t: prefix over warps of digit t
#pragma unroll
    for (int q = 0; q < RS_WARPS; ++q) {
      const unsigned c = wcnt[q][t];
      wcnt[q][t] = acc;
      acc += c;
    }
    __syncthreads();
    if (valid) {
      const unsigned pos = run[d] + wcnt[w][d] + (unsigned)__popc(below);
      if (pos < (unsigned)n) {                     // always true: the counts sum to n
        kout[pos] = key;
        vout[pos] = val;
      }
    }
    __syncthreads();
    run[t] += acc;
  }
}

__global__ void bin_gather_kernel(const int* __restrict__ perm, const float* __restrict__ x,
                                  const float* __restrict__ y, const float* __restrict__ r,
                                  const float* __restrict__ g, int n, float* __restrict__ bx,
                                  float* __restrict__ by, float* __restrict__ br, float* __restrict__ bg) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= n) return;
  int i = perm[k];
  if ((unsigned)i >= (unsigned)n) i = k;          // never taken: perm is a permutation of 0..n-1
  bx[k] = x[i];
  by[k] = y[i];
  if (r) br[k] = r[i];
  if (g) bg[k] = g[i];
}

size_t al256(size_t b) { return (b + 255) & ~(size_t)255; }

}  // namespace

// scratch: header (bb, digit totals) | table[256][ntiles] | keys A | keys B | payload B
size_t bin_scratch_bytes(int n) {
  const size_t ntiles = ((size_t)n + RS_TILE - 1) / RS_TILE;
  return HDR_BYTES + al256(RS_THREADS * ntiles * sizeof(unsigned)) + 3 * al256((size_t)n * sizeof(unsigned));
}

cudaError_t bin_order(const float* x, const float* y, int n, void* scratch, int* perm, cudaStream_t st,
                      int* launches) {
  if (n <= 0) return cudaSuccess;
  const int ntiles = (n + RS_TILE - 1) / RS_TILE;
  char* p = static_cast<char*>(scratch);
  unsigned* bb = reinterpret_cast<unsigned*>(p);
  unsigned* tot0 = reinterpret_cast<unsigned*>(p + 256);
  unsigned* tot1 = tot0 + RS_THREADS;
  unsigned* table = reinterpret_cast<unsigned*>(p + HDR_BYTES);
  unsigned* ka = reinterpret_cast<unsigned*>(p + HDR_BYTES + al256(RS_THREADS * (size_t)ntiles * sizeof(unsigned)));
  unsigned* kb = ka + al256((size_t)n * sizeof(unsigned)) / sizeof(unsigned);
  int* vb = reinterpret_cast<int*>(kb + al256((size_t)n * sizeof(unsigned)) / sizeof(unsigned));
  cudaError_t e = cudaMemsetAsync(p, 0, HDR_BYTES, st);
  if (e != cudaSuccess) return e;
  const int threads = 256;
  const int blocks = (n + threads - 1) / threads;
  bin_bbox_kernel<<<blocks < 512 ? blocks : 512, threads, 0, st>>>(x, y, n, bb);
  bin_key_kernel<<<blocks, threads, 0, st>>>(x, y, n, bb, ka);
  // pass 1: low digit, identity payload, (ka) -> (kb, vb)
  rs_count_kernel<<<ntiles, RS_THREADS, 0, st>>>(ka, n, 0, table, ntiles, tot0);
  rs_offsets_kernel<<<RS_THREADS / 8, 256, 0, st>>>(table, ntiles, tot0);
  rs_scatter_kernel<<<ntiles, RS_THREADS, 0, st>>>(ka, nullptr, n, 0, table, ntiles, kb, vb);
  // pass 2: high digit, (kb, vb) -> (ka, perm)
  rs_count_kernel<<<ntiles, RS_THREADS, 0, st>>>(kb, n, BIN_BITS, table, ntiles, tot1);
  rs_offsets_kernel<<<RS_THREADS / 8, 256, 0, st>>>(table, ntiles, tot1);
  rs_scatter_kernel<<<ntiles, RS_THREADS, 0, st>>>(kb, vb, n, BIN_BITS, table, ntiles, ka, perm);
  if (launches) *launches += 8;
  return cudaGetLastError();
}

cudaError_t bin_gather(const int* perm, const float* x, const float* y, const float* r, const float* g, int n,
                       float* bx, float* by, float* br, float* bg, cudaStream_t st, int* launches) {
  if (n <= 0) return cudaSuccess;
  bin_gather_kernel<<<(n + 255) / 256, 256, 0, st>>>(perm, x, y, r, g, n, bx, by, br, bg);
  if (launches) *launches += 1;
  return cudaGetLastError();
}

}  // namespace obs
