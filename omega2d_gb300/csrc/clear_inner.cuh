// clear_inner.cuh -- per-point logic of clear_inner_panp2 (src/Reflect.h:491-729), shared by the
// CUDA kernel (csrc/clear_inner.cu) and by a host build the CPU tests compile with g++.
//
// A point inside a body's cutoff layer is cropped (method 0: strength scaled and the point
// shifted outward by the cut tables of src/Reflect.h:383-480) or pushed onto the layer
// (method 1).  The reference sweeps all untested points until none is modified; a point's
// fate depends only on its own position and the panels, so the same result comes from
// repeating the test per point until it passes, which is what clear_point does.
//
// Float semantics follow the reference's float build: std::pow(S, 2) and the 1.0 literals
// promote to double, so those sub-expressions are formed in double and rounded to float where
// the reference stores them.  Every build of this file forms each product and sum separately
// (no fused multiply-add: nvcc -fmad=false, host -ffp-contract=off), which is how the oracle is
// built too, so the engine and the oracle agree bit for bit.  Its closest-panel tests `d < nextafter(min, 0.0)` (a double
// nextafter: strictly below) and `d < nextafterf(min, FLT_MAX)` (at most equal) are, for float
// d, "new closest if d < min" and "tie if d == min".
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define OBS_HD __host__ __device__ __forceinline__
#else
#define OBS_HD inline
#endif

namespace obs {
namespace clear {

constexpr int CUT_N = 63;            // init_cut_tables(0.1): 2 * 30 + 3 entries

struct Geo {
  const float* nx;                   // nodes
  const float* ny;
  const unsigned* idx;               // node-index pairs, validated against nnodes
  int npan;
  const float* pnx;                  // panel normals (Surfaces::compute_bases)
  const float* pny;
  const float* nnx;                  // node normals: sums of the adjacent panel normals
  const float* nny;
  const float* cpos;                 // cut table: position in core radii, strength kept, shift
  const float* ckeep;
  const float* cshift;
};

// init_cut_tables(0.1) (src/Reflect.h:383-443) in the reference's float build: std::pow and the
// 1.0 literals are double, the accumulators float.  Host only (63 entries, built once).
inline void cut_table(float* pos, float* keep, float* shift) {
  const float max_rad = 3.0f, dx_in = 0.1f;
  const int nx = (int)(0.5 + (double)(max_rad / dx_in));
  const float dx = max_rad / (float)nx;
  int k = 0;
  pos[k] = (float)(-nx - 0.5) * dx; keep[k] = 0.0f; shift[k] = 0.0f; ++k;
  float twgt = 0.0f, tmom = 0.0f;
  for (int i = -nx; i < nx + 1; ++i) {
    const float pi_ = (float)i * dx;
    const float distxs = (float)((double)pi_ * (double)pi_);
    float rwgt = 0.0f;
    for (int j = -nx; j < nx + 1; ++j) {
      const float pj = (float)j * dx;
      const float distxys = (float)((double)distxs + (double)pj * (double)pj);
      rwgt += expf(-distxys);
    }
    rwgt = (float)((double)rwgt * ((double)dx * (double)dx));
    rwgt = (float)((double)rwgt * (1.0 / 3.14159265358979323846));
    twgt += rwgt;
    tmom += ((float)i * dx) * rwgt;
    pos[k] = (float)(i + 0.5) * dx; keep[k] = twgt; shift[k] = -tmom / twgt; ++k;
  }
  pos[k] = (float)(nx + 1.5) * dx; keep[k] = 1.0f; shift[k] = 0.0f;
}

// Panel normals (Surfaces::compute_bases, src/Surfaces.h:682-724) and node normals summed in
// panel order (src/Reflect.h:521-533), sequentially.  Returns 0, or 1 + the first panel with a
// node index out of range or zero length.
OBS_HD int normals(int nnodes, const float* nx, const float* ny, int npan, const unsigned* idx, float* pnx,
                   float* pny, float* nnx, float* nny) {
  for (int j = 0; j < npan; ++j)
    if (idx[2 * j] >= (unsigned)nnodes || idx[2 * j + 1] >= (unsigned)nnodes) return 1 + j;
  for (int k = 0; k < nnodes; ++k) nnx[k] = nny[k] = 0.0f;
  for (int j = 0; j < npan; ++j) {
    const unsigned a = idx[2 * j], b = idx[2 * j + 1];
    float tx = nx[b] - nx[a], ty = ny[b] - ny[a];
    const float base = sqrtf(tx * tx + ty * ty);
    if (!(base > 0.0f)) return 1 + j;
    tx = (float)((double)tx * (1.0 / (double)base));
    ty = (float)((double)ty * (1.0 / (double)base));
    pnx[j] = -ty;
    pny[j] = tx;
  }
  for (int j = 0; j < npan; ++j) {
    const unsigned a = idx[2 * j], b = idx[2 * j + 1];
    nnx[a] += pnx[j]; nny[a] += pny[j];
    nnx[b] += pnx[j]; nny[b] += pny[j];
  }
  return 0;
}

// panel_point_distance (src/Reflect.h:111-165)
OBS_HD void seg_closest(float x0, float y0, float x1, float y1, float tx, float ty, float& d2, float& cx,
                        float& cy, int& kind, int& which) {
  const float bx = x1 - x0, by = y1 - y0;
  const float blensq = bx * bx + by * by;
  const float ax = tx - x0, ay = ty - y0;
  const float t = (ax * bx + ay * by) / blensq;
  if (t > 0.0f && t < 1.0f) {
    const float c = ay * bx - ax * by;
    d2 = (float)(((double)c * (double)c) / (double)blensq);
    cx = (float)((1.0 - (double)t) * (double)x0 + (double)(t * x1));
    cy = (float)((1.0 - (double)t) * (double)y0 + (double)(t * y1));
    kind = 0;
    which = -1;
    return;
  }
  const float ex = tx - x1, ey = ty - y1;
  const float r0 = (float)((double)ax * (double)ax + (double)ay * (double)ay);
  const float r1 = (float)((double)ex * (double)ex + (double)ey * (double)ey);
  kind = 1;
  if (r0 < r1) {
    which = 0; d2 = r0; cx = x0; cy = y0;
  } else {
    which = 1; d2 = r1; cx = x1; cy = y1;
  }
}

// get_cut_entry (src/Reflect.h:448-480)
OBS_HD void cut_entry(const Geo& g, float p, float& smult, float& dshift) {
  smult = 1.0f;
  dshift = 0.0f;
  if (p < g.cpos[0]) {
    smult = 0.0f;
    dshift = (float)(1.0 - (double)p);
    return;
  }
  if (p > g.cpos[CUT_N - 1]) return;
  for (int i = 1; i < CUT_N; ++i) {
    if (p < g.cpos[i]) {
      const float frac = (p - g.cpos[i - 1]) / (g.cpos[i] - g.cpos[i - 1]);
      smult = (float)((double)(frac * g.ckeep[i]) + (1.0 - (double)frac) * (double)g.ckeep[i - 1]);
      dshift = (float)((double)(frac * g.cshift[i]) + (1.0 - (double)frac) * (double)g.cshift[i - 1]);
      return;
    }
  }
}

// A lower bound, in FP32, on the squared distance seg_closest computes for one panel (its
// exact float/double arithmetic).  The differences ax, ay, bx, by, the cross product c and the
// dot product are formed exactly as seg_closest forms them, so they are the same floats; only
// t = dot/blensq is taken as dot * ibl (ibl = 1/blensq in FP32, within a few ulps).  Where t is
// at least 2^-20 inside (0, 1), seg_closest takes the panel case, c^2/blensq; where it is at
// least 2^-20 outside, the node case, min(ax^2 + ay^2, ex^2 + ey^2) -- either way the FP32 value
// is within a few ulps of seg_closest's double-then-float one, and (1 - 2^-20) times it bounds
// that from below.  In the 2^-20 band around 0 and 1 the bound is the smaller of the two cases
// (seg_closest's value is one of them).  Non-finite inputs give NaN or inf, which never reject.
OBS_HD float seg_lower_bound(float x0, float y0, float x1, float y1, float ibl, float tx, float ty) {
  const float bx = x1 - x0, by = y1 - y0;
  const float ax = tx - x0, ay = ty - y0;
  const float t = (ax * bx + ay * by) * ibl;
  const float c = ay * bx - ax * by;
  const float dp = (c * c) * ibl;
  const float ex = tx - x1, ey = ty - y1;
  const float dn = fminf(ax * ax + ay * ay, ex * ex + ey * ey);
  const float eps = 9.5367431640625e-7f;          // 2^-20
  const bool inside = t > eps && t < 1.0f - eps;
  const bool outside = t < -eps || t > 1.0f + eps;
  const float d = inside ? dp : (outside ? dn : fminf(dp, dn));
  return d * 0.99999904632568359375f;
}

// bound > T (1 + 2^-16): the panel cannot be the closest or tie it when T bounds the minimum
OBS_HD bool beyond(float bound, float T) { return bound > T * 1.0000152587890625f && bound <= 3.0e38f; }

// the closest panels or nodes of one point (ties kept), as clear_inner_panp2's hits
// (src/Reflect.h:560-604), reduced to the sums its normal and closest-point averages need
struct Closest {
  float mind, snx, sny, scx, scy;
  int cnt;
};

OBS_HD void closest_init(Closest& c) {
  c.mind = (float)(0.1 * 3.4028234663852886e38);
  c.snx = c.sny = c.scx = c.scy = 0.0f;
  c.cnt = 0;
}

// panel j (nodes a -> b at (x0, y0) -> (x1, y1), normal (pnx, pny)) against the point (tx, ty)
OBS_HD void closest_add(const Geo& g, Closest& c, unsigned a, unsigned b, float x0, float y0, float x1, float y1,
                        float pnx, float pny, float tx, float ty) {
  float d2, cx, cy;
  int kind, which;
  seg_closest(x0, y0, x1, y1, tx, ty, d2, cx, cy, kind, which);
  if (d2 < c.mind) {                         // a new closest panel or node
    c.mind = d2;
    c.snx = c.sny = c.scx = c.scy = 0.0f;
    c.cnt = 0;
  } else if (!(d2 == c.mind)) {
    return;
  }
  if (kind == 0) {
    c.snx += pnx;
    c.sny += pny;
  } else {
    const unsigned nd = which ? b : a;
    c.snx += g.nnx[nd];
    c.sny += g.nny[nd];
  }
  c.scx += cx;
  c.scy += cy;
  ++c.cnt;
}

// The test after one sweep (src/Reflect.h:606-700): crop (method 0) or push (method 1) the point
// when it lies inside the layer.  Returns 0 when the point passes (done), 1 when it was
// modified (test it again), 2 when no panel was found.
OBS_HD int clear_apply(const Geo& g, const Closest& c, int method, float cutoff_mult, float ips, float rad, float& x,
                       float& y, float& s, double& lost) {
  if (c.cnt == 0) return 2;                  // no panel (the reference would spin)
  float snx = c.snx, sny = c.sny;
  const float normilen = (float)(1.0 / (double)sqrtf(snx * snx + sny * sny));
  snx *= normilen;
  sny *= normilen;
  const float scx = c.scx / (float)c.cnt;
  const float scy = c.scy / (float)c.cnt;
  const float dotp = snx * (x - scx) + sny * (y - scy) - cutoff_mult * ips;
  if (method == 0) {
    if (!(dotp < rad)) return 0;
    float smult, dshift;
    cut_entry(g, dotp / rad, smult, dshift);
    lost += (double)s * (1.0 - (double)smult);
    s *= smult;
    x += dshift * rad * snx;
    y += dshift * rad * sny;
  } else {
    if (!((double)dotp < -0.001 * (double)ips)) return 0;
    x -= dotp * snx;
    y -= dotp * sny;
  }
  return 1;
}

// One point, tested until it passes (at most max_sweeps times), against all panels of g read
// from its arrays.  rad = the point's core radius (ips for field points).  Returns the number
// of modifications, or -1 when max_sweeps ran out; lost receives the circulation removed
// (method 0).  Each sweep takes two passes: the panel with the smallest lower bound gives, by
// its exact distance, a bound T on the minimum; then only panels whose lower bound does not
// exceed T are evaluated exactly, in panel order.  The reference's hits are the panels at the
// exact minimum (ties included, in panel order), which this reproduces bit for bit.  The CUDA
// kernel runs the same passes over panel records staged in shared memory.
OBS_HD int clear_point(const Geo& g, int method, float cutoff_mult, float ips, float rad, float& x, float& y,
                       float& s, double& lost, int max_sweeps) {
  int crops = 0;
  lost = 0.0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    float lbmin = 3.4028234663852886e38f;
    int jstar = -1;
    for (int j = 0; j < g.npan; ++j) {
      const unsigned a = g.idx[2 * j], b = g.idx[2 * j + 1];
      const float bx = g.nx[b] - g.nx[a], by = g.ny[b] - g.ny[a];
      const float lb = seg_lower_bound(g.nx[a], g.ny[a], g.nx[b], g.ny[b], 1.0f / (bx * bx + by * by), x, y);
      if (lb < lbmin) { lbmin = lb; jstar = j; }
    }
    float T = INFINITY;                           // no candidate: no rejection
    if (jstar >= 0) {
      const unsigned a = g.idx[2 * jstar], b = g.idx[2 * jstar + 1];
      float cx, cy;
      int kind, which;
      seg_closest(g.nx[a], g.ny[a], g.nx[b], g.ny[b], x, y, T, cx, cy, kind, which);
    }
    Closest c;
    closest_init(c);
    for (int j = 0; j < g.npan; ++j) {
      const unsigned a = g.idx[2 * j], b = g.idx[2 * j + 1];
      const float x0 = g.nx[a], y0 = g.ny[a], x1 = g.nx[b], y1 = g.ny[b];
      const float bx = x1 - x0, by = y1 - y0;
      if (beyond(seg_lower_bound(x0, y0, x1, y1, 1.0f / (bx * bx + by * by), x, y), T)) continue;
      closest_add(g, c, a, b, x0, y0, x1, y1, g.pnx[j], g.pny[j], x, y);
    }
    const int r = clear_apply(g, c, method, cutoff_mult, ips, rad, x, y, s, lost);
    if (r != 1) return crops;
    ++crops;
  }
  return -1;
}

}  // namespace clear
}  // namespace obs
