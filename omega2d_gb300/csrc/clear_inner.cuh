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
// the reference stores them.  Its closest-panel tests `d < nextafter(min, 0.0)` (a double
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

// One point, tested until it passes (at most max_sweeps times).  rad = the point's core radius
// (ips for field points).  Returns the number of modifications, or -1 when max_sweeps ran out;
// lost receives the circulation removed (method 0).
OBS_HD int clear_point(const Geo& g, int method, float cutoff_mult, float ips, float rad, float& x, float& y,
                       float& s, double& lost, int max_sweeps) {
  const float big = (float)(0.1 * 3.4028234663852886e38);
  int crops = 0;
  lost = 0.0;
  for (int sweep = 0; sweep < max_sweeps; ++sweep) {
    float mind = big, snx = 0.0f, sny = 0.0f, scx = 0.0f, scy = 0.0f;
    int cnt = 0;
    for (int j = 0; j < g.npan; ++j) {
      const unsigned a = g.idx[2 * j], b = g.idx[2 * j + 1];
      float d2, cx, cy;
      int kind, which;
      seg_closest(g.nx[a], g.ny[a], g.nx[b], g.ny[b], x, y, d2, cx, cy, kind, which);
      if (d2 < mind) {                       // a new closest panel or node
        mind = d2;
        snx = sny = scx = scy = 0.0f;
        cnt = 0;
      } else if (!(d2 == mind)) {
        continue;
      }
      if (kind == 0) {
        snx += g.pnx[j];
        sny += g.pny[j];
      } else {
        const unsigned nd = which ? b : a;
        snx += g.nnx[nd];
        sny += g.nny[nd];
      }
      scx += cx;
      scy += cy;
      ++cnt;
    }
    if (cnt == 0) return crops;                // no panel (the reference would spin)
    const float normilen = (float)(1.0 / (double)sqrtf(snx * snx + sny * sny));
    snx *= normilen;
    sny *= normilen;
    scx /= (float)cnt;
    scy /= (float)cnt;
    const float dotp = snx * (x - scx) + sny * (y - scy) - cutoff_mult * ips;
    if (method == 0) {
      if (!(dotp < rad)) return crops;
      float smult, dshift;
      cut_entry(g, dotp / rad, smult, dshift);
      lost += (double)s * (1.0 - (double)smult);
      s *= smult;
      x += dshift * rad * snx;
      y += dshift * rad * sny;
    } else {
      if (!((double)dotp < -0.001 * (double)ips)) return crops;
      x -= dotp * snx;
      y -= dotp * sny;
    }
    ++crops;
  }
  return -1;
}

}  // namespace clear
}  // namespace obs
