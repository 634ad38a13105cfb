/* oracle_impl.h -- body of the CPU restatement, included twice by oracle.c.
 *
 * TEST INFRASTRUCTURE ONLY: the oracle is the checker for the CUDA path and the timed CPU
 * baseline ("port"); it is never linked into or called by the product library.
 *
 * Before inclusion the includer defines
 *   R      pair-arithmetic type (float for the reference's non-Vc build, double for FP64)
 *   A      accumulator type (double in both instantiations, src/Simulation.h:44-50)
 *   SFX(n) name decoration (n##_f or n##_d)
 *
 * Conventions shared with the reference (cited per function):
 *   - every influence sum is left unscaled: the 1/(2 pi) factor and the freestream are applied
 *     by the finalize step (src/ElementBase.h:215-234);
 *   - drivers ACCUMULATE into the target arrays (+=), like src/Influence.h:207-208, 359-360;
 *   - "thick" targets carry a core radius and use the two-radius core forms
 *     (src/CoreFunc.h, "non-singular targets"); tr == NULL means field points (0p forms).
 */

/* ---------------------------------------------------------------- core functions */

/* Velocity-only core value K(d^2) such that the pair velocity is ss*K*(-dy, dx).
 * core ids follow omega2d_gb300.h (OBS_CORE_*). */
static inline R SFX(core_vel)(int core, R d2, R sr, R tr, int thick) {
  switch (core) {
  case 1: { /* Rosenhead-Moore, src/CoreFunc.h:47-59 */
    R r2 = thick ? d2 + sr*sr + tr*tr : d2 + sr*sr;
    return (R)1.0 / r2;
  }
  case 2: { /* Gaussian-blob ("exponential") core with cut-offs, src/CoreFunc.h:111-153 */
    R ood2 = (R)1.0 / d2;
    R corefac = (R)1.0 / (thick ? sr*sr + tr*tr : sr*sr);
    R reld2 = corefac / ood2;
    if (reld2 > (R)16.0) return ood2;
    if (reld2 < (R)0.001) return corefac;
    return ood2 * ((R)1.0 - EXP(-reld2));
  }
  case 3: { /* Vatistas n=2, src/CoreFunc.h:238-252 */
    R s2 = sr*sr, t2 = tr*tr;
    return thick ? (R)1.0 / SQRT(d2*d2 + s2*s2 + t2*t2) : (R)1.0 / SQRT(d2*d2 + s2*s2);
  }
  case 4: { /* Winckelmans-Leonard, src/CoreFunc.h:189-203 */
    R s2 = thick ? sr*sr + tr*tr : sr*sr;
    R dd = d2 + s2;
    return (dd + s2) / (dd*dd);
  }
  case 5: { /* Vatistas n=3, src/CoreFunc.h:283-297 */
    R s2 = sr*sr, t2 = tr*tr;
    R a = thick ? d2*d2*d2 + s2*s2*s2 + t2*t2*t2 : d2*d2*d2 + s2*s2*s2;
    return (R)1.0 / CBRT(a);
  }
  case 6: /* singular point vortex: RM with zero radii, coincident pair excluded */
    return d2 > (R)0 ? (R)1.0 / d2 : (R)0;
  case 7: { /* compact exponential (no counterpart in the reference):
             * K = (1 - exp(-y)) / d^2 with y = (d^2/s^2)^(3/2), s^2 = sr^2 (+ tr^2);
             * y > 16 -> 1/d^2; y < 0.001 -> (d/s^3)(1 - y/2) (two-term series). */
    R s2 = thick ? sr*sr + tr*tr : sr*sr;
    R x = d2 / s2;
    R y = x * SQRT(x);
    if (y > (R)16.0) return (R)1.0 / d2;
    if (y < (R)0.001) return SQRT(d2) / (s2 * SQRT(s2)) * ((R)1.0 - (R)0.5 * y);
    return ((R)1.0 - EXP(-y)) / d2;
  }
  default:
    return (R)0;
  }
}

/* Core value plus bbb = 2 dK/d(d^2), the gradient form used by kernelug/kerneluw/kernelue.
 * Reference forms: RM src/CoreFunc.h:64-80, Gaussian :145-181, WL :208-229, V2 :257-274,
 * V3 :302-321.  Coincident pairs (d2 == 0) return bbb = 0 so that no 0*inf appears (the
 * reference's Gaussian form yields NaN there); the pair's r2 term is still the core's value
 * at the origin, which is the limit of the smooth kernel. */
static inline void SFX(core_grad)(int core, R d2, R sr, R tr, int thick, R* r2, R* bbb) {
  switch (core) {
  case 1: {
    R td2 = thick ? d2 + sr*sr + tr*tr : d2 + sr*sr;
    *r2 = (R)1.0 / td2;
    *bbb = (R)(-2.0) * (*r2) * (*r2);
    return;
  }
  case 2: {
    R ood2 = (R)1.0 / d2;
    R corefac = (R)1.0 / (thick ? sr*sr + tr*tr : sr*sr);
    R reld2 = corefac / ood2;
    if (reld2 > (R)16.0) *r2 = ood2;
    else if (reld2 < (R)0.001) *r2 = corefac;
    else *r2 = ood2 * ((R)1.0 - EXP(-reld2));
    if (d2 == (R)0) { *bbb = (R)0; return; }
    *bbb = (R)(-2.0) * (*r2) * ood2 + (R)2.0 * corefac * ood2 * EXP(-reld2);
    return;
  }
  case 3: {
    R s2 = sr*sr, t2 = tr*tr;
    *r2 = thick ? (R)1.0 / SQRT(d2*d2 + s2*s2 + t2*t2) : (R)1.0 / SQRT(d2*d2 + s2*s2);
    *bbb = (R)(-2.0) * (*r2) * (*r2) * (*r2) * d2;
    return;
  }
  case 4: {
    R s2 = thick ? sr*sr + tr*tr : sr*sr;
    R dd = d2 + s2;
    R ood2s = (R)1.0 / (dd*dd);
    *r2 = (dd + s2) * ood2s;
    *bbb = ((R)2.0 - (R)4.0 * (*r2) * dd) * ood2s;
    return;
  }
  case 5: {
    R s2 = sr*sr, t2 = tr*tr;
    R ds6 = thick ? d2*d2*d2 + s2*s2*s2 + t2*t2*t2 : d2*d2*d2 + s2*s2*s2;
    *r2 = (R)1.0 / CBRT(ds6);
    *bbb = (R)(-2.0) * d2*d2 * (*r2) / ds6;
    return;
  }
  case 6:
    if (d2 > (R)0) { *r2 = (R)1.0 / d2; *bbb = (R)(-2.0) * (*r2) * (*r2); }
    else { *r2 = (R)0; *bbb = (R)0; }
    return;
  case 7: {
    R s2 = thick ? sr*sr + tr*tr : sr*sr;
    if (d2 == (R)0) { *r2 = (R)0; *bbb = (R)0; return; }
    R x = d2 / s2;
    R y = x * SQRT(x);
    R ood2 = (R)1.0 / d2;
    if (y > (R)16.0) { *r2 = ood2; *bbb = (R)(-2.0) * ood2 * ood2; return; }
    R e = EXP(-y);
    *r2 = (y < (R)0.001) ? SQRT(d2) / (s2 * SQRT(s2)) * ((R)1.0 - (R)0.5 * y) : ((R)1.0 - e) * ood2;
    /* 2 dK/d(d^2) = (3 y e^{-y} / d^2 - 2 K) / d^2 */
    *bbb = ((R)3.0 * y * e * ood2 - (R)2.0 * (*r2)) * ood2;
    return;
  }
  default:
    *r2 = (R)0; *bbb = (R)0;
  }
}

/* ---------------------------------------------------------------- points on points */

/* points_affect_points, src/Influence.h:56-416 (x86 branches); restype as results_t
 * (src/ResultsType.h:26-32): 1 velonly, 2 velandgrad, 3 psionly, 4 velandvort, 5 velandshear.
 * extra: velandgrad -> e0..e3 = (ux, vx, uy, vy); psionly -> e0 = psi; vort -> e0 = w;
 * shear -> e0 = e.  Pair kernels: kernelu_0v_0b/0p (src/Kernels.h:81-106), kernelug_0v_0b
 * (:112-133, with a field-point twin), kerneluw (:139-179), kernelue (:185-231),
 * kernelp (:52-74). */
void SFX(o_points_affect_points)(int core, int restype,
                                 int ns, const R* sx, const R* sy, const R* sr, const R* ss,
                                 int nt, const R* tx, const R* ty, const R* tr,
                                 R* tu, R* tv, R* e0, R* e1, R* e2, R* e3) {
  const int thick = (tr != 0);
  #pragma omp parallel for schedule(static)
  for (int i = 0; i < nt; ++i) {
    A au = 0, av = 0, a0 = 0, a1 = 0, a2 = 0, a3 = 0;
    const R xi = tx[i], yi = ty[i], ri = thick ? tr[i] : (R)0;
    for (int j = 0; j < ns; ++j) {
      const R dx = xi - sx[j];
      const R dy = yi - sy[j];
      const R d2 = dx*dx + dy*dy;
      if (restype == 1) {
        const R r2 = ss[j] * SFX(core_vel)(core, d2, sr[j], ri, thick);
        au -= r2 * dy;
        av += r2 * dx;
      } else if (restype == 3) {
        /* kernelp_0v_0b / 0v_0p: -ss * 0.5*log(d^2 + sr^2 (+ tr^2)) */
        const R a = thick ? d2 + sr[j]*sr[j] + ri*ri : d2 + sr[j]*sr[j];
        a0 -= ss[j] * ((R)0.5 * LOG(a));
      } else {
        R r2, bbb;
        SFX(core_grad)(core, d2, sr[j], ri, thick, &r2, &bbb);
        r2 *= ss[j];
        bbb *= ss[j];
        au -= r2 * dy;
        av += r2 * dx;
        if (restype == 2) {
          a0 += -bbb*dx*dy;          /* du/dx */
          a1 +=  bbb*dx*dx + r2;     /* dv/dx */
          a2 += -bbb*dy*dy - r2;     /* du/dy */
          a3 +=  bbb*dx*dy;          /* dv/dy */
        } else if (restype == 4) {
          const R dudy = -bbb*dy*dy - r2;
          const R dvdx =  bbb*dx*dx + r2;
          a0 += dvdx - dudy;
        } else if (restype == 5) {
          const R dudx = -bbb*dx*dy;
          const R asym = bbb*(dx*dx - dy*dy);
          a0 += SQRT(dudx*dudx + (R)0.25*asym*asym);
        }
      }
    }
    if (restype != 3) {
      tu[i] = (R)((A)tu[i] + au);
      tv[i] = (R)((A)tv[i] + av);
    }
    if (restype == 2) {
      e0[i] = (R)((A)e0[i] + a0); e1[i] = (R)((A)e1[i] + a1);
      e2[i] = (R)((A)e2[i] + a2); e3[i] = (R)((A)e3[i] + a3);
    } else if (restype >= 3) {
      e0[i] = (R)((A)e0[i] + a0);
    }
  }
}

/* points_affect_points_vorticity, src/InfluenceVort.h:96-110 (the non-Vc branch, no cut-off):
 * Gaussian-blob vorticity at field points, tw += sum 2 ss exp(-d^2/sr^2) / sr^2; the
 * differences are formed in R and the rest in A, as there. */
void SFX(o_points_affect_points_vorticity)(int ns, const R* sx, const R* sy, const R* sr, const R* ss,
                                           int nt, const R* tx, const R* ty, R* tw) {
  #pragma omp parallel for schedule(static)
  for (int i = 0; i < nt; ++i) {
    A aw = 0;
    for (int j = 0; j < ns; ++j) {
      const A dx = (A)(tx[i] - sx[j]);
      const A dy = (A)(ty[i] - sy[j]);
      const A s2 = (A)sr[j] * (A)sr[j];
      const A distsq = (dx*dx + dy*dy) / s2;
      aw += (A)((R)2.0 * ss[j]) * exp(-distsq) / s2;
    }
    tw[i] = (R)((A)tw[i] + aw);
  }
}

/* ---------------------------------------------------------------- panels */

/* get_ustar, src/Kernels.h:256-268 (non-Vc): angle subtended by the panel, wrapped to [-pi, pi] */
static inline R SFX(ustar)(R dx0, R dy0, R dx1, R dy1) {
  R u = ATAN2(dx1, dy1) - ATAN2(dx0, dy0);
  if ((double)u < -M_PI) u = (R)((double)u + 2.0 * M_PI);
  if ((double)u > M_PI) u = (R)((double)u - 2.0 * M_PI);
  return u;
}

/* kernelu_1v_0p, src/Kernels.h:311-354: constant-strength vortex panel on a point */
static inline void SFX(k1v)(R sx0, R sy0, R sx1, R sy1, R str, R tx, R ty, R* u, R* v) {
  const R dx0 = tx - sx0, dy0 = ty - sy0, dx1 = tx - sx1, dy1 = ty - sy1;
  const R px = sx1 - sx0, py = sy1 - sy0;
  const R rij2 = dx0*dx0 + dy0*dy0, rij12 = dx1*dx1 + dy1*dy1, panl = px*px + py*py;
  const R us = SFX(ustar)(dx0, dy0, dx1, dy1);
  const R vs = (R)0.5 * LOG(rij2 / rij12);
  const R velx = us*px - vs*py, vely = us*py + vs*px;
  const R mult = str * ((R)1.0 / SQRT(panl));
  *u = mult * velx;
  *v = mult * vely;
}

/* kernelu_1vs_0p, src/Kernels.h:362-405: vortex (vs) + source (ss) panel on a point */
static inline void SFX(k1vs)(R sx0, R sy0, R sx1, R sy1, R vstr, R sstr, R tx, R ty, R* u, R* v) {
  const R dx0 = tx - sx0, dy0 = ty - sy0, dx1 = tx - sx1, dy1 = ty - sy1;
  R px = sx1 - sx0, py = sy1 - sy0;
  const R rij2 = dx0*dx0 + dy0*dy0, rij12 = dx1*dx1 + dy1*dy1, panl = px*px + py*py;
  const R mult = (R)1.0 / SQRT(panl);
  px *= mult; py *= mult;
  const R us = SFX(ustar)(dx0, dy0, dx1, dy1);
  const R vs = (R)0.5 * LOG(rij2 / rij12);
  *u = vstr * (us*px - vs*py) + sstr * (us*py + vs*px);
  *v = vstr * (us*py + vs*px) + sstr * (vs*py - us*px);
}

/* kernelu_1vos_0p, src/Kernels.h:412-458: vortex and source parts kept separate (unit strengths) */
static inline void SFX(k1vos)(R sx0, R sy0, R sx1, R sy1, R tx, R ty, R* vu, R* vv, R* su, R* sv) {
  const R dx0 = tx - sx0, dy0 = ty - sy0, dx1 = tx - sx1, dy1 = ty - sy1;
  R px = sx1 - sx0, py = sy1 - sy0;
  const R rij2 = dx0*dx0 + dy0*dy0, rij12 = dx1*dx1 + dy1*dy1, panl = px*px + py*py;
  const R mult = (R)1.0 / SQRT(panl);
  px *= mult; py *= mult;
  const R us = SFX(ustar)(dx0, dy0, dx1, dy1);
  const R vs = (R)0.5 * LOG(rij2 / rij12);
  *vu = us*px - vs*py;
  *vv = us*py + vs*px;
  *su = us*py + vs*px;
  *sv = vs*py - us*px;
}

/* panels_affect_points, src/Influence.h:422-614 (x86 branch): ss == NULL selects the
 * vortex-only kernelu_1v_0p loop (:576-594), otherwise kernelu_1vs_0p (:558-575). */
void SFX(o_panels_affect_points)(const R* nx, const R* ny, int npan, const unsigned* idx,
                                 const R* vs, const R* ss,
                                 int nt, const R* tx, const R* ty, R* tu, R* tv) {
  #pragma omp parallel for schedule(static)
  for (int i = 0; i < nt; ++i) {
    A au = 0, av = 0;
    for (int j = 0; j < npan; ++j) {
      const unsigned j0 = idx[2*j], j1 = idx[2*j+1];
      R ru, rv;
      if (ss) SFX(k1vs)(nx[j0], ny[j0], nx[j1], ny[j1], vs[j], ss[j], tx[i], ty[i], &ru, &rv);
      else    SFX(k1v)(nx[j0], ny[j0], nx[j1], ny[j1], vs[j], tx[i], ty[i], &ru, &rv);
      au += ru; av += rv;
    }
    tu[i] = (R)((A)tu[i] + au);
    tv[i] = (R)((A)tv[i] + av);
  }
}

/* points_affect_panels, src/Influence.h:633-771 (x86 branch): the panel is the "source" of
 * kernelu_1v_0p and the particle the "target", so the sum is subtracted and scaled by the
 * inverse panel length (ta = panel length, src/Surfaces.h:702-706). Particle radii unused. */
void SFX(o_points_affect_panels)(int ns, const R* sx, const R* sy, const R* ss,
                                 const R* nx, const R* ny, int npan, const unsigned* idx,
                                 R* pu, R* pv) {
  #pragma omp parallel for schedule(static)
  for (int i = 0; i < npan; ++i) {
    const unsigned i0 = idx[2*i], i1 = idx[2*i+1];
    const R lx = nx[i1] - nx[i0], ly = ny[i1] - ny[i0];
    const R ta = SQRT(lx*lx + ly*ly);
    const A plen = (A)1.0 / (A)ta;
    A au = 0, av = 0;
    for (int j = 0; j < ns; ++j) {
      R ru, rv;
      SFX(k1v)(nx[i0], ny[i0], nx[i1], ny[i1], ss[j], sx[j], sy[j], &ru, &rv);
      au += ru; av += rv;
    }
    pu[i] = (R)((A)pu[i] - plen * au);
    pv[i] = (R)((A)pv[i] - plen * av);
  }
}

/* panel bases, src/Surfaces.h:682-724: unit tangent node0->node1, normal to its left, length */
static inline void SFX(panel_basis)(const R* nx, const R* ny, const unsigned* idx, int i,
                                    R* tx, R* ty, R* nxo, R* nyo, R* len) {
  const unsigned i0 = idx[2*i], i1 = idx[2*i+1];
  R x1 = nx[i1] - nx[i0], y1 = ny[i1] - ny[i0];
  const R base = SQRT(x1*x1 + y1*y1);
  x1 = (R)((double)x1 * (1.0 / (double)base));
  y1 = (R)((double)y1 * (1.0 / (double)base));
  *tx = x1; *ty = y1; *nxo = -y1; *nyo = x1; *len = base;
}

/* panels_on_panels_coeff, src/Coefficients.h:155-427 (x86 branch, use_two_way = true):
 * column-major nrows x ncols block (targets are rows), scaled by 1/(2 pi).  nunk = 2 is the
 * reference's vortex+source system (src/Surfaces.h:69); nunk = 1 the vortex-only branch
 * (:366-385).  self != 0 sets the self-influence diagonal pi (:389-401) before scaling. */
void SFX(o_panels_on_panels_coeff)(int nunk, int self,
                                   const R* snx, const R* sny, int nsrc, const unsigned* sidx,
                                   const R* tnx, const R* tny, int ntarg, const unsigned* tidx,
                                   R* out) {
  const size_t nrows = (size_t)ntarg * nunk;
  #pragma omp parallel for schedule(static)
  for (int j = 0; j < nsrc; ++j) {
    const unsigned s0 = sidx[2*j], s1 = sidx[2*j+1];
    const R sx0 = snx[s0], sy0 = sny[s0], sx1 = snx[s1], sy1 = sny[s1];
    R stx, sty, snx_, sny_, sa;
    SFX(panel_basis)(snx, sny, sidx, j, &stx, &sty, &snx_, &sny_, &sa);
    R* col1 = out + (size_t)j * nunk * nrows;
    R* col2 = col1 + nrows;
    for (int i = 0; i < ntarg; ++i) {
      const unsigned t0 = tidx[2*i], t1 = tidx[2*i+1];
      const R tx0 = tnx[t0], ty0 = tny[t0], tx1 = tnx[t1], ty1 = tny[t1];
      R ttx, tty, tnx_, tny_, ta;
      SFX(panel_basis)(tnx, tny, tidx, i, &ttx, &tty, &tnx_, &tny_, &ta);
      const R xi = (R)0.5 * (tx1 + tx0), yi = (R)0.5 * (ty1 + ty0);
      if (nunk == 2) {
        R vu, vv, su, sv;
        SFX(k1vos)(sx0, sy0, sx1, sy1, xi, yi, &vu, &vv, &su, &sv);
        R c11 = vu*ttx + vv*tty, c12 = vu*tnx_ + vv*tny_;
        R c21 = su*ttx + sv*tty, c22 = su*tnx_ + sv*tny_;
        SFX(k1vos)(tx0, ty0, tx1, ty1, (R)0.5*(sx0+sx1), (R)0.5*(sy0+sy1), &vu, &vv, &su, &sv);
        const R fact = sa / ta;
        c11 -= fact * (vu*ttx + vv*tty);
        c12 -= fact * (vu*tnx_ + vv*tny_);
        c21 -= fact * (su*ttx + sv*tty);
        c22 -= fact * (su*tnx_ + sv*tny_);
        col1[2*i] = c11 * (R)0.5; col1[2*i+1] = c12 * (R)0.5;
        col2[2*i] = c21 * (R)0.5; col2[2*i+1] = c22 * (R)0.5;
      } else {
        R vu, vv;
        SFX(k1v)(sx0, sy0, sx1, sy1, (R)1.0, xi, yi, &vu, &vv);
        R c = vu*ttx + vv*tty;
        SFX(k1v)(tx0, ty0, tx1, ty1, (R)1.0, (R)0.5*(sx0+sx1), (R)0.5*(sy0+sy1), &vu, &vv);
        c -= (vu*ttx + vv*tty) * (sa / ta);
        col1[i] = c * (R)0.5;
      }
    }
    if (self) {
      if (nunk == 2) {
        col1[2*j] = (R)M_PI; col1[2*j+1] = (R)0;
        col2[2*j] = (R)0;    col2[2*j+1] = (R)M_PI;
      } else {
        col1[j] = (R)M_PI;
      }
    }
    const R fac = (R)(1.0 / (2.0 * M_PI));
    for (size_t k = 0; k < (size_t)nunk * nrows; ++k) col1[k] *= fac;
  }
}

/* vels_to_rhs_panels, src/RHS.h:54-115 */
void SFX(o_vels_to_rhs_panels)(int nunk, const R* nx, const R* ny, int npan, const unsigned* idx,
                               const R* pu, const R* pv, const R* bcn, R* rhs) {
  for (int i = 0; i < npan; ++i) {
    R ttx, tty, tnx_, tny_, len;
    SFX(panel_basis)(nx, ny, idx, i, &ttx, &tty, &tnx_, &tny_, &len);
    if (nunk == 1) {
      rhs[i] = -(pu[i]*ttx + pv[i]*tty);
    } else {
      rhs[2*i] = -(pu[i]*ttx + pv[i]*tty);
      rhs[2*i+1] = -(pu[i]*tnx_ + pv[i]*tny_) + (bcn ? bcn[i] : (R)0);
    }
  }
}

/* ElementBase::finalize_vels, src/ElementBase.h:215-234: u = fs + u/(2 pi) */
void SFX(o_finalize_vels)(int n, R* u, R* v, double fsx, double fsy) {
  const double factor = 0.5 / M_PI;
  for (int i = 0; i < n; ++i) {
    u[i] = (R)(fsx + u[i] * factor);
    v[i] = (R)(fsy + v[i] * factor);
  }
}

/* One velocity evaluation of particles on themselves, finalized (src/Convection.h:172-223). */
static void SFX(self_vels)(int core, int n, const R* x, const R* y, const R* r, const R* s,
                           double fsx, double fsy, R* u, R* v) {
  for (int i = 0; i < n; ++i) { u[i] = 0; v[i] = 0; }
  SFX(o_points_affect_points)(core, 1, n, x, y, r, s, n, x, y, r, u, v, 0, 0, 0, 0);
  SFX(o_finalize_vels)(n, u, v, fsx, fsy);
}

/* Convection::advect_1st without bodies (src/Convection.h:274-303, ElementBase.h:276-296) */
void SFX(o_advect_1st)(int core, int n, R* x, R* y, const R* r, const R* s,
                       double fsx, double fsy, double dt, int nsteps) {
  R* u = (R*)malloc(sizeof(R) * (size_t)n);
  R* v = (R*)malloc(sizeof(R) * (size_t)n);
  for (int k = 0; k < nsteps; ++k) {
    SFX(self_vels)(core, n, x, y, r, s, fsx, fsy, u, v);
    for (int i = 0; i < n; ++i) {
      x[i] += (R)dt * (R)(1.0 * u[i]);
      y[i] += (R)dt * (R)(1.0 * v[i]);
    }
  }
  free(u); free(v);
}

/* Convection::advect_2nd_ralston without bodies (src/Convection.h:390-466,
 * ElementBase.h:299-327): u = 1/4 u(x) + 3/4 u(x + 2/3 dt u(x)); x += dt u */
void SFX(o_advect_2nd_ralston)(int core, int n, R* x, R* y, const R* r, const R* s,
                               double fsx, double fsy, double dt, int nsteps) {
  R* u1 = (R*)malloc(sizeof(R) * (size_t)n);
  R* v1 = (R*)malloc(sizeof(R) * (size_t)n);
  R* u2 = (R*)malloc(sizeof(R) * (size_t)n);
  R* v2 = (R*)malloc(sizeof(R) * (size_t)n);
  R* x2 = (R*)malloc(sizeof(R) * (size_t)n);
  R* y2 = (R*)malloc(sizeof(R) * (size_t)n);
  const double tt = 2.0 / 3.0;
  for (int k = 0; k < nsteps; ++k) {
    SFX(self_vels)(core, n, x, y, r, s, fsx, fsy, u1, v1);
    for (int i = 0; i < n; ++i) {
      x2[i] = x[i] + (R)(tt * dt) * (R)(1.0 * u1[i]);
      y2[i] = y[i] + (R)(tt * dt) * (R)(1.0 * v1[i]);
    }
    SFX(self_vels)(core, n, x2, y2, r, s, fsx, fsy, u2, v2);
    for (int i = 0; i < n; ++i) {
      const R uu = (R)(0.25 * u1[i] + 0.75 * u2[i]);
      const R vv = (R)(0.25 * v1[i] + 0.75 * v2[i]);
      x[i] += (R)dt * uu;
      y[i] += (R)dt * vv;
    }
  }
  free(u1); free(v1); free(u2); free(v2); free(x2); free(y2);
}


/* panels_affect_panels, src/Influence.h:774-795: the target panels become collocation points
 * as Surfaces::represent_as_particles(1e-4, -1) builds them (src/Surfaces.h:830-876, with the
 * bases of compute_bases, :682-724): nshed = 1 + max(0, (int)(len_i / (1.2 len_0))) points per
 * panel at weights (1+2j)/(2 nshed) along it, pushed 1e-4 along the normal into the fluid;
 * the panels' influence on those points (from zero) is then added to the first ntp panel
 * velocities, index by index, as the reference's std::transform does. */
void SFX(o_panels_affect_panels)(const R* snx, const R* sny, int snp, const unsigned* sidx,
                                 const R* vs, const R* ss,
                                 const R* tnx, const R* tny, int tnp, const unsigned* tidx,
                                 R* pu, R* pv) {
  if (tnp <= 0) return;
  R* px = (R*)malloc(sizeof(R) * (size_t)tnp);
  R* py = (R*)malloc(sizeof(R) * (size_t)tnp);
  R* qu = (R*)calloc((size_t)tnp, sizeof(R));
  R* qv = (R*)calloc((size_t)tnp, sizeof(R));
  const float off = 0.0001f;
  float len0 = 0.0f;
  int m = 0;
  for (int i = 0; i < tnp && m < tnp; ++i) {
    const float x0 = (float)tnx[tidx[2*i]], y0 = (float)tny[tidx[2*i]];
    const float x1 = (float)tnx[tidx[2*i+1]], y1 = (float)tny[tidx[2*i+1]];
    float tx = x1 - x0, ty = y1 - y0;
    const float len = sqrtf(tx*tx + ty*ty);
    tx = (float)(tx * (1.0 / len));
    ty = (float)(ty * (1.0 / len));
    const float nxv = -ty, nyv = tx;
    if (i == 0) len0 = len;
    const int q = (int)(len / (1.2 * len0));
    const int nshed = 1 + (q > 0 ? q : 0);
    for (int j = 0; j < nshed && m < tnp; ++j, ++m) {
      const float w = (float)(1 + 2*j) / (float)(2*nshed);
      px[m] = (R)(float)((double)(w * x1) + (1.0 - w) * x0 + (double)(off * nxv));
      py[m] = (R)(float)((double)(w * y1) + (1.0 - w) * y0 + (double)(off * nyv));
    }
  }
  SFX(o_panels_affect_points)(snx, sny, snp, sidx, vs, ss, tnp, px, py, qu, qv);
  for (int i = 0; i < tnp; ++i) { pu[i] += qu[i]; pv[i] += qv[i]; }
  free(px); free(py); free(qu); free(qv);
}

/* ElementBase::move with one weight 1.0 (src/ElementBase.h:276-296): x += (S)h * 1.0 * u,
 * the product formed in double; into (xo, yo) */
static void SFX(move_one)(int n, const R* x, const R* y, const R* u, const R* v, double h, R* xo, R* yo) {
  const double hs = (double)(R)h;
  for (int i = 0; i < n; ++i) {
    xo[i] = (R)((double)x[i] + hs * (double)u[i]);
    yo[i] = (R)((double)y[i] + hs * (double)v[i]);
  }
}

/* ElementBase::move with two or three weights (src/ElementBase.h:299-359): u = sum w_k u_k in
 * double, stored as S; x += (S)dt * u (one fused multiply-add, as the reference's optimised
 * build contracts it) */
static void SFX(move_comb)(int n, R* x, R* y, double dt, int nw, const double* w, R* const* us, R* const* vs) {
  for (int i = 0; i < n; ++i) {
    double cu = w[0] * us[0][i], cv = w[0] * vs[0][i];
    for (int k = 1; k < nw; ++k) { cu += w[k] * us[k][i]; cv += w[k] * vs[k][i]; }
    x[i] = FMA((R)dt, (R)cu, x[i]);
    y[i] = FMA((R)dt, (R)cv, y[i]);
  }
}

/* Convection::advect_2nd_heun without bodies (src/Convection.h:310-387):
 * y = x + dt u(x); x += dt (1/2 u(x) + 1/2 u(y)) */
void SFX(o_advect_2nd_heun)(int core, int n, R* x, R* y, const R* r, const R* s,
                            double fsx, double fsy, double dt, int nsteps) {
  R* buf = (R*)malloc(sizeof(R) * 6 * (size_t)n);
  R *u1 = buf, *v1 = buf + n, *u2 = buf + 2*n, *v2 = buf + 3*n, *x2 = buf + 4*n, *y2 = buf + 5*n;
  const double w[2] = {0.5, 0.5};
  R* const us[2] = {u1, u2};
  R* const vv[2] = {v1, v2};
  for (int k = 0; k < nsteps; ++k) {
    SFX(self_vels)(core, n, x, y, r, s, fsx, fsy, u1, v1);
    SFX(move_one)(n, x, y, u1, v1, dt, x2, y2);
    SFX(self_vels)(core, n, x2, y2, r, s, fsx, fsy, u2, v2);
    SFX(move_comb)(n, x, y, dt, 2, w, us, vv);
  }
  free(buf);
}

/* Convection::advect_3rd without bodies (src/Convection.h:473-598):
 * y1 = x + dt/2 u(x); y2 = x + 3/4 dt u(y1); x += dt (2/9 u(x) + 3/9 u(y1) + 4/9 u(y2)) */
void SFX(o_advect_3rd)(int core, int n, R* x, R* y, const R* r, const R* s,
                       double fsx, double fsy, double dt, int nsteps) {
  R* buf = (R*)malloc(sizeof(R) * 10 * (size_t)n);
  R *u1 = buf, *v1 = buf + n, *u2 = buf + 2*n, *v2 = buf + 3*n, *u3 = buf + 4*n, *v3 = buf + 5*n;
  R *x1 = buf + 6*n, *y1 = buf + 7*n, *x2 = buf + 8*n, *y2 = buf + 9*n;
  const double w[3] = {2.0 / 9.0, 3.0 / 9.0, 4.0 / 9.0};
  R* const us[3] = {u1, u2, u3};
  R* const vv[3] = {v1, v2, v3};
  for (int k = 0; k < nsteps; ++k) {
    SFX(self_vels)(core, n, x, y, r, s, fsx, fsy, u1, v1);
    SFX(move_one)(n, x, y, u1, v1, 0.5 * dt, x1, y1);
    SFX(self_vels)(core, n, x1, y1, r, s, fsx, fsy, u2, v2);
    SFX(move_one)(n, x, y, u2, v2, 0.75 * dt, x2, y2);
    SFX(self_vels)(core, n, x2, y2, r, s, fsx, fsy, u3, v3);
    SFX(move_comb)(n, x, y, dt, 3, w, us, vv);
  }
  free(buf);
}

/* ---------------------------------------------------------------- clear_inner_panp2
 * src/Reflect.h:491-729 (with panel_point_distance :111-165, init_cut_tables :383-443,
 * get_cut_entry :448-480 and the panel normals of Surfaces::compute_bases, src/Surfaces.h:
 * 682-724).  The reference's C++ promotions are spelled out: std::pow(S, 2) and the 1.0
 * literals are double, so those sub-expressions are formed in double and rounded to R where
 * the reference stores them. */

/* closest point of the segment (x0,y0)-(x1,y1) to (tx,ty): kind 0 interior, 1 a node (which) */
static inline void SFX(seg_closest)(R x0, R y0, R x1, R y1, R tx, R ty, R* d2, R* cx, R* cy, int* kind,
                                    int* which) {
  const R bx = x1 - x0, by = y1 - y0;
  const R blensq = bx * bx + by * by;
  const R ax = tx - x0, ay = ty - y0;
  const R t = (ax * bx + ay * by) / blensq;
  if (t > 0.0 && t < 1.0) {
    const R c = ay * bx - ax * by;
    *d2 = (R)(((double)c * (double)c) / (double)blensq);
    *cx = (R)((1.0 - (double)t) * (double)x0 + (double)(t * x1));
    *cy = (R)((1.0 - (double)t) * (double)y0 + (double)(t * y1));
    *kind = 0;
    *which = -1;
    return;
  }
  const R ex = tx - x1, ey = ty - y1;
  const R r0 = (R)((double)ax * (double)ax + (double)ay * (double)ay);
  const R r1 = (R)((double)ex * (double)ex + (double)ey * (double)ey);
  *kind = 1;
  if (r0 < r1) { *which = 0; *d2 = r0; *cx = x0; *cy = y0; }
  else { *which = 1; *d2 = r1; *cx = x1; *cy = y1; }
}

/* init_cut_tables(0.1): entries (position in core radii, strength kept, shift in core radii) */
#define CUT_N 63
static void SFX(cut_tables)(R* pos, R* keep, R* shift) {
  const R max_rad = (R)3.0, dx_in = (R)0.1;
  const int nx = (int)(0.5 + (double)(max_rad / dx_in));
  const R dx = max_rad / (R)(float)nx;
  int k = 0;
  pos[k] = (R)(-nx - 0.5) * dx; keep[k] = 0; shift[k] = 0; ++k;
  R twgt = 0, tmom = 0;
  for (int i = -nx; i < nx + 1; ++i) {
    const R pi_ = (R)i * dx;
    const R distxs = (R)((double)pi_ * (double)pi_);
    R rwgt = 0;
    for (int j = -nx; j < nx + 1; ++j) {
      const R pj = (R)j * dx;
      const R distxys = (R)((double)distxs + (double)pj * (double)pj);
      rwgt += EXP(-distxys);
    }
    rwgt = (R)((double)rwgt * ((double)dx * (double)dx));
    rwgt = (R)((double)rwgt * (1.0 / M_PI));
    twgt += rwgt;
    tmom += ((R)i * dx) * rwgt;
    pos[k] = (R)(i + 0.5) * dx; keep[k] = twgt; shift[k] = -tmom / twgt; ++k;
  }
  pos[k] = (R)(nx + 1.5) * dx; keep[k] = 1; shift[k] = 0;
}

static void SFX(cut_entry)(const R* pos, const R* keep, const R* shift, R p, R* smult, R* dshift) {
  *smult = 1;
  *dshift = 0;
  if (p < pos[0]) {
    *smult = 0;
    *dshift = (R)(1.0 - (double)p);
  } else if (p > pos[CUT_N - 1]) {
    return;
  } else {
    for (int i = 1; i < CUT_N; ++i) {
      if (p < pos[i]) {
        const R frac = (p - pos[i - 1]) / (pos[i] - pos[i - 1]);
        *smult = (R)((double)(frac * keep[i]) + (1.0 - (double)frac) * (double)keep[i - 1]);
        *dshift = (R)((double)(frac * shift[i]) + (1.0 - (double)frac) * (double)shift[i - 1]);
        return;
      }
    }
  }
}

/* One body's panels clear the particles (r given) or field points (r NULL) lying within the
 * cutoff layer: method 0 crops strength and shifts outward with the cut tables, method 1
 * pushes the point onto the layer (src/Reflect.h:644-696).  Each sweep visits the untested
 * points in order (the reference's OpenMP loop run on one thread); a point stays untested while
 * it is modified.  Returns the circulation removed (method 0, particles); *ncropped counts the
 * modifications.  Method 0 on field points never terminates in the reference and is refused
 * here (returns NAN). */
double SFX(o_clear_inner)(int method, R cutoff_mult, R ips, int nnodes, const R* nx, const R* ny, int npan,
                          const unsigned* idx, int n, R* x, R* y, R* s, const R* r, long* ncropped) {
  const int fld = (r == NULL);
  if ((method == 0 && fld) || npan <= 0) return NAN;
  R* pn = (R*)calloc(2 * (size_t)npan + 2 * (size_t)nnodes, sizeof(R));
  R *pnx = pn, *pny = pn + npan, *nnx = pn + 2 * npan, *nny = nnx + nnodes;
  for (int j = 0; j < npan; ++j) {
    const unsigned a = idx[2 * j], b = idx[2 * j + 1];
    R tx1 = nx[b] - nx[a], ty1 = ny[b] - ny[a];
    const R base = SQRT(tx1 * tx1 + ty1 * ty1);
    tx1 = (R)((double)tx1 * (1.0 / (double)base));
    ty1 = (R)((double)ty1 * (1.0 / (double)base));
    pnx[j] = -ty1;
    pny[j] = tx1;
  }
  for (int j = 0; j < npan; ++j) {
    const unsigned a = idx[2 * j], b = idx[2 * j + 1];
    nnx[a] += pnx[j]; nny[a] += pny[j];
    nnx[b] += pnx[j]; nny[b] += pny[j];
  }
  R cpos[CUT_N], ckeep[CUT_N], cshift[CUT_N];
  SFX(cut_tables)(cpos, ckeep, cshift);
  unsigned char* untested = (unsigned char*)malloc((size_t)n + 1);
  memset(untested, 1, (size_t)n + 1);
  const R big = (R)(0.1 * (double)(sizeof(R) == 4 ? 3.40282347e+38 : 1.7976931348623157e+308));
  R circ = 0;
  long crop = 0;
  for (;;) {
    int any = 0;
    for (int i = 0; i < n; ++i) any |= untested[i];
    if (!any) break;
    R part = 0;
    for (int i = 0; i < n; ++i) {
      if (!untested[i]) continue;
      R mind = big, snx = 0, sny = 0, scx = 0, scy = 0;
      int cnt = 0;
      for (int j = 0; j < npan; ++j) {
        const unsigned a = idx[2 * j], b = idx[2 * j + 1];
        R d2, cx, cy;
        int kind, which;
        SFX(seg_closest)(nx[a], ny[a], nx[b], ny[b], x[i], y[i], &d2, &cx, &cy, &kind, &which);
        int add = 0;
        if ((double)d2 < nextafter((double)mind, 0.0)) {          /* a new closest */
          mind = d2;
          snx = sny = scx = scy = 0;
          cnt = 0;
          add = 1;
        } else if (d2 < NEXTAFTER(mind, big * (R)10)) {            /* a tie */
          add = 1;
        }
        if (add) {
          if (kind == 0) { snx += pnx[j]; sny += pny[j]; }
          else { const unsigned nd = which ? b : a; snx += nnx[nd]; sny += nny[nd]; }
          scx += cx; scy += cy;
          ++cnt;
        }
      }
      if (cnt == 0) { untested[i] = 0; continue; }
      const R normilen = (R)(1.0 / (double)SQRT(snx * snx + sny * sny));
      snx *= normilen;
      sny *= normilen;
      scx /= (R)cnt;
      scy /= (R)cnt;
      const R dotp = snx * (x[i] - scx) + sny * (y[i] - scy) - cutoff_mult * ips;
      const R rad = fld ? ips : r[i];
      if (method == 0) {
        if (dotp < rad) {
          R smult, dshift;
          SFX(cut_entry)(cpos, ckeep, cshift, dotp / rad, &smult, &dshift);
          part = (R)((double)part + (double)s[i] * (1.0 - (double)smult));
          s[i] *= smult;
          x[i] += dshift * rad * snx;
          y[i] += dshift * rad * sny;
          ++crop;
        } else {
          untested[i] = 0;
        }
      } else {
        if ((double)dotp < -0.001 * (double)ips) {
          x[i] -= dotp * snx;
          y[i] -= dotp * sny;
          ++crop;
        } else {
          untested[i] = 0;
        }
      }
    }
    circ += part;
  }
  free(untested);
  free(pn);
  if (ncropped) *ncropped = crop;
  return (double)circ;
}
#undef CUT_N
