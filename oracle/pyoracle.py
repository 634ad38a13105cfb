"""numpy front-end to the oracle libraries (TEST INFRASTRUCTURE ONLY).

* ``Restatement`` wraps oracle/liboracle.so (oracle.c): the C restatement of the reference's
  direct-sum path in reference semantics (float pairs + double accumulators, ``*_f``) and in
  FP64 (``*_d``), plus FP64 adjoint references.
* ``Reference`` wraps oracle/_ref/libref_<core>.so: the reference's own code compiled from its
  sources (only where the reference tree exists).

Only tests/, __graft_entry__.smoke() and bench.py's CPU arms may import this module; the
engine package never does.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_DIR = os.path.join(HERE, "_ref")

# core ids (same numbering as include/omega2d_gb300.h)
RM, GAUSS, V2, WL, V3, SINGULAR, CEXP = 1, 2, 3, 4, 5, 6, 7
CORE_TO_REF = {RM: "rm", GAUSS: "exp", V2: "v2", WL: "wl", V3: "v3"}
VELONLY, VELANDGRAD, PSIONLY, VELANDVORT, VELANDSHEAR = 1, 2, 3, 4, 5

_vp = ctypes.c_void_p


def build(force: bool = False) -> str:
    """Compile oracle.c into liboracle.so (portable flags: runs on x86 and aarch64)."""
    src = os.path.join(HERE, "oracle.c")
    impl = os.path.join(HERE, "oracle_impl.h")
    if (not force and os.path.exists(LIB)
            and os.path.getmtime(LIB) > max(os.path.getmtime(src), os.path.getmtime(impl))):
        return LIB
    # no contraction into fused multiply-adds, on x86 and aarch64 alike (GCC fuses by default
    # where the ISA has FMA): every product and sum rounds as written
    subprocess.run(["gcc", "-O3", "-fopenmp", "-fPIC", "-shared", "-std=gnu11", "-ffp-contract=off",
                    src, "-o", LIB, "-lm"], check=True)
    return LIB


LIB_NATIVE = os.path.join(HERE, "liboracle_native.so")


def build_native(force: bool = False) -> str:
    """Compile oracle.c once more with the reference's Release flags (CMakeLists.txt:57:
    -O3 -march=native, OpenMP; -mcpu=native on aarch64) into liboracle_native.so: the timed CPU
    baseline.  The checker (liboracle.so) keeps the portable, non-fused build."""
    import platform
    src = os.path.join(HERE, "oracle.c")
    impl = os.path.join(HERE, "oracle_impl.h")
    if (not force and os.path.exists(LIB_NATIVE)
            and os.path.getmtime(LIB_NATIVE) > max(os.path.getmtime(src), os.path.getmtime(impl))):
        return LIB_NATIVE
    arch = "-mcpu=native" if platform.machine().lower() in ("aarch64", "arm64") else "-march=native"
    subprocess.run(["gcc", "-O3", arch, "-fopenmp", "-fPIC", "-shared", "-std=gnu11",
                    src, "-o", LIB_NATIVE, "-lm"], check=True)
    return LIB_NATIVE


def _p(a):
    return None if a is None else a.ctypes.data_as(_vp)


def _arr(a, dt):
    return None if a is None else np.ascontiguousarray(a, dtype=dt)


class Restatement:
    def __init__(self, native: bool = False):
        """native: the build with the reference's Release flags (the timed CPU baseline)."""
        path = build_native() if native else (LIB if os.path.exists(LIB) else build())
        self.native = native
        self.lib = ctypes.CDLL(path)
        for name in ("o_centroid_loss_d", "o_rk2_centroid_grad_d", "o_rk2_centroid_loss_d"):
            getattr(self.lib, name).restype = ctypes.c_double

    # ---- points on points
    def points_affect_points(self, core, restype, sx, sy, sr, ss, tx, ty, tr=None,
                             fp64=False, tu=None, tv=None, extra=None):
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, tx, ty, tr = (_arr(a, dt) for a in (sx, sy, sr, ss, tx, ty, tr))
        nt = tx.size
        tu = np.zeros(nt, dt) if tu is None else np.array(tu, dtype=dt)
        tv = np.zeros(nt, dt) if tv is None else np.array(tv, dtype=dt)
        nex = {1: 0, 2: 4, 3: 1, 4: 1, 5: 1}[restype]
        ex = [np.zeros(nt, dt) for _ in range(nex)] if extra is None else [np.array(e, dtype=dt) for e in extra]
        ptrs = [_p(e) for e in ex] + [None] * (4 - len(ex))
        fn = self.lib.o_points_affect_points_d if fp64 else self.lib.o_points_affect_points_f
        fn(ctypes.c_int(core), ctypes.c_int(restype), ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss),
           ctypes.c_int(nt), _p(tx), _p(ty), _p(tr), _p(tu), _p(tv), *ptrs)
        return tu, tv, ex

    # ---- panels
    def panels_affect_points(self, nx, ny, idx, vs, ss, tx, ty, fp64=False):
        dt = np.float64 if fp64 else np.float32
        nx, ny, vs, ss, tx, ty = (_arr(a, dt) for a in (nx, ny, vs, ss, tx, ty))
        idx = _arr(idx, np.uint32)
        tu = np.zeros(tx.size, dt); tv = np.zeros(tx.size, dt)
        fn = self.lib.o_panels_affect_points_d if fp64 else self.lib.o_panels_affect_points_f
        fn(_p(nx), _p(ny), ctypes.c_int(vs.size), _p(idx), _p(vs), _p(ss),
           ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tu), _p(tv))
        return tu, tv

    def points_affect_panels(self, sx, sy, ss, nx, ny, idx, fp64=False):
        dt = np.float64 if fp64 else np.float32
        sx, sy, ss, nx, ny = (_arr(a, dt) for a in (sx, sy, ss, nx, ny))
        idx = _arr(idx, np.uint32)
        npan = idx.size // 2
        pu = np.zeros(npan, dt); pv = np.zeros(npan, dt)
        fn = self.lib.o_points_affect_panels_d if fp64 else self.lib.o_points_affect_panels_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(ss), _p(nx), _p(ny), ctypes.c_int(npan), _p(idx),
           _p(pu), _p(pv))
        return pu, pv

    def panels_on_panels_coeff(self, nunk, nx, ny, idx, fp64=False, self_block=True,
                               tnx=None, tny=None, tidx=None):
        dt = np.float64 if fp64 else np.float32
        nx, ny = _arr(nx, dt), _arr(ny, dt)
        idx = _arr(idx, np.uint32)
        if tnx is None:
            tnx, tny, tidx = nx, ny, idx
        else:
            tnx, tny, tidx = _arr(tnx, dt), _arr(tny, dt), _arr(tidx, np.uint32)
        ns, nt = idx.size // 2, tidx.size // 2
        out = np.zeros(ns * nunk * nt * nunk, dt)
        fn = self.lib.o_panels_on_panels_coeff_d if fp64 else self.lib.o_panels_on_panels_coeff_f
        fn(ctypes.c_int(nunk), ctypes.c_int(1 if self_block else 0), _p(nx), _p(ny), ctypes.c_int(ns), _p(idx),
           _p(tnx), _p(tny), ctypes.c_int(nt), _p(tidx), _p(out))
        # column-major (targets are rows) -> (nrows, ncols) array
        return out.reshape(ns * nunk, nt * nunk).T.copy()

    def vels_to_rhs_panels(self, nunk, nx, ny, idx, pu, pv, bcn=None, fp64=False):
        dt = np.float64 if fp64 else np.float32
        nx, ny, pu, pv, bcn = (_arr(a, dt) for a in (nx, ny, pu, pv, bcn))
        idx = _arr(idx, np.uint32)
        npan = idx.size // 2
        rhs = np.zeros(npan * nunk, dt)
        fn = self.lib.o_vels_to_rhs_panels_d if fp64 else self.lib.o_vels_to_rhs_panels_f
        fn(ctypes.c_int(nunk), _p(nx), _p(ny), ctypes.c_int(npan), _p(idx), _p(pu), _p(pv), _p(bcn), _p(rhs))
        return rhs

    def finalize_vels(self, u, v, fs, fp64=False):
        dt = np.float64 if fp64 else np.float32
        u = np.array(u, dtype=dt); v = np.array(v, dtype=dt)
        fn = self.lib.o_finalize_vels_d if fp64 else self.lib.o_finalize_vels_f
        fn(ctypes.c_int(u.size), _p(u), _p(v), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]))
        return u, v

    def advect(self, order, core, x, y, r, s, fs, dt_, nsteps, fp64=False):
        dt = np.float64 if fp64 else np.float32
        x = np.array(x, dtype=dt); y = np.array(y, dtype=dt)
        r, s = _arr(r, dt), _arr(s, dt)
        sfx = "_d" if fp64 else "_f"
        name = {1: "o_advect_1st", 2: "o_advect_2nd_ralston", 3: "o_advect_3rd", 4: "o_advect_2nd_heun"}[order]
        fn = getattr(self.lib, name + sfx)
        fn(ctypes.c_int(core), ctypes.c_int(x.size), _p(x), _p(y), _p(r), _p(s),
           ctypes.c_double(fs[0]), ctypes.c_double(fs[1]), ctypes.c_double(dt_), ctypes.c_int(nsteps))
        return x, y

    def points_affect_points_vorticity(self, sx, sy, sr, ss, tx, ty, tw=None, fp64=False):
        """Gaussian-blob vorticity at field points (src/InfluenceVort.h:47-126), accumulated."""
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, tx, ty = (_arr(a, dt) for a in (sx, sy, sr, ss, tx, ty))
        tw = np.zeros(tx.size, dt) if tw is None else np.array(tw, dtype=dt)
        fn = self.lib.o_points_affect_points_vorticity_d if fp64 else self.lib.o_points_affect_points_vorticity_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss), ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tw))
        return tw

    def panels_affect_panels(self, snx, sny, sidx, vs, ss, tnx, tny, tidx, pu=None, pv=None, fp64=False):
        """Panel-centre velocities of the target panels (src/Influence.h:774-795), accumulated."""
        dt = np.float64 if fp64 else np.float32
        snx, sny, vs, ss, tnx, tny = (_arr(a, dt) for a in (snx, sny, vs, ss, tnx, tny))
        sidx, tidx = _arr(sidx, np.uint32), _arr(tidx, np.uint32)
        tnp = tidx.size // 2
        pu = np.zeros(tnp, dt) if pu is None else np.array(pu, dtype=dt)
        pv = np.zeros(tnp, dt) if pv is None else np.array(pv, dtype=dt)
        fn = self.lib.o_panels_affect_panels_d if fp64 else self.lib.o_panels_affect_panels_f
        fn(_p(snx), _p(sny), ctypes.c_int(sidx.size // 2), _p(sidx), _p(vs), _p(ss),
           _p(tnx), _p(tny), ctypes.c_int(tnp), _p(tidx), _p(pu), _p(pv))
        return pu, pv

    # ---- FP64 adjoints
    def probe_vjp(self, core, sx, sy, sr, ss, px, py, lu, lv):
        sx, sy, sr, ss, px, py, lu, lv = (_arr(a, np.float64) for a in (sx, sy, sr, ss, px, py, lu, lv))
        gx = np.zeros(sx.size); gy = np.zeros(sx.size); gs = np.zeros(sx.size)
        self.lib.o_probe_vjp_d(ctypes.c_int(core), ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss),
                               ctypes.c_int(px.size), _p(px), _p(py), _p(lu), _p(lv), _p(gx), _p(gy), _p(gs))
        return gx, gy, gs

    def self_vjp(self, core, x, y, r, s, lu, lv):
        x, y, r, s, lu, lv = (_arr(a, np.float64) for a in (x, y, r, s, lu, lv))
        gx = np.zeros(x.size); gy = np.zeros(x.size); gs = np.zeros(x.size)
        self.lib.o_self_vjp_d(ctypes.c_int(core), ctypes.c_int(x.size), _p(x), _p(y), _p(r), _p(s),
                              _p(lu), _p(lv), _p(gx), _p(gy), _p(gs))
        return gx, gy, gs

    def clear_inner(self, method, cutoff_mult, ips, nx, ny, idx, x, y, s=None, r=None, fp64=False):
        """clear_inner_panp2 (src/Reflect.h:491-729): returns (x, y, s, circulation removed,
        modifications); r None means field points."""
        dt = np.float64 if fp64 else np.float32
        nx, ny = _arr(nx, dt), _arr(ny, dt)
        idx = _arr(idx, np.uint32)
        x, y = np.array(x, dt), np.array(y, dt)
        s = np.array(s, dt) if s is not None else np.zeros(x.size, dt)
        r = _arr(r, dt)
        fn = self.lib.o_clear_inner_d if fp64 else self.lib.o_clear_inner_f
        fn.restype = ctypes.c_double
        cast = ctypes.c_double if fp64 else ctypes.c_float
        nc = ctypes.c_long()
        lost = fn(ctypes.c_int(method), cast(cutoff_mult), cast(ips), ctypes.c_int(nx.size), _p(nx), _p(ny),
                  ctypes.c_int(idx.size // 2), _p(idx), ctypes.c_int(x.size), _p(x), _p(y), _p(s), _p(r),
                  ctypes.byref(nc))
        return x, y, s, lost, nc.value

    def rk2_centroid_grad(self, core, x, y, r, s, label, fs, dt_, nsteps):
        x, y, r, s = (_arr(a, np.float64) for a in (x, y, r, s))
        label = _arr(label, np.int32)
        gs = np.zeros(x.size); gx = np.zeros(x.size); gy = np.zeros(x.size)
        L = self.lib.o_rk2_centroid_grad_d(ctypes.c_int(core), ctypes.c_int(x.size), _p(x), _p(y), _p(r), _p(s),
                                           _p(label), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                           ctypes.c_double(dt_), ctypes.c_int(nsteps), _p(gs), _p(gx), _p(gy))
        return L, gs, gx, gy

    def rk2_centroid_loss(self, core, x, y, r, s, label, fs, dt_, nsteps):
        x, y, r, s = (_arr(a, np.float64) for a in (x, y, r, s))
        label = _arr(label, np.int32)
        return self.lib.o_rk2_centroid_loss_d(ctypes.c_int(core), ctypes.c_int(x.size), _p(x), _p(y), _p(r),
                                              _p(s), _p(label), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
                                              ctypes.c_double(dt_), ctypes.c_int(nsteps))


class Reference:
    """The reference's own compiled code for one core (oracle/_ref/libref_<core>.so)."""

    def __init__(self, core: int):
        path = os.path.join(REF_DIR, f"libref_{CORE_TO_REF[core]}.so")
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = ctypes.CDLL(path)

    @staticmethod
    def available(core: int = V2) -> bool:
        return core in CORE_TO_REF and os.path.exists(os.path.join(REF_DIR, f"libref_{CORE_TO_REF[core]}.so"))

    def points_affect_points(self, restype, sx, sy, sr, ss, tx, ty, tr=None, fp64=False,
                             tu=None, tv=None, extra=None):
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, tx, ty, tr = (_arr(a, dt) for a in (sx, sy, sr, ss, tx, ty, tr))
        nt = tx.size
        tu = np.zeros(nt, dt) if tu is None else np.array(tu, dtype=dt)
        tv = np.zeros(nt, dt) if tv is None else np.array(tv, dtype=dt)
        ex = np.zeros(nt, dt) if extra is None else np.array(extra, dtype=dt)
        fn = self.lib.ref_points_affect_points_d if fp64 else self.lib.ref_points_affect_points_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss), ctypes.c_int(nt), _p(tx), _p(ty), _p(tr),
           ctypes.c_int(restype), _p(tu), _p(tv), _p(ex))
        return tu, tv, ex

    def psi(self, sx, sy, sr, ss, tx, ty, tr=None, fp64=False, tp=None):
        """The reference's streamfunction kernels kernelp_0v_0b / kernelp_0v_0p
        (src/Kernels.h:52-74) in the velonly driver loop; tr None selects the 0p kernel."""
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, tx, ty, tr = (_arr(a, dt) for a in (sx, sy, sr, ss, tx, ty, tr))
        out = np.zeros(tx.size, dt) if tp is None else np.array(tp, dtype=dt)
        fn = self.lib.ref_psi_d if fp64 else self.lib.ref_psi_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss), ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tr),
           _p(out))
        return out

    def velgrad_thick(self, sx, sy, sr, ss, tx, ty, tr, fp64=False):
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, tx, ty, tr = (_arr(a, dt) for a in (sx, sy, sr, ss, tx, ty, tr))
        out = [np.zeros(tx.size, dt) for _ in range(6)]
        fn = self.lib.ref_velgrad_thick_d if fp64 else self.lib.ref_velgrad_thick_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss), ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tr),
           *[_p(o) for o in out])
        return out

    def panels_affect_points(self, nx, ny, idx, vs, ss, tx, ty, fp64=False):
        dt = np.float64 if fp64 else np.float32
        nx, ny, vs, ss, tx, ty = (_arr(a, dt) for a in (nx, ny, vs, ss, tx, ty))
        idx = _arr(idx, np.uint32)
        tu = np.zeros(tx.size, dt); tv = np.zeros(tx.size, dt)
        if ss is None:
            assert not fp64
            self.lib.ref_panels_affect_points_vortex_f(ctypes.c_int(nx.size), _p(nx), _p(ny), ctypes.c_int(vs.size),
                                                       _p(idx), _p(vs), ctypes.c_int(tx.size), _p(tx), _p(ty),
                                                       _p(tu), _p(tv))
        else:
            fn = self.lib.ref_panels_affect_points_d if fp64 else self.lib.ref_panels_affect_points_f
            fn(ctypes.c_int(nx.size), _p(nx), _p(ny), ctypes.c_int(vs.size), _p(idx), _p(vs), _p(ss),
               ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tu), _p(tv))
        return tu, tv

    def points_affect_panels(self, sx, sy, sr, ss, nx, ny, idx, fp64=False):
        dt = np.float64 if fp64 else np.float32
        sx, sy, sr, ss, nx, ny = (_arr(a, dt) for a in (sx, sy, sr, ss, nx, ny))
        idx = _arr(idx, np.uint32)
        npan = idx.size // 2
        pu = np.zeros(npan, dt); pv = np.zeros(npan, dt)
        fn = self.lib.ref_points_affect_panels_d if fp64 else self.lib.ref_points_affect_panels_f
        fn(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss), ctypes.c_int(nx.size), _p(nx), _p(ny),
           ctypes.c_int(npan), _p(idx), _p(pu), _p(pv))
        return pu, pv

    def panels_on_panels_coeff(self, nx, ny, idx, fp64=False):
        dt = np.float64 if fp64 else np.float32
        nx, ny = _arr(nx, dt), _arr(ny, dt)
        idx = _arr(idx, np.uint32)
        npan = idx.size // 2
        out = np.zeros((2 * npan) ** 2, dt)
        fn = self.lib.ref_panels_on_panels_coeff_d if fp64 else self.lib.ref_panels_on_panels_coeff_f
        fn(ctypes.c_int(nx.size), _p(nx), _p(ny), ctypes.c_int(npan), _p(idx), _p(out))
        return out.reshape(2 * npan, 2 * npan).T.copy()

    def panels_on_panels_coeff_pair(self, snx, sny, sidx, tnx, tny, tidx):
        """The reference's block of one body's panels (source) on another body's (target):
        src/Coefficients.h:155-427 with src != targ, so no self term; (rows, cols) array."""
        snx, sny, tnx, tny = (_arr(a, np.float32) for a in (snx, sny, tnx, tny))
        sidx, tidx = _arr(sidx, np.uint32), _arr(tidx, np.uint32)
        snp, tnp = sidx.size // 2, tidx.size // 2
        out = np.zeros(4 * snp * tnp, np.float32)
        self.lib.ref_panels_on_panels_coeff_pair_f(ctypes.c_int(snx.size), _p(snx), _p(sny), ctypes.c_int(snp),
                                                   _p(sidx), ctypes.c_int(tnx.size), _p(tnx), _p(tny),
                                                   ctypes.c_int(tnp), _p(tidx), _p(out))
        return out.reshape(2 * snp, 2 * tnp).T.copy()

    def clear_inner(self, method, cutoff_mult, ips, nx, ny, idx, x, y, s=None, r=None):
        """The reference's clear_inner_panp2 (src/Reflect.h:491-729) on one body: returns
        (x, y, s, circulation removed).  Its sweep is an OpenMP loop with a reduction; run the
        process with OMP_NUM_THREADS=1 for a reproducible circulation sum."""
        nx, ny = _arr(nx, np.float32), _arr(ny, np.float32)
        idx = _arr(idx, np.uint32)
        x, y = np.array(x, np.float32), np.array(y, np.float32)
        s = np.array(s, np.float32) if s is not None else np.zeros(x.size, np.float32)
        r = _arr(r, np.float32)
        fn = self.lib.ref_clear_inner_f
        fn.restype = ctypes.c_float
        lost = fn(ctypes.c_int(method), ctypes.c_float(cutoff_mult), ctypes.c_float(ips), ctypes.c_int(nx.size),
                  _p(nx), _p(ny), ctypes.c_int(idx.size // 2), _p(idx), ctypes.c_int(x.size), _p(x), _p(y), _p(s),
                  _p(r))
        return x, y, s, float(lost)

    def vels_to_rhs_panels(self, nx, ny, idx, pu, pv, bct, bcn):
        nx, ny, pu, pv, bct, bcn = (_arr(a, np.float32) for a in (nx, ny, pu, pv, bct, bcn))
        idx = _arr(idx, np.uint32)
        npan = idx.size // 2
        rhs = np.zeros(2 * npan, np.float32)
        self.lib.ref_vels_to_rhs_panels_f(ctypes.c_int(nx.size), _p(nx), _p(ny), ctypes.c_int(npan), _p(idx),
                                          _p(pu), _p(pv), _p(bct), _p(bcn), _p(rhs))
        return rhs

    def finalize_vels(self, u, v, fs):
        u = np.array(u, dtype=np.float32); v = np.array(v, dtype=np.float32)
        self.lib.ref_finalize_vels_f(ctypes.c_int(u.size), _p(u), _p(v), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]))
        return u, v

    def advect(self, order, x, y, r, s, fs, dt_, nsteps):
        x = np.array(x, dtype=np.float32); y = np.array(y, dtype=np.float32)
        r, s = _arr(r, np.float32), _arr(s, np.float32)
        fn = {1: self.lib.ref_advect_1st_f, 2: self.lib.ref_advect_2nd_ralston_f, 3: self.lib.ref_advect_3rd_f,
              4: self.lib.ref_advect_2nd_heun_f}[order]
        fn(ctypes.c_int(x.size), _p(x), _p(y), _p(r), _p(s), ctypes.c_double(fs[0]), ctypes.c_double(fs[1]),
           ctypes.c_double(dt_), ctypes.c_int(nsteps))
        return x, y

    def points_affect_points_vorticity(self, sx, sy, sr, ss, tx, ty, tw=None):
        sx, sy, sr, ss, tx, ty = (_arr(a, np.float32) for a in (sx, sy, sr, ss, tx, ty))
        tw = np.zeros(tx.size, np.float32) if tw is None else np.array(tw, dtype=np.float32)
        self.lib.ref_points_affect_points_vorticity_f(ctypes.c_int(sx.size), _p(sx), _p(sy), _p(sr), _p(ss),
                                                      ctypes.c_int(tx.size), _p(tx), _p(ty), _p(tw))
        return tw

    def panels_affect_panels(self, snx, sny, sidx, vs, ss, tnx, tny, tidx, pu=None, pv=None):
        snx, sny, vs, ss, tnx, tny = (_arr(a, np.float32) for a in (snx, sny, vs, ss, tnx, tny))
        sidx, tidx = _arr(sidx, np.uint32), _arr(tidx, np.uint32)
        tnp = tidx.size // 2
        pu = np.zeros(tnp, np.float32) if pu is None else np.array(pu, dtype=np.float32)
        pv = np.zeros(tnp, np.float32) if pv is None else np.array(pv, dtype=np.float32)
        self.lib.ref_panels_affect_panels_f(ctypes.c_int(snx.size), _p(snx), _p(sny), ctypes.c_int(sidx.size // 2),
                                            _p(sidx), _p(vs), _p(ss), ctypes.c_int(tnx.size), _p(tnx), _p(tny),
                                            ctypes.c_int(tnp), _p(tidx), _p(pu), _p(pv))
        return pu, pv

    def flop_counts(self):
        out = (ctypes.c_int * 8)()
        self.lib.ref_flop_counts(out)
        keys = ["u_0v_0b", "u_0v_0p", "ug_0v_0b", "uw_0v_0b", "ue_0v_0b", "u_1v_0p", "u_1vs_0p", "u_1vos_0p"]
        return dict(zip(keys, list(out)))
