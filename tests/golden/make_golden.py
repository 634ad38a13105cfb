"""Generate the golden vectors in tests/golden/*.npz from the reference's own compiled code.

Run in a checkout that has the reference tree (it builds oracle/_ref first):

    python tests/golden/make_golden.py

Every fixture stores its seeded inputs and the reference outputs (float32 storage, double
accumulators: the reference's default non-Vc build).  The reference itself has no tests or
fixtures for this path; these vectors are produced by compiling its src/Influence.h,
src/Kernels.h, src/CoreFunc.h, src/Coefficients.h, src/RHS.h and src/Reflect.h unmodified (see
oracle/build_ref.py) and calling its drivers through oracle/ref_harness.cpp.
"""
from __future__ import annotations

import os
import sys

# the reference's clear_inner_panp2 sums the removed circulation in an OpenMP reduction: one
# thread gives a reproducible order (the other fixtures do not depend on the thread count)
os.environ.setdefault("OMP_NUM_THREADS", "1")

import numpy as np  # noqa: E402

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import build_ref, pyoracle as po  # noqa: E402

CORES = {"rm": po.RM, "exp": po.GAUSS, "v2": po.V2, "wl": po.WL, "v3": po.V3}


def particles(rng, n, lo=-1.0, hi=1.0, rmin=0.02, rmax=0.08):
    x = rng.uniform(lo, hi, n).astype(np.float32)
    y = rng.uniform(lo, hi, n).astype(np.float32)
    r = rng.uniform(rmin, rmax, n).astype(np.float32)
    s = rng.normal(0.0, 1.0 / np.sqrt(n), n).astype(np.float32)
    return x, y, r, s


def circle_panels(npan, diameter=1.0):
    """Clockwise circle nodes (fluid to the left walking node0 -> node1), as
    SolidCircle builds them (src/BoundaryFeature.cpp:489-531)."""
    th = -2.0 * np.pi * np.arange(npan) / npan
    nx = (0.5 * diameter * np.cos(th)).astype(np.float32)
    ny = (0.5 * diameter * np.sin(th)).astype(np.float32)
    idx = np.stack([np.arange(npan), (np.arange(npan) + 1) % npan], 1).ravel().astype(np.uint32)
    return nx, ny, idx


def make_p2p(out):
    rng = np.random.default_rng(20240601)
    ns, nt = 257, 193
    sx, sy, sr, ss = particles(rng, ns)
    # targets: 40 coincide with sources (self pairs), the rest are fresh points
    tx, ty, tr, _ = particles(rng, nt)
    tx[:40], ty[:40], tr[:40] = sx[:40], sy[:40], sr[:40]
    tu0 = rng.normal(0, 0.1, nt).astype(np.float32)   # non-zero: the drivers accumulate
    tv0 = rng.normal(0, 0.1, nt).astype(np.float32)
    ex0 = rng.normal(0, 0.1, nt).astype(np.float32)
    d = dict(sx=sx, sy=sy, sr=sr, ss=ss, tx=tx, ty=ty, tr=tr, tu0=tu0, tv0=tv0, ex0=ex0)
    for name, core in CORES.items():
        ref = po.Reference(core)
        for restype in (po.VELONLY, po.VELANDVORT, po.VELANDSHEAR):
            for thick in (True, False):
                tu, tv, ex = ref.points_affect_points(restype, sx, sy, sr, ss, tx, ty, tr if thick else None,
                                                      tu=tu0, tv=tv0, extra=ex0)
                key = f"{name}_r{restype}_{'b' if thick else 'p'}"
                d[key + "_u"], d[key + "_v"] = tu, tv
                if restype != po.VELONLY:
                    d[key + "_e"] = ex
        g = ref.velgrad_thick(sx, sy, sr, ss, tx, ty, tr)
        for k, nm in enumerate(["u", "v", "ux", "vx", "uy", "vy"]):
            d[f"{name}_grad_{nm}"] = g[k]
        d[f"{name}_flops"] = np.array(list(ref.flop_counts().values()), np.int32)
    np.savez_compressed(out, **d)


def make_panels(out):
    rng = np.random.default_rng(20240602)
    npan = 64
    nx, ny, idx = circle_panels(npan)
    vs = rng.normal(0, 1, npan).astype(np.float32)
    ss = rng.normal(0, 1, npan).astype(np.float32)
    nt = 150
    rr = np.sqrt(rng.uniform(0.55 ** 2, 3.0 ** 2, nt))
    aa = rng.uniform(0, 2 * np.pi, nt)
    tx = (rr * np.cos(aa)).astype(np.float32)
    ty = (rr * np.sin(aa)).astype(np.float32)
    tr = np.full(nt, 0.01, np.float32)
    tg = rng.normal(0, 1e-2, nt).astype(np.float32)
    ref = po.Reference(po.V2)
    d = dict(nx=nx, ny=ny, idx=idx, vs=vs, ss=ss, tx=tx, ty=ty, tr=tr, tg=tg)
    d["p2pt_1vs_u"], d["p2pt_1vs_v"] = ref.panels_affect_points(nx, ny, idx, vs, ss, tx, ty)
    d["p2pt_1v_u"], d["p2pt_1v_v"] = ref.panels_affect_points(nx, ny, idx, vs, None, tx, ty)
    d["pt2p_u"], d["pt2p_v"] = ref.points_affect_panels(tx, ty, tr, tg, nx, ny, idx)
    d["coeff"] = ref.panels_on_panels_coeff(nx, ny, idx)
    pu = rng.normal(0, 1, npan).astype(np.float32)
    pv = rng.normal(0, 1, npan).astype(np.float32)
    bcn = rng.normal(0, 0.1, npan).astype(np.float32)
    d["pu"], d["pv"], d["bcn"] = pu, pv, bcn
    d["rhs"] = ref.vels_to_rhs_panels(nx, ny, idx, pu, pv, np.zeros(npan, np.float32), bcn)
    d["fin_u"], d["fin_v"] = ref.finalize_vels(pu, pv, (1.0, -0.5))
    np.savez_compressed(out, **d)


def make_advect(out):
    rng = np.random.default_rng(20240603)
    n = 300
    x, y, _, s = particles(rng, n)
    r = np.full(n, 0.05, np.float32)
    d = dict(x=x, y=y, r=r, s=s)
    d["euler_x"], d["euler_y"] = po.Reference(po.RM).advect(1, x, y, r, s, (1.0, 0.0), 0.01, 10)
    d["rk2_x"], d["rk2_y"] = po.Reference(po.GAUSS).advect(2, x, y, r, s, (0.0, 0.0), 0.01, 4)
    np.savez_compressed(out, **d)


def make_extras(out):
    """Blob vorticity (src/InfluenceVort.h), panels on panels (src/Influence.h:774-795) and the
    Heun / RK3 integrators (src/Convection.h:310-387, 473-598)."""
    rng = np.random.default_rng(20240604)
    ns, nt = 300, 211
    sx, sy, sr, ss = particles(rng, ns)
    tx, ty, _, _ = particles(rng, nt)
    tx[:30], ty[:30] = sx[:30], sy[:30]
    tw0 = rng.normal(0, 0.1, nt).astype(np.float32)
    d = dict(sx=sx, sy=sy, sr=sr, ss=ss, tx=tx, ty=ty, tw0=tw0)
    d["vort_w"] = po.Reference(po.GAUSS).points_affect_points_vorticity(sx, sy, sr, ss, tx, ty, tw0)
    # panels on panels: a circle of 96 panels acting on an uneven open polyline (long panels
    # shed several collocation points, the reference adds the first npan velocities back)
    snx, sny, sidx = circle_panels(96)
    vs = rng.normal(0, 1, 96).astype(np.float32)
    sss = rng.normal(0, 1, 96).astype(np.float32)
    tnx = np.array([0.7, 0.8, 1.2, 1.3, 2.0, 2.0, 2.1], np.float32)
    tny = np.array([0.0, 0.0, 0.05, 0.1, 0.1, 0.5, 0.55], np.float32)
    tidx = np.array([0, 1, 1, 2, 2, 3, 3, 4, 4, 5, 5, 6], np.uint32)
    pu0 = rng.normal(0, 0.1, 6).astype(np.float32)
    pv0 = rng.normal(0, 0.1, 6).astype(np.float32)
    d.update(snx=snx, sny=sny, sidx=sidx, vs=vs, sss=sss, tnx=tnx, tny=tny, tidx=tidx, pu0=pu0, pv0=pv0)
    d["pap_u"], d["pap_v"] = po.Reference(po.V2).panels_affect_panels(snx, sny, sidx, vs, sss, tnx, tny, tidx,
                                                                       pu0, pv0)
    n = 300
    x, y, _, s = particles(rng, n)
    r = np.full(n, 0.05, np.float32)
    d.update(x=x, y=y, r=r, s=s)
    d["rk3_x"], d["rk3_y"] = po.Reference(po.GAUSS).advect(3, x, y, r, s, (0.5, 0.0), 0.01, 4)
    d["heun_x"], d["heun_y"] = po.Reference(po.RM).advect(4, x, y, r, s, (0.0, 0.25), 0.01, 4)
    np.savez_compressed(out, **d)


def make_augment(out):
    """The reference's rotation-augmented self block (src/Coefficients.h:429-572, prepared as
    src/BEMHelper.h:197-205 does) for a circle and an irregular closed polygon."""
    import ctypes
    ref = po.Reference(po.V2)
    d = {}
    rng = np.random.default_rng(20240605)
    th = -2.0 * np.pi * np.sort(rng.uniform(0, 1, 40))
    rad = 0.5 + 0.1 * np.sin(3 * th)
    shapes = {"circle": circle_panels(48),
              "poly": ((0.2 + rad * np.cos(th)).astype(np.float32), (-0.1 + rad * np.sin(th)).astype(np.float32),
                       np.stack([np.arange(40), (np.arange(40) + 1) % 40], 1).ravel().astype(np.uint32))}
    for name, (nx, ny, idx) in shapes.items():
        npan = idx.size // 2
        m = 2 * npan + 1
        A = np.zeros(m * m, np.float32)
        geom = np.zeros(4)
        ref.lib.ref_panels_on_panels_coeff_augmented_f(ctypes.c_int(nx.size), po._p(nx), po._p(ny),
                                                       ctypes.c_int(npan), po._p(idx), po._p(A), po._p(geom))
        d[name + "_nx"], d[name + "_ny"], d[name + "_idx"] = nx, ny, idx
        d[name + "_A"] = A.reshape(m, m).T.copy()     # (rows, cols)
        d[name + "_vol"] = geom[:1]
    np.savez_compressed(out, **d)


def make_bodies(out):
    """Two bodies in one BEM system, assembled block by block as solve_bem does
    (src/BEMHelper.h:166-221): a circle and an irregular closed polygon; block (t, s) is
    panels_on_panels_coeff of body s on body t, the self term only on the diagonal blocks."""
    rng = np.random.default_rng(20240606)
    bodies = []
    nx, ny, idx = circle_panels(36)
    bodies.append((nx, ny, idx))
    th = -2.0 * np.pi * np.sort(rng.uniform(0, 1, 24))
    rad = 0.3 + 0.06 * np.sin(2 * th)
    bodies.append(((1.3 + rad * np.cos(th)).astype(np.float32), (0.4 + rad * np.sin(th)).astype(np.float32),
                   np.stack([np.arange(24), (np.arange(24) + 1) % 24], 1).ravel().astype(np.uint32)))
    ref = po.Reference(po.V2)
    rows = []
    for t in bodies:
        blocks = []
        for s in bodies:
            if s is t:
                blocks.append(ref.panels_on_panels_coeff(*s))
            else:
                blocks.append(ref.panels_on_panels_coeff_pair(*s, *t))
        rows.append(np.concatenate(blocks, axis=1))
    d = {"A": np.concatenate(rows, axis=0)}
    for k, (nx, ny, idx) in enumerate(bodies):
        d[f"nx{k}"], d[f"ny{k}"], d[f"idx{k}"] = nx, ny, idx
    np.savez_compressed(out, **d)


def make_bodies_aug(out):
    """Two rotating bodies in one BEM system, assembled as solve_bem does (src/BEMHelper.h:
    166-221): block (t, s) is panels_on_panels_coeff of body s on body t with both augmented
    (src/Coefficients.h:429-572; the source's unit-rotation sheet acting on the target's panels
    supplies the augmented column), each body's rows and columns followed by its rotation row
    and column.  Stored in the reference's order with the bodies' volumes."""
    import ctypes
    rng = np.random.default_rng(20240609)
    bodies = [circle_panels(36)]
    th = -2.0 * np.pi * np.sort(rng.uniform(0, 1, 24))
    rad = 0.3 + 0.06 * np.sin(2 * th)
    bodies.append(((1.3 + rad * np.cos(th)).astype(np.float32), (0.4 + rad * np.sin(th)).astype(np.float32),
                   np.stack([np.arange(24), (np.arange(24) + 1) % 24], 1).ravel().astype(np.uint32)))
    ref = po.Reference(po.V2)
    d = {}
    rows = []
    for ti, (tnx, tny, tidx) in enumerate(bodies):
        blocks = []
        tn = tidx.size // 2
        for si, (snx, sny, sidx) in enumerate(bodies):
            sn = sidx.size // 2
            if si == ti:
                m = 2 * sn + 1
                A = np.zeros(m * m, np.float32)
                geom = np.zeros(4)
                ref.lib.ref_panels_on_panels_coeff_augmented_f(ctypes.c_int(snx.size), po._p(snx), po._p(sny),
                                                               ctypes.c_int(sn), po._p(sidx), po._p(A), po._p(geom))
                blocks.append(A.reshape(m, m).T)
                d[f"vol{si}"] = geom[:1]
            else:
                A = np.zeros((2 * tn + 1) * (2 * sn + 1), np.float32)
                ref.lib.ref_panels_on_panels_coeff_augmented_pair_f(
                    ctypes.c_int(snx.size), po._p(snx), po._p(sny), ctypes.c_int(sn), po._p(sidx),
                    ctypes.c_int(tnx.size), po._p(tnx), po._p(tny), ctypes.c_int(tn), po._p(tidx), po._p(A))
                blocks.append(A.reshape(2 * sn + 1, 2 * tn + 1).T)
        rows.append(np.concatenate(blocks, axis=1))
    d["A"] = np.concatenate(rows, axis=0)
    for k, (nx, ny, idx) in enumerate(bodies):
        d[f"nx{k}"], d[f"ny{k}"], d[f"idx{k}"] = nx, ny, idx
    np.savez_compressed(out, **d)


def star_panels(arms=5, r_out=0.5, r_in=0.25, center=(0.0, 0.0)):
    """A clockwise star polygon (concave corners: ties between panels and nodes)."""
    k = 2 * arms
    th = -2.0 * np.pi * np.arange(k) / k
    rad = np.where(np.arange(k) % 2 == 0, r_out, r_in)
    nx = (center[0] + rad * np.cos(th)).astype(np.float32)
    ny = (center[1] + rad * np.sin(th)).astype(np.float32)
    idx = np.stack([np.arange(k), (np.arange(k) + 1) % k], 1).ravel().astype(np.uint32)
    return nx, ny, idx


def make_clear(out):
    """clear_inner_panp2 (src/Reflect.h:491-729) on a circle and a star: particles scattered
    across each surface (method 0 crops, method 1 pushes) and field points (method 1)."""
    rng = np.random.default_rng(20240607)
    ref = po.Reference(po.V2)
    cut = np.float32(0.5 / np.sqrt(2.0 * np.pi))       # Convection.h:301's cutoff factor
    ips = np.float32(0.02)
    d = {"cut": np.array([cut]), "ips": np.array([ips])}
    for name, (nx, ny, idx) in {"circle": circle_panels(64), "star": star_panels()}.items():
        n = 300
        rad = rng.uniform(0.15, 0.65, n)
        a = rng.uniform(0, 2 * np.pi, n)
        x = (rad * np.cos(a)).astype(np.float32)
        y = (rad * np.sin(a)).astype(np.float32)
        s = rng.normal(0, 1, n).astype(np.float32)
        r = rng.uniform(0.015, 0.025, n).astype(np.float32)
        d[name + "_nx"], d[name + "_ny"], d[name + "_idx"] = nx, ny, idx
        d[name + "_x"], d[name + "_y"], d[name + "_s"], d[name + "_r"] = x, y, s, r
        for m in (0, 1):
            ox, oy, os_, lost = ref.clear_inner(m, cut, ips, nx, ny, idx, x, y, s, r)
            d[f"{name}_m{m}_x"], d[f"{name}_m{m}_y"], d[f"{name}_m{m}_s"] = ox, oy, os_
            d[f"{name}_m{m}_lost"] = np.array([lost])
        fx, fy, _, _ = ref.clear_inner(1, np.float32(0.0), ips, nx, ny, idx, x, y, None, None)
        d[name + "_fld_x"], d[name + "_fld_y"] = fx, fy
    np.savez_compressed(out, **d)


def make_pins(out):
    """The streamfunction and the singular core from the reference's own code.

    * psi: kernelp_0v_0b / kernelp_0v_0p (src/Kernels.h:52-74) in the velonly driver loop,
      thick and field-point targets, accumulated onto non-zero starting values.
    * singular: the reference has no separate point-vortex core; it is the Rosenhead-Moore core
      (src/CoreFunc.h:42-82) with zero radii.  libref_rm with sr = tr = 0 on targets that do not
      coincide with any source gives the point-vortex velocity (and, through kernelug_0v_0b, its
      gradient); field-point targets use the 0p kernel with sr = 0."""
    rng = np.random.default_rng(20240608)
    ns, nt = 301, 187
    sx, sy, sr, ss = particles(rng, ns)
    tx, ty, tr, _ = particles(rng, nt)
    tx[:30], ty[:30], tr[:30] = sx[:30], sy[:30], sr[:30]     # coincident pairs (psi is finite there)
    tp0 = rng.normal(0, 0.1, nt).astype(np.float32)
    tu0 = rng.normal(0, 0.1, nt).astype(np.float32)
    tv0 = rng.normal(0, 0.1, nt).astype(np.float32)
    ref = po.Reference(po.RM)
    d = dict(sx=sx, sy=sy, sr=sr, ss=ss, tx=tx, ty=ty, tr=tr, tp0=tp0, tu0=tu0, tv0=tv0)
    d["psi_b"] = ref.psi(sx, sy, sr, ss, tx, ty, tr, tp=tp0)
    d["psi_p"] = ref.psi(sx, sy, sr, ss, tx, ty, None, tp=tp0)
    # singular: off-source targets only (a coincident pair is 0/0 in the reference)
    qx, qy, _, _ = particles(rng, 211)
    z = np.zeros(ns, np.float32)
    zt = np.zeros(qx.size, np.float32)
    d.update(qx=qx, qy=qy)
    for thick in (True, False):
        tu, tv, _ = ref.points_affect_points(po.VELONLY, sx, sy, z, ss, qx, qy, zt if thick else None)
        d[f"sing_{'b' if thick else 'p'}_u"], d[f"sing_{'b' if thick else 'p'}_v"] = tu, tv
    g = ref.velgrad_thick(sx, sy, z, ss, qx, qy, zt)
    for k, nm in enumerate(["u", "v", "ux", "vx", "uy", "vy"]):
        d[f"sing_grad_{nm}"] = g[k]
    np.savez_compressed(out, **d)


def main():
    if not build_ref.available():
        raise SystemExit("the reference tree is needed to generate golden vectors")
    build_ref.build()
    if sys.argv[1:]:
        # named fixtures only, e.g. `make_golden.py pins`
        for name in sys.argv[1:]:
            globals()["make_" + name](os.path.join(HERE, name + ".npz"))
        return
    make_p2p(os.path.join(HERE, "p2p.npz"))
    make_panels(os.path.join(HERE, "panels.npz"))
    make_advect(os.path.join(HERE, "advect.npz"))
    make_extras(os.path.join(HERE, "extras.npz"))
    make_augment(os.path.join(HERE, "augment.npz"))
    make_bodies(os.path.join(HERE, "bodies.npz"))
    make_clear(os.path.join(HERE, "clear.npz"))
    make_pins(os.path.join(HERE, "pins.npz"))
    make_bodies_aug(os.path.join(HERE, "bodies_aug.npz"))
    for f in sorted(os.listdir(HERE)):
        if f.endswith(".npz"):
            print(f, os.path.getsize(os.path.join(HERE, f)))


if __name__ == "__main__":
    main()
