"""GPU tests of the blob-vorticity sum (src/InfluenceVort.h), panels on panels
(src/Influence.h:774-795), the RK3 / Heun integrators (src/Convection.h:310-598), their
checkpointed reverse, and the recorded-forward tape, through the C ABI."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_blob_vorticity_golden(ctx, golden, accum):
    g = golden("extras")
    t = og.Points(g["tx"], g["ty"])
    t.vort = np.array(g["tw0"])
    og.points_affect_points_vorticity(og.Points(g["sx"], g["sy"], g["sr"], g["ss"]), t, og.ExecEnv(accum=accum,
                                                                                                    context=ctx))
    assert rel_err(g["vort_w"], t.vort) < (2e-6 if accum == og.COMPENSATED else 2e-5)


@pytest.mark.parametrize("uniform", [True, False])
def test_blob_vorticity_vs_fp64_and_finalize(ctx, restatement, uniform):
    rng = np.random.default_rng(5 + uniform)
    ns, nt = 6000, 3001
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = np.full(ns, 0.03, np.float32) if uniform else rng.uniform(0.01, 0.05, ns).astype(np.float32)
    ss = rng.normal(0, 1e-2, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tx[:50], ty[:50] = sx[:50], sy[:50]
    w64 = restatement.points_affect_points_vorticity(sx, sy, sr, ss, tx, ty, fp64=True)
    t = og.Points(tx, ty)
    og.points_affect_points_vorticity(og.Points(sx, sy, sr, ss), t, og.ExecEnv(context=ctx))
    assert rel_err(w64, t.vort) < 2e-6
    t2 = og.Points(tx, ty)
    og.points_affect_points_vorticity(og.Points(sx, sy, sr, ss), t2, og.ExecEnv(context=ctx), finalize=True)
    assert rel_err(w64 / (2 * np.pi), t2.vort) < 2e-6


def test_blob_vorticity_device_path(ctx, restatement):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(9)
    ns, nt = 4000, 2500
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = np.full(ns, 0.02, np.float32)
    ss = rng.normal(0, 1e-2, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    dev = torch.device("cuda", 0)
    T = [torch.from_numpy(a).to(dev) for a in (sx, sy, sr, ss, tx, ty)]
    W = torch.zeros(nt, device=dev)
    og.points_affect_points_vorticity_dev(ctx, og.COMPENSATED, *T, W)
    ctx.synchronize()
    w64 = restatement.points_affect_points_vorticity(sx, sy, sr, ss, tx, ty, fp64=True)
    assert rel_err(w64, W.cpu().numpy()) < 2e-6


@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_panels_affect_panels_golden(ctx, golden, accum):
    """An uneven open polyline as target: long panels shed several collocation points and the
    first npan point velocities go to the npan panels, as in the reference."""
    g = golden("extras")
    src = og.Surfaces(g["snx"], g["sny"], g["sidx"], vs=g["vs"], ss=g["sss"])
    tgt = og.Surfaces(g["tnx"], g["tny"], g["tidx"], pu=np.array(g["pu0"]), pv=np.array(g["pv0"]))
    og.panels_affect_panels(src, tgt, og.ExecEnv(accum=accum, context=ctx))
    assert rel_err(g["pap_u"], tgt.pu) < 2e-5 and rel_err(g["pap_v"], tgt.pv) < 2e-5


def test_panels_affect_panels_two_bodies_vs_fp64(ctx, restatement):
    rng = np.random.default_rng(12)
    src = og.circle_panels(700)
    src.vs = rng.normal(0, 1, 700).astype(np.float32)
    src.ss = rng.normal(0, 1, 700).astype(np.float32)
    tgt = og.circle_panels(513, diameter=0.6, center=(1.2, 0.3))
    og.panels_affect_panels(src, tgt, og.ExecEnv(context=ctx))
    pu, pv = restatement.panels_affect_panels(src.nx, src.ny, src.idx, src.vs, src.ss, tgt.nx, tgt.ny, tgt.idx,
                                              fp64=True)
    # far-field panels: log(r0^2/r1^2) of a ratio near 1 in FP32 (the reference's float build is
    # 1.4e-4 / 2.0e-4 off FP64 on this case; the engine 3e-5)
    assert rel_err(pu, tgt.pu) < 1e-4 and rel_err(pv, tgt.pv) < 1e-4


@pytest.mark.parametrize("order,key,core,fs", [(og.ADVECT_RK3, "rk3", og.CORE_GAUSSIAN, (0.5, 0.0)),
                                               (og.ADVECT_RK2_HEUN, "heun", og.CORE_RM, (0.0, 0.25))])
def test_rk3_heun_match_reference_trajectories(ctx, golden, order, key, core, fs):
    g = golden("extras")
    p = og.Points(g["x"], g["y"], g["r"], g["s"])
    og.advect(p, fs=fs, dt=0.01, nsteps=4, order=order, env=og.ExecEnv(core, og.COMPENSATED, ctx))
    disp = np.max(np.hypot(g[key + "_x"] - g["x"], g[key + "_y"] - g["y"]))
    assert np.max(np.hypot(p.x - g[key + "_x"], p.y - g[key + "_y"])) < 2e-5 * disp


def _two_patches(n, seed=3):
    rng = np.random.default_rng(seed)
    lab = (np.arange(n) % 2).astype(np.int32)
    cx = np.where(lab == 0, -0.3, 0.3)
    x = cx + rng.normal(0, 0.1, n)
    y = rng.normal(0, 0.1, n)
    w = np.exp(-((x - cx) ** 2 + y ** 2) / (2 * 0.1 ** 2))
    s = np.where(lab == 0, w / w[lab == 0].sum(), w / w[lab == 1].sum())
    return x.astype(np.float32), y.astype(np.float32), s.astype(np.float32), lab


def _centroid_loss(restatement, x, y, s, lab):
    n = x.size
    gx, gy, gs = np.zeros(n), np.zeros(n), np.zeros(n)
    L = restatement.lib.o_centroid_loss_d(n, po._p(np.ascontiguousarray(x, np.float64)),
                                          po._p(np.ascontiguousarray(y, np.float64)),
                                          po._p(np.ascontiguousarray(s, np.float64)), po._p(lab), po._p(gx),
                                          po._p(gy), po._p(gs))
    return L, gx, gy, gs


@pytest.mark.parametrize("order", [og.ADVECT_RK3, og.ADVECT_RK2_HEUN, og.ADVECT_EULER])
def test_advect_vjp_new_schemes_vs_fp64_differences(ctx, restatement, order):
    """dL/dG (through the trajectory + the loss's own dependence) and dL/dx0 against FP64
    central differences of the restatement's FP64 forward."""
    n, K, dt = 240, 5, 0.01
    x, y, s, lab = _two_patches(n)
    r = np.full(n, 0.05, np.float32)
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    p = og.Points(x, y, r, s)
    og.advect(p, dt=dt, nsteps=K, order=order, env=env)
    L, gxT, gyT, gs_direct = _centroid_loss(restatement, p.x, p.y, s, lab)
    gs, gx0, gy0, _ = og.advect_vjp(og.Points(x, y, r, s), gxT, gyT, dt=dt, nsteps=K, order=order,
                                    checkpoint_every=2, env=env)
    gs_tot = gs + gs_direct

    def loss(xx, yy, ss):
        xf, yf = restatement.advect(order, po.GAUSS, xx, yy, r, ss, (0.0, 0.0), dt, K, fp64=True)
        return _centroid_loss(restatement, xf, yf, ss, lab)[0]

    rng = np.random.default_rng(order)
    x64, y64, s64 = x.astype(np.float64), y.astype(np.float64), s.astype(np.float64)
    scale_s = np.max(np.abs(gs_tot))
    scale_x = np.max(np.abs(gx0))
    for i in rng.choice(n, 6, replace=False):
        h = 1e-6 * max(1.0, abs(s64[i]))
        sp, sm = s64.copy(), s64.copy()
        sp[i] += h
        sm[i] -= h
        fd = (loss(x64, y64, sp) - loss(x64, y64, sm)) / (2 * h)
        assert abs(fd - gs_tot[i]) < 2e-3 * scale_s, (i, fd, gs_tot[i])
        hx = 1e-6
        xp, xm = x64.copy(), x64.copy()
        xp[i] += hx
        xm[i] -= hx
        fdx = (loss(xp, y64, s64) - loss(xm, y64, s64)) / (2 * hx)
        assert abs(fdx - gx0[i]) < 2e-3 * scale_x, (i, fdx, gx0[i])


@pytest.mark.parametrize("order", [1, 2, 3, 4])
def test_recorded_tape_matches_one_shot_vjp(ctx, order):
    torch = pytest.importorskip("torch")
    n, K, dt = 3000, 6, 0.01
    x, y, s, _ = _two_patches(n, seed=order)
    r = np.full(n, 0.04, np.float32)
    dev = torch.device("cuda", 0)
    X0, Y0, R, S = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    rng = np.random.default_rng(order)
    LX, LY = [torch.from_numpy(a).to(dev) for a in rng.normal(size=(2, n)).astype(np.float32)]
    a = [torch.zeros(n, device=dev) for _ in range(3)]
    og.advect_vjp_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, order, X0, Y0, R, S, (0.1, 0.0), dt, K, 4, LX, LY, *a)
    X, Y = X0.clone(), Y0.clone()
    og.advect_record_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, order, X, Y, R, S, (0.1, 0.0), dt, K, 4)
    Xf, Yf = X0.clone(), Y0.clone()
    og.advect_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, order, Xf, Yf, R, S, (0.1, 0.0), dt, K)
    b = [torch.zeros(n, device=dev) for _ in range(3)]
    launches = ctx.launches
    og.advect_vjp_tape_dev(ctx, LX, LY, *b)
    ck_launches = ctx.launches - launches
    c = [torch.zeros(n, device=dev) for _ in range(3)]
    og.advect_vjp_tape_dev(ctx, LX, LY, *c)                  # the tape can be replayed
    # full tape: every step's positions and stage positions kept, nothing recomputed
    X2, Y2 = X0.clone(), Y0.clone()
    og.advect_record_dev(ctx, og.CORE_GAUSSIAN, og.COMPENSATED, order, X2, Y2, R, S, (0.1, 0.0), dt, K, og.TAPE_ALL)
    d = [torch.zeros(n, device=dev) for _ in range(3)]
    launches = ctx.launches
    og.advect_vjp_tape_dev(ctx, LX, LY, *d)
    full_launches = ctx.launches - launches
    ctx.synchronize()
    assert torch.equal(X, Xf) and torch.equal(Y, Yf)        # recording moves like advect_dev
    assert torch.equal(X2, Xf) and torch.equal(Y2, Yf)
    for u, v, w, z in zip(a, b, c, d):
        assert torch.equal(u, v) and torch.equal(v, w) and torch.equal(u, z)
    assert 0 < full_launches < ck_launches                 # no recomputed velocity sums


def test_tape_required(ctx):
    torch = pytest.importorskip("torch")
    other = og.Context(0)
    z = torch.zeros(4, device="cuda")
    with pytest.raises(og.EngineError):
        og.advect_vjp_tape_dev(other, z, z, z, z, z)
    other.close()


@pytest.mark.parametrize("which,code", [(0, 901), (1, 700)])
def test_bounded_wait_gives_up_and_context_stays_usable(restatement, which, code):
    """Failure path of the device waits, made without a fault: an mbarrier phase with no
    arrival (0) and a grid barrier waiting for one block more than the grid (1) give up after
    their poll limit, record where, and the host reads OBS_ERR_TIMEOUT; the same context then
    computes a correct sum."""
    ctx = og.Context()
    assert ctx.selftest_bounded_wait(which, 64 if which == 0 else 2000) == -4   # OBS_ERR_TIMEOUT
    bits, got_code, _, _ = ctx.last_failure()
    assert bits & 1 and got_code == code
    rng = np.random.default_rng(3)
    sx, sy = rng.uniform(-1, 1, (2, 2000)).astype(np.float32)
    sr = np.full(2000, 0.02, np.float32)
    ss = rng.normal(0, 1e-3, 2000).astype(np.float32)
    t = og.Points(sx, sy, sr, None)
    og.points_affect_points(og.Points(sx, sy, sr, ss), t, og.VELONLY, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    u64, v64, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, sx, sy, sr, fp64=True)
    assert rel_err(u64, t.u) < 2e-6 and rel_err(v64, t.v) < 2e-6
    assert ctx.selftest_bounded_wait(which, 0) == -1                            # OBS_ERR_ARG
