"""GPU tests of the hand-written reverse mode and the device time stepping, through the C ABI.

Pins: the FP64 adjoint references of the oracle (themselves checked by finite differences in
tests/test_oracle.py), FP64 central finite differences of the FP64 forward on 64 seeded
coordinates, and the reference's own Euler/RK2 trajectories (golden vectors)."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu


def probe_case(n=20_000, grid=30, seed=4):
    rng = np.random.default_rng(seed)
    sx, sy = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    sr = np.full(n, 0.01, np.float32)
    ss = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    g = np.linspace(-0.5, 0.5, grid)
    px, py = [a.ravel().astype(np.float32) for a in np.meshgrid(g, g)]
    return sx, sy, sr, ss, px, py


def fp64_probe_loss(restatement, sx, sy, sr, ss, px, py, core=po.GAUSS):
    u, v, _ = restatement.points_affect_points(core, 1, sx, sy, sr, ss, px, py, None, fp64=True)
    u, v = u / (2 * np.pi), v / (2 * np.pi)
    return float(np.sum(u * u + v * v)), u, v


@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_probe_vjp_matches_fp64_reference_adjoint(ctx, restatement, accum):
    sx, sy, sr, ss, px, py = probe_case()
    env = og.ExecEnv(og.CORE_GAUSSIAN, accum, ctx)
    src, probes = og.Points(sx, sy, sr, ss), og.Points(px, py)
    og.points_affect_points(src, probes, og.VELONLY, env, finalize=True)
    gx, gy, gs, gtx, gty = og.points_affect_points_vjp(src, probes, 2 * probes.u, 2 * probes.v, env,
                                                        want_targets=True)
    L, u, v = fp64_probe_loss(restatement, sx, sy, sr, ss, px, py)
    rx, ry, rs = restatement.probe_vjp(po.GAUSS, sx, sy, sr, ss, px, py, 2 * u, 2 * v)
    tol = 2e-5 if accum == og.COMPENSATED else 1e-4
    assert rel_err(rs, gs) < tol and rel_err(rx, gx) < tol and rel_err(ry, gy) < tol
    # target side: (1/2pi) (grad u)^T lam, against FP64 finite differences in the probe positions
    rng = np.random.default_rng(8)
    for p in rng.choice(px.size, 4, replace=False):
        for arr, g in ((px, gtx), (py, gty)):
            h = 1e-6
            a = arr.astype(np.float64).copy(); a[p] += h
            b = arr.astype(np.float64).copy(); b[p] -= h
            args_a = (a, py) if arr is px else (px, a)
            args_b = (b, py) if arr is px else (px, b)
            fd = (fp64_probe_loss(restatement, sx, sy, sr, ss, *args_a)[0]
                  - fp64_probe_loss(restatement, sx, sy, sr, ss, *args_b)[0]) / (2 * h)
            assert abs(fd - g[p]) < 1e-4 * max(1.0, abs(fd)), (p, fd, g[p])


def test_probe_vjp_against_fp64_finite_differences_64_coordinates(ctx, restatement):
    """Config-4 style check at reduced size: 64 seeded coordinates among all source positions
    and strengths, central differences of the FP64 forward loss."""
    sx, sy, sr, ss, px, py = probe_case(n=4000, grid=20, seed=5)
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    src, probes = og.Points(sx, sy, sr, ss), og.Points(px, py)
    og.points_affect_points(src, probes, og.VELONLY, env, finalize=True)
    gx, gy, gs = og.points_affect_points_vjp(src, probes, 2 * probes.u, 2 * probes.v, env)
    base = [a.astype(np.float64) for a in (sx, sy, ss)]
    rng = np.random.default_rng(64)
    picks = [(rng.integers(3), rng.integers(sx.size)) for _ in range(64)]
    for which, j in picks:
        arr = base[which]
        h = 1e-6 * max(1.0, abs(arr[j]))
        ap, am = arr.copy(), arr.copy()
        ap[j] += h
        am[j] -= h
        def L(a):
            v = list(base)
            v[which] = a
            return fp64_probe_loss(restatement, v[0], v[1], sr, v[2], px, py)[0]
        fd = (L(ap) - L(am)) / (2 * h)
        got = (gx, gy, gs)[which][j]
        scale = max(np.max(np.abs((gx, gy, gs)[which])), 1e-30)
        assert abs(fd - got) < 1e-4 * scale, (which, j, fd, got)


def test_autograd_wrapper_matches_c_abi(ctx):
    torch = pytest.importorskip("torch")
    from autograd_ops import ProbeVelocity
    sx, sy, sr, ss, px, py = probe_case(n=8000, grid=16, seed=6)
    dev = torch.device("cuda:0")
    T = lambda a, g=False: torch.tensor(a, device=dev, requires_grad=g)
    tsx, tsy, tss = T(sx, True), T(sy, True), T(ss, True)
    u, v = ProbeVelocity.apply(tsx, tsy, T(sr), tss, T(px), T(py), ctx, og.CORE_GAUSSIAN, og.COMPENSATED)
    loss = (u * u + v * v).sum()
    loss.backward()
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    ctx.set_stream(None)
    src, probes = og.Points(sx, sy, sr, ss), og.Points(px, py)
    og.points_affect_points(src, probes, og.VELONLY, env, finalize=True)
    gx, gy, gs = og.points_affect_points_vjp(src, probes, 2 * probes.u, 2 * probes.v, env)
    assert rel_err(gs, tss.grad.cpu().numpy()) < 1e-6
    assert rel_err(gx, tsx.grad.cpu().numpy()) < 1e-6 and rel_err(gy, tsy.grad.cpu().numpy()) < 1e-6


@pytest.mark.parametrize("core", [og.CORE_GAUSSIAN, og.CORE_RM, og.CORE_V2])
def test_self_vjp_matches_fp64_reference_adjoint(ctx, restatement, core):
    rng = np.random.default_rng(core)
    n = 3000
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = rng.uniform(0.01, 0.03, n).astype(np.float32)
    s = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    lu, lv = rng.normal(size=(2, n)).astype(np.float32)
    gx, gy, gs = og.points_affect_points_vjp_self(og.Points(x, y, r, s), lu, lv, og.ExecEnv(core, og.COMPENSATED, ctx))
    rx, ry, rs = restatement.self_vjp(core, x, y, r, s, lu, lv)
    assert rel_err(rx, gx) < 2e-5 and rel_err(ry, gy) < 2e-5 and rel_err(rs, gs) < 2e-5


def test_advect_matches_reference_trajectories(ctx, golden):
    g = golden("advect")
    p = og.Points(g["x"], g["y"], g["r"], g["s"])
    og.advect(p, fs=(1.0, 0.0), dt=0.01, nsteps=10, order=1, env=og.ExecEnv(og.CORE_RM, og.COMPENSATED, ctx))
    assert np.max(np.abs(p.x - g["euler_x"])) < 2e-6 and np.max(np.abs(p.y - g["euler_y"])) < 2e-6
    p = og.Points(g["x"], g["y"], g["r"], g["s"])
    og.advect(p, fs=(0.0, 0.0), dt=0.01, nsteps=4, order=2, env=og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    assert np.max(np.abs(p.x - g["rk2_x"])) < 2e-6 and np.max(np.abs(p.y - g["rk2_y"])) < 2e-6


def two_patches(n, seed=12):
    rng = np.random.default_rng(seed)
    lab = (np.arange(n) >= n // 2).astype(np.int32)
    x = np.where(lab == 0, -0.3, 0.3) + rng.normal(0, 0.1, n)
    y = rng.normal(0, 0.1, n)
    w = np.exp(-((x - np.where(lab == 0, -0.3, 0.3)) ** 2 + y ** 2) / (2 * 0.1 ** 2))
    s = np.where(lab == 0, w / w[lab == 0].sum(), w / w[lab == 1].sum())
    return x.astype(np.float32), y.astype(np.float32), s.astype(np.float32), lab


@pytest.mark.parametrize("order", [2, 1])
def test_advect_vjp_centroid_gradient_matches_fp64_reference(ctx, restatement, order):
    n, K, dt = 400, 12, 0.01
    x, y, s, lab = two_patches(n)
    r = np.full(n, 0.05, np.float32)
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    p = og.Points(x, y, r, s)
    og.advect(p, dt=dt, nsteps=K, order=order, env=env)
    gxT, gyT, gs_direct = np.zeros(n), np.zeros(n), np.zeros(n)
    xT, yT, s64 = p.x.astype(np.float64), p.y.astype(np.float64), s.astype(np.float64)
    lab32 = lab.astype(np.int32)
    L = restatement.lib.o_centroid_loss_d(n, po._p(xT), po._p(yT), po._p(s64), po._p(lab32),
                                          po._p(gxT), po._p(gyT), po._p(gs_direct))
    results = []
    for every in (0, 1, 5, K, og.TAPE_ALL):
        gs, gx0, gy0, peak = og.advect_vjp(og.Points(x, y, r, s), gxT, gyT, dt=dt, nsteps=K, order=order,
                                           checkpoint_every=every, env=env)
        results.append((gs, gx0, gy0))
        assert peak > 0
    for other in results[1:]:
        for a, b in zip(results[0], other):
            np.testing.assert_array_equal(a, b)
    if order == 2:
        Lr, gs_ref, gx_ref, gy_ref = restatement.rk2_centroid_grad(po.GAUSS, x, y, r, s, lab, (0.0, 0.0), dt, K)
        assert abs(Lr - L) < 1e-5 * abs(Lr)
        gs_tot = results[0][0] + gs_direct
        assert rel_err(gs_ref, gs_tot) < 1e-4
        assert rel_err(gx_ref, results[0][1]) < 1e-4 and rel_err(gy_ref, results[0][2]) < 1e-4
