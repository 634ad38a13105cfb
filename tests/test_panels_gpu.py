"""GPU parity tests of the panel path and the BEM solve through the C ABI.

The reference's float panel kernel differences two atan2 values and logs a ratio near 1, so
its own float results carry ~1e-5..1e-4 relative error at distant targets; the engine removes
those cancellations.  Each kernel is therefore checked tightly against the FP64 restatement and
loosely against the reference's float golden vectors."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err

pytestmark = pytest.mark.gpu

TOL64 = 5e-6     # engine (FP32 pairs, better-conditioned forms) vs FP64 restatement
TOLREF = 2e-4    # engine vs the reference's float results


def golden_surfaces(g):
    return og.Surfaces(g["nx"], g["ny"], g["idx"], vs=g["vs"], ss=g["ss"])


@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("vortex_only", [False, True])
def test_panels_affect_points(ctx, golden, restatement, accum, vortex_only):
    g = golden("panels")
    src = golden_surfaces(g)
    targ = og.Points(g["tx"], g["ty"])
    og.panels_affect_points(src, targ, og.ExecEnv(accum=accum, context=ctx), vortex_only=vortex_only)
    key = "p2pt_1v" if vortex_only else "p2pt_1vs"
    u64, v64 = restatement.panels_affect_points(g["nx"], g["ny"], g["idx"], g["vs"], None if vortex_only else g["ss"],
                                                g["tx"], g["ty"], fp64=True)
    assert rel_err(u64, targ.u) < TOL64 and rel_err(v64, targ.v) < TOL64
    assert rel_err(g[key + "_u"], targ.u) < TOLREF and rel_err(g[key + "_v"], targ.v) < TOLREF


@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_points_affect_panels(ctx, golden, restatement, accum):
    g = golden("panels")
    targ = og.Surfaces(g["nx"], g["ny"], g["idx"])
    src = og.Points(g["tx"], g["ty"], g["tr"], g["tg"])
    og.points_affect_panels(src, targ, og.ExecEnv(accum=accum, context=ctx))
    u64, v64 = restatement.points_affect_panels(g["tx"], g["ty"], g["tg"], g["nx"], g["ny"], g["idx"], fp64=True)
    assert rel_err(u64, targ.pu) < TOL64 and rel_err(v64, targ.pv) < TOL64
    assert rel_err(g["pt2p_u"], targ.pu) < TOLREF and rel_err(g["pt2p_v"], targ.pv) < TOLREF


@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_panel_sums_near_and_far_targets(ctx, restatement, accum):
    """Targets from a hundredth of a panel length off the body to a thousand radii away mix
    the series form of the log (|s| <= 0.2) and the near forms inside one warp."""
    rng = np.random.default_rng(41)
    c = og.circle_panels(256)
    surf = og.Surfaces(c.nx, c.ny, c.idx, vs=rng.normal(0, 1, 256).astype(np.float32),
                       ss=rng.normal(0, 1, 256).astype(np.float32))
    h = np.pi / 256
    n = 4096
    rad = 0.5 + np.concatenate([rng.choice([-1, 1], n // 2) * h * 10.0 ** rng.uniform(-2, 1, n // 2),
                                10.0 ** rng.uniform(-1, 3, n // 2)])
    th = rng.uniform(0, 2 * np.pi, n)
    x, y = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    targ = og.Points(x, y)
    og.panels_affect_points(surf, targ, og.ExecEnv(accum=accum, context=ctx))
    u64, v64 = restatement.panels_affect_points(surf.nx, surf.ny, surf.idx, surf.vs, surf.ss, x, y, fp64=True)
    # per target: relative to the largest term of that target's sum
    scale = np.abs(surf.vs).max() + np.abs(surf.ss).max()
    assert np.max(np.abs(targ.u - u64)) < 2e-5 * scale * np.pi
    # far targets: sums of 256 random-sign terms cancel to a small result, so plain FP32
    # accumulation shows its rounding; the compensated sums hold the FP64 restatement's value
    far = rad > 2.0
    tol = TOL64 if accum == og.COMPENSATED else 5e-5
    assert rel_err(u64[far], targ.u[far]) < tol and rel_err(v64[far], targ.v[far]) < tol
    # points -> panels with the same cloud as particles
    s = rng.normal(0, 1e-2, n).astype(np.float32)
    surf2 = og.circle_panels(256)
    og.points_affect_panels(og.Points(x, y, np.full(n, 0.01, np.float32), s), surf2,
                            og.ExecEnv(accum=accum, context=ctx))
    pu64, pv64 = restatement.points_affect_panels(x, y, s, surf2.nx, surf2.ny, surf2.idx, fp64=True)
    assert rel_err(pu64, surf2.pu) < 2e-5 and rel_err(pv64, surf2.pv) < 2e-5


def test_points_affect_panels_many_sources_split(ctx, restatement):
    """200k particles on 256 panels: exercises the source splits and the FP64 split reduction."""
    rng = np.random.default_rng(31)
    surf = og.circle_panels(256)
    n = 200_000
    r = np.sqrt(rng.uniform(0.55 ** 2, 9.0, n))
    a = rng.uniform(0, 2 * np.pi, n)
    x, y = (r * np.cos(a)).astype(np.float32), (r * np.sin(a)).astype(np.float32)
    s = rng.normal(0, 1e-2, n).astype(np.float32)
    og.points_affect_panels(og.Points(x, y, np.full(n, 0.01, np.float32), s), surf,
                            og.ExecEnv(accum=og.COMPENSATED, context=ctx))
    u64, v64 = restatement.points_affect_panels(x, y, s, surf.nx, surf.ny, surf.idx, fp64=True)
    # 200k random-sign strengths: the sums cancel to ~1/sqrt(n) of the term scale, so FP32 pair
    # rounding shows up ~sqrt(n) larger relative to the result than in the coherent cases
    assert rel_err(u64, surf.pu) < 2e-5 and rel_err(v64, surf.pv) < 2e-5


def test_panel_matrix_self_block(ctx, golden, restatement):
    g = golden("panels")
    s = og.Surfaces(g["nx"], g["ny"], g["idx"])
    A = og.panels_on_panels_coeff(s, nunk=2, context=ctx)
    assert A.shape == (128, 128)
    A64 = restatement.panels_on_panels_coeff(2, g["nx"], g["ny"], g["idx"], fp64=True)
    assert rel_err(A64, A) < TOL64
    assert rel_err(g["coeff"], A) < TOLREF
    np.testing.assert_allclose(np.diag(A), 0.5, rtol=1e-7)
    Ad = og.panels_on_panels_coeff(s, nunk=2, fp64=True, context=ctx)
    np.testing.assert_array_equal(Ad, A.astype(np.float64))


def test_panel_matrix_vortex_only_and_pair_block(ctx, restatement):
    a = og.circle_panels(48, 1.0)
    b = og.circle_panels(40, 0.6, center=(2.0, 0.3))
    A1 = og.panels_on_panels_coeff(a, nunk=1, context=ctx)
    R1 = restatement.panels_on_panels_coeff(1, a.nx, a.ny, a.idx, fp64=True)
    assert rel_err(R1, A1) < TOL64
    Ab = og.panels_on_panels_coeff(a, b, nunk=2, context=ctx)
    Rb = restatement.panels_on_panels_coeff(2, a.nx, a.ny, a.idx, fp64=True, self_block=False,
                                            tnx=b.nx, tny=b.ny, tidx=b.idx)
    assert Ab.shape == (80, 96)
    assert rel_err(Rb, Ab) < TOL64


def test_vels_to_rhs(ctx, golden):
    g = golden("panels")
    s = og.Surfaces(g["nx"], g["ny"], g["idx"], bcn=g["bcn"], pu=g["pu"].copy(), pv=g["pv"].copy())
    rhs = og.vels_to_rhs_panels(s, nunk=2, context=ctx)
    assert rel_err(g["rhs"], rhs) < 1e-6


@pytest.mark.parametrize("n", [1, 2, 7, 64, 333, 1024])
def test_dense_solve_fp64(ctx, n):
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + n * np.eye(n) * 0.1
    b = rng.normal(size=n)
    x, rel = og.solve_dense_f64(A, b, context=ctx)
    xr = np.linalg.solve(A, b)
    assert np.max(np.abs(x - xr)) < 1e-10 * max(1.0, np.max(np.abs(xr)))
    assert rel < 1e-13


def test_dense_solve_needs_pivoting(ctx):
    A = np.array([[0.0, 2.0, 1.0], [1.0, 1.0, 0.0], [3.0, 0.0, 1.0]])
    b = np.array([1.0, 2.0, 3.0])
    x, rel = og.solve_dense_f64(A, b, context=ctx)
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-13)


def test_dense_solve_reports_singular(ctx):
    A = np.zeros((4, 4))
    with pytest.raises(og.EngineError) as ei:
        og.solve_dense_f64(A, np.ones(4), context=ctx)
    assert ei.value.status == -6


def _restated_bem(restatement, surf, x, y, s, fs, nunk):
    pu, pv = restatement.points_affect_panels(x, y, s, surf.nx, surf.ny, surf.idx, fp64=True)
    pu, pv = fs[0] + pu / (2 * np.pi), fs[1] + pv / (2 * np.pi)
    rhs = restatement.vels_to_rhs_panels(nunk, surf.nx, surf.ny, surf.idx, pu, pv, None, fp64=True)
    A = restatement.panels_on_panels_coeff(nunk, surf.nx, surf.ny, surf.idx, fp64=True)
    return np.linalg.solve(A, rhs)


@pytest.mark.parametrize("direct_lu", [False, True])
@pytest.mark.parametrize("nunk", [2, 1])
def test_solve_bem_matches_fp64_restatement(ctx, restatement, nunk, direct_lu):
    rng = np.random.default_rng(41)
    surf = og.circle_panels(512)
    n = 20_000
    r = np.sqrt(rng.uniform(0.55 ** 2, 9.0, n))
    a = rng.uniform(0, 2 * np.pi, n)
    x, y = (r * np.cos(a)).astype(np.float32), (r * np.sin(a)).astype(np.float32)
    s = rng.normal(0, 1e-2, n).astype(np.float32)
    vort = og.Points(x, y, np.full(n, 0.01, np.float32), s)
    rel = og.solve_bem(vort, surf, fs=(1.0, 0.0), nunk=nunk, env=og.ExecEnv(accum=og.COMPENSATED, context=ctx),
                       direct_lu=direct_lu)
    assert rel < 1e-12
    xr = _restated_bem(restatement, surf, x, y, s, (1.0, 0.0), nunk)
    got = np.stack([surf.vs, surf.ss], 1).ravel() if nunk == 2 else surf.vs
    # the matrix is assembled in FP32 like the reference; with cond(A) ~ 1.5e3 at 512 panels
    # that alone moves the FP64 solution by up to ~cond * 1e-7
    assert rel_err(xr, got) < 3e-4
    # reuse the factorisation: same answer
    vs0 = surf.vs.copy()
    og.solve_bem(vort, surf, fs=(1.0, 0.0), nunk=nunk, env=og.ExecEnv(accum=og.COMPENSATED, context=ctx),
                 reuse_matrix=True, direct_lu=direct_lu)
    np.testing.assert_allclose(surf.vs, vs0, rtol=0, atol=1e-6 * np.max(np.abs(vs0)))


def test_solve_bem_cylinder_in_uniform_flow(ctx):
    """Potential flow past a unit-diameter cylinder: surface speed 2 U |sin(theta)|; the solved
    vortex sheet strength carries it, the source strength vanishes (no-through-flow BC)."""
    npan = 2048
    surf = og.circle_panels(npan)
    og.solve_bem(og.Points(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0)), surf, fs=(1.0, 0.0), nunk=2,
                 env=og.ExecEnv(context=ctx))
    th = -2 * np.pi * (np.arange(npan) + 0.5) / npan
    assert np.max(np.abs(np.abs(surf.vs) - 2.0 * np.abs(np.sin(th)))) < 5e-3
    assert np.max(np.abs(surf.ss)) < 5e-3


def test_gmres_and_lu_agree_on_the_bem_system(ctx):
    rng = np.random.default_rng(77)
    surf = og.circle_panels(1024)
    n = 30_000
    r = np.sqrt(rng.uniform(0.55 ** 2, 9.0, n))
    a = rng.uniform(0, 2 * np.pi, n)
    vort = og.Points((r * np.cos(a)).astype(np.float32), (r * np.sin(a)).astype(np.float32),
                     np.full(n, 0.01, np.float32), rng.normal(0, 1e-2, n).astype(np.float32))
    env = og.ExecEnv(accum=og.COMPENSATED, context=ctx)
    og.solve_bem(vort, surf, fs=(0.3, -0.2), env=env)
    g = np.concatenate([surf.vs, surf.ss])
    og.solve_bem(vort, surf, fs=(0.3, -0.2), env=env, direct_lu=True)
    d = np.concatenate([surf.vs, surf.ss])
    assert rel_err(d, g) < 1e-6       # both FP64 solves of one FP64 matrix; outputs are FP32


def test_gmres_dense_and_no_convergence(ctx):
    rng = np.random.default_rng(78)
    n = 700
    A = np.eye(n) * 4.0 + rng.normal(0, 1.0 / np.sqrt(n), (n, n))
    xt = rng.normal(size=n)
    b = A @ xt
    x, it, rel = og.solve_gmres_f64(A, b, tol=1e-13, restart=50, context=ctx)
    assert rel < 1e-13 and it < 100
    assert np.max(np.abs(x - xt)) < 1e-10 * np.max(np.abs(xt))
    # restart from the solution: converged on entry
    x2, it2, rel2 = og.solve_gmres_f64(A, b, x0=x, tol=1e-12, context=ctx)
    assert it2 == 0 and rel2 < 1e-12
    with pytest.raises(og.EngineError) as ei:
        og.solve_gmres_f64(A, b, tol=1e-15, restart=3, maxiter=4, context=ctx)
    assert ei.value.status == -9


@pytest.mark.parametrize("n", [1, 5, 33, 1000, 4100])
def test_gmres_fused_cycle_matches_per_step_kernels(n):
    """One cooperative launch per restart cycle (restart <= 64; products with the FP32 plane of
    A, each restart refining against the FP64 matrix) against one FP64 kernel per step: both
    solutions are exact to the tolerance, and refinement costs at most a few extra
    iterations; ragged orders leave part of the last 32-row group empty."""
    rng = np.random.default_rng(90 + n)
    A = np.eye(n) * 3.0 + rng.normal(0, 1.0 / np.sqrt(n), (n, n))
    xt = rng.normal(size=n)
    b = A @ xt
    out = {}
    for variant in (og.VARIANT_AUTO, og.VARIANT_GENERIC):
        c = og.Context()
        c.set_kernel_variant(variant)
        out[variant] = og.solve_gmres_f64(A, b, tol=1e-12, restart=40, maxiter=400, context=c)
    (xf, itf, relf), (xg, itg, relg) = out[og.VARIANT_AUTO], out[og.VARIANT_GENERIC]
    assert relf < 1e-12 and relg < 1e-12
    assert itf <= itg + 12
    assert np.max(np.abs(xf - xt)) < 1e-9 * np.max(np.abs(xt))
    assert np.max(np.abs(xf - xg)) < 1e-9 * np.max(np.abs(xt))


@pytest.mark.parametrize("scale", [1e-35, 1e-20, 1.0, 1e20, 1e35])
def test_gmres_matrix_scales(scale):
    """Entries beyond 2^+-99 cannot be carried by the FP32 planes of the fused cycle: such a
    matrix takes the FP64 per-step kernels; every scale converges to the same solution."""
    rng = np.random.default_rng(7)
    n = 300
    A = (np.eye(n) * 3.0 + rng.normal(0, 1.0 / np.sqrt(n), (n, n))) * scale
    xt = rng.normal(size=n)
    b = A @ xt
    x, it, rel = og.solve_gmres_f64(A, b, tol=1e-12, restart=40, maxiter=400, context=og.Context())
    assert rel < 1e-12
    assert np.max(np.abs(x - xt)) < 1e-9 * np.max(np.abs(xt))


@pytest.mark.parametrize("shape", ["circle", "poly"])
def test_augmented_block_matches_reference(ctx, golden, shape):
    g = golden("augment")
    body = og.Surfaces(g[shape + "_nx"], g[shape + "_ny"], g[shape + "_idx"])
    A, (vol, cx, cy) = og.panels_on_panels_coeff_augmented(body, context=ctx)
    R = g[shape + "_A"].astype(np.float64)
    assert abs(vol - g[shape + "_vol"][0]) < 1e-6 * abs(vol)
    np.testing.assert_allclose(A[-1, :], R[-1, :], rtol=0, atol=1e-6 * np.max(np.abs(R[-1, :])))   # lengths, 2 area
    # the rotation column comes through panels_affect_panels (collocation points 1e-4 off the panels)
    assert rel_err(R[:-1, -1], A[:-1, -1]) < 2e-6
    # the reference forms the block in FP32 (src/Coefficients.h:155-427)
    assert rel_err(R[:-1, :-1], A[:-1, :-1]) < 3e-6


def test_augmented_solve_circulation_and_rotation(ctx):
    """A cylinder in uniform flow: with zero net circulation the solved rotation rate is ~0 and
    the strengths match the plain solve; a prescribed circulation C gives sum(vs * len) = C."""
    surf = og.circle_panels(512)
    empty = og.Points(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    env = og.ExecEnv(accum=og.COMPENSATED, context=ctx)
    og.solve_bem(empty, surf, fs=(1.0, 0.0), env=env)
    vs0 = surf.vs.copy()
    om, rel = og.solve_bem_augmented(empty, surf, circ_rhs=0.0, fs=(1.0, 0.0), env=env)
    assert rel < 1e-12 and abs(om) < 1e-4
    assert rel_err(vs0, surf.vs) < 1e-4
    L = np.hypot(np.diff(np.append(surf.nx, surf.nx[0])), np.diff(np.append(surf.ny, surf.ny[0])))
    om, rel = og.solve_bem_augmented(empty, surf, circ_rhs=0.7, fs=(1.0, 0.0), env=env)
    A, (vol, _, _) = og.panels_on_panels_coeff_augmented(surf, context=ctx)
    assert rel < 1e-12
    # the bottom row of the system: sum(vs * len) + 2 area * omega = C
    assert abs(np.sum(surf.vs.astype(np.float64) * L) + 2 * vol * om - 0.7) < 1e-4


@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_panel_strength_vjp_vs_fp64(ctx, restatement, accum):
    """Reverse mode of panels_affect_points w.r.t. the vortex and source strengths against the
    FP64 restatement's unit-strength responses (the forward is linear in the strengths, so those
    are the exact gradients), with points far from and close to the body."""
    rng = np.random.default_rng(12)
    npan = 64
    c = og.circle_panels(npan)
    n = 1500
    rad = np.concatenate([np.sqrt(rng.uniform(0.55 ** 2, 9.0, n - 100)), 0.5 + rng.choice([-1, 1], 100) * 0.02])
    th = rng.uniform(0, 2 * np.pi, n)
    x, y = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    lu, lv = rng.normal(size=(2, n)).astype(np.float32)
    gv, gs = og.panels_affect_points_vjp(og.Surfaces(c.nx, c.ny, c.idx), og.Points(x, y), lu, lv,
                                         og.ExecEnv(accum=accum, context=ctx))
    gv_ref, gs_ref = np.zeros(npan), np.zeros(npan)
    zero = np.zeros(npan, np.float32)
    for p in range(npan):
        e = zero.copy()
        e[p] = 1.0
        u, v = restatement.panels_affect_points(c.nx, c.ny, c.idx, e, zero, x, y, fp64=True)
        gv_ref[p] = (lu @ u + lv @ v) / (2 * np.pi)
        u, v = restatement.panels_affect_points(c.nx, c.ny, c.idx, zero, e, x, y, fp64=True)
        gs_ref[p] = (lu @ u + lv @ v) / (2 * np.pi)
    tol = 5e-6 if accum == og.COMPENSATED else 5e-5
    assert rel_err(gv_ref, gv) < tol and rel_err(gs_ref, gs) < tol


def test_panel_strength_vjp_homogeneity(ctx):
    """Large case, size-independent check: the forward is linear in the strengths, so
    sum_p (dL/dg_p g_p + dL/ds_p s_p) equals L = sum_t lambda_t . u_t / (2 pi)."""
    rng = np.random.default_rng(13)
    npan, n = 2048, 200_000
    c = og.circle_panels(npan)
    surf = og.Surfaces(c.nx, c.ny, c.idx, vs=rng.normal(0, 1, npan).astype(np.float32),
                       ss=rng.normal(0, 1, npan).astype(np.float32))
    rad = np.sqrt(rng.uniform(0.55 ** 2, 9.0, n))
    th = rng.uniform(0, 2 * np.pi, n)
    x, y = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    lu, lv = rng.normal(size=(2, n)).astype(np.float32)
    env = og.ExecEnv(accum=og.COMPENSATED, context=ctx)
    targ = og.Points(x, y)
    og.panels_affect_points(surf, targ, env, finalize=True)
    L = float(lu.astype(np.float64) @ targ.u + lv.astype(np.float64) @ targ.v)
    gv, gs = og.panels_affect_points_vjp(surf, og.Points(x, y), lu, lv, env)
    lin = float(gv.astype(np.float64) @ surf.vs + gs.astype(np.float64) @ surf.ss)
    scale = float(np.abs(lu).astype(np.float64) @ np.abs(targ.u) + np.abs(lv).astype(np.float64) @ np.abs(targ.v))
    assert abs(lin - L) < 1e-5 * scale


def test_panel_autograd_wrapper_matches_c_abi(ctx):
    """torch autograd through the panel forward/backward pair gives the C-ABI VJP for the
    loss sum(u^2 + v^2)."""
    torch = pytest.importorskip("torch")
    from autograd_ops import PanelVelocity
    rng = np.random.default_rng(14)
    npan, n = 256, 20_000
    c = og.circle_panels(npan)
    vs = rng.normal(0, 1, npan).astype(np.float32)
    ss = rng.normal(0, 1, npan).astype(np.float32)
    rad = np.sqrt(rng.uniform(0.55 ** 2, 4.0, n))
    th = rng.uniform(0, 2 * np.pi, n)
    x, y = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    dev = torch.device("cuda:0")
    T = lambda a, g=False: torch.tensor(a, device=dev, requires_grad=g)
    tvs, tss = T(vs, True), T(ss, True)
    idx = torch.from_numpy(c.idx.astype(np.int32)).to(dev)
    u, v = PanelVelocity.apply(tvs, tss, T(c.nx), T(c.ny), idx, T(x), T(y), ctx, og.COMPENSATED)
    (u * u + v * v).sum().backward()
    ctx.set_stream(None)
    env = og.ExecEnv(accum=og.COMPENSATED, context=ctx)
    surf = og.Surfaces(c.nx, c.ny, c.idx, vs=vs, ss=ss)
    targ = og.Points(x, y)
    og.panels_affect_points(surf, targ, env, finalize=True)
    assert rel_err(targ.u, u.detach().cpu().numpy()) < 1e-6
    gv, gs = og.panels_affect_points_vjp(surf, og.Points(x, y), 2 * targ.u, 2 * targ.v, env)
    assert rel_err(gv, tvs.grad.cpu().numpy()) < 1e-6 and rel_err(gs, tss.grad.cpu().numpy()) < 1e-6


def test_two_bodies_matrix_matches_reference_block_assembly(ctx, golden, restatement):
    """The joined panel set of two bodies against the reference's block-by-block assembly
    (tests/golden/bodies.npz; src/BEMHelper.h:166-221)."""
    g = golden("bodies")
    j, _ = og.join_surfaces([og.Surfaces(g["nx0"], g["ny0"], g["idx0"]), og.Surfaces(g["nx1"], g["ny1"], g["idx1"])])
    A = og.panels_on_panels_coeff(j, nunk=2, context=ctx)
    assert A.shape == (120, 120)
    assert rel_err(g["A"], A) < TOLREF
    A64 = restatement.panels_on_panels_coeff(2, j.nx, j.ny, j.idx, fp64=True)
    # the FP32 assembly is 1.2e-5 off FP64 on this pair of bodies (uneven polygon panels near
    # the circle), as the reference's own float build is (1.2e-5)
    assert rel_err(A64, A) < 2e-5


def test_solve_bem_two_bodies_matches_fp64_restatement(ctx, restatement):
    rng = np.random.default_rng(5)
    n = 20_000
    r = np.sqrt(rng.uniform(0.55 ** 2, 9.0, n))
    t = rng.uniform(0, 2 * np.pi, n)
    x, y = r * np.cos(t), r * np.sin(t)
    keep = np.hypot(x - 1.5, y - 0.3) > 0.36                 # outside the second body too
    x, y = x[keep].astype(np.float32), y[keep].astype(np.float32)
    s = rng.normal(0, 1e-2, x.size).astype(np.float32)
    a, b = og.circle_panels(256), og.circle_panels(128, 0.6, center=(1.5, 0.3))
    vort = og.Points(x, y, np.full(x.size, 0.01, np.float32), s)
    rel = og.solve_bem_bodies(vort, [a, b], fs=(1.0, 0.0), nunk=2,
                              env=og.ExecEnv(accum=og.COMPENSATED, context=ctx))
    assert rel < 1e-12
    j, offs = og.join_surfaces([og.circle_panels(256), og.circle_panels(128, 0.6, center=(1.5, 0.3))])
    assert list(offs) == [0, 256, 384]
    xr = _restated_bem(restatement, j, x, y, s, (1.0, 0.0), 2)
    got = np.stack([np.concatenate([a.vs, b.vs]), np.concatenate([a.ss, b.ss])], 1).ravel()
    # FP32 assembly as in the reference; cond(A) ~ 850 here moves the FP64 solution by ~2e-5
    assert rel_err(xr, got) < 3e-4


def _clear_check_method0(g_x, g_y, g_s, x, y, s, r):
    """A fully cropped particle lands exactly on the layer and the rounding of that shift
    decides whether it is cut again, possibly along another closest panel or node normal: such
    particles carry no circulation and their positions are compared within half a core radius;
    everything else tightly."""
    cropped = g_s == 0.0
    d = np.hypot(g_x - x, g_y - y)
    assert np.all(d[~cropped] < 1e-5), np.max(d[~cropped])
    assert np.all(d[cropped] <= 0.5 * r[cropped])
    assert np.all(s[cropped] == 0.0)
    np.testing.assert_allclose(s, g_s, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("shape", ["circle", "star"])
def test_clear_inner_layer_matches_reference(ctx, golden, restatement, shape):
    """clear_inner_layer (src/Reflect.h:491-760) against the reference's own routine
    (tests/golden/clear.npz): crop, push, and push of field points."""
    g = golden("clear")
    cut, ips = float(g["cut"][0]), float(g["ips"][0])
    body = og.Surfaces(g[shape + "_nx"], g[shape + "_ny"], g[shape + "_idx"])
    env = og.ExecEnv(context=ctx)
    x, y, s, r = g[shape + "_x"], g[shape + "_y"], g[shape + "_s"], g[shape + "_r"]
    p = og.Points(x, y, r, s)
    lost, nc = og.clear_inner_layer(p, body, ips, method=0, cutoff_mult=cut, env=env)
    _clear_check_method0(g[shape + "_m0_x"], g[shape + "_m0_y"], g[shape + "_m0_s"], p.x, p.y, p.s, r)
    # the oracle is built without fused multiply-adds, like the kernel: equal bit for bit
    ox, oy, os_, _, onc = restatement.clear_inner(0, cut, ips, body.nx, body.ny, body.idx, x, y, s, r)
    np.testing.assert_array_equal(p.x, ox)
    np.testing.assert_array_equal(p.y, oy)
    np.testing.assert_array_equal(p.s, os_)
    assert nc == onc
    glost = float(g[shape + "_m0_lost"][0])
    assert abs(lost - glost) < 1e-5 * max(1.0, abs(glost)) and nc > 0
    p = og.Points(x, y, r, s)
    lost, nc = og.clear_inner_layer(p, body, ips, method=1, cutoff_mult=cut, env=env)
    assert lost == 0.0 and nc > 0
    np.testing.assert_array_equal(p.s, s)
    assert np.max(np.hypot(p.x - g[shape + "_m1_x"], p.y - g[shape + "_m1_y"])) < 1e-5
    f = og.Points(x, y)
    og.clear_inner_layer(f, body, ips, method=1, cutoff_mult=0.0, env=env)
    assert np.max(np.hypot(f.x - g[shape + "_fld_x"], f.y - g[shape + "_fld_y"])) < 1e-5


def test_clear_inner_layer_large_vs_oracle(ctx, restatement):
    rng = np.random.default_rng(21)
    body = og.circle_panels(2048)
    n = 20_000
    rad = rng.uniform(0.3, 0.6, n)
    a = rng.uniform(0, 2 * np.pi, n)
    x, y = (rad * np.cos(a)).astype(np.float32), (rad * np.sin(a)).astype(np.float32)
    s = rng.normal(0, 1, n).astype(np.float32)
    r = np.full(n, 0.004, np.float32)
    ips = 0.004
    p = og.Points(x, y, r, s)
    lost, nc = og.clear_inner_layer(p, body, ips, method=0, env=og.ExecEnv(context=ctx))
    ox, oy, os_, olost, onc = restatement.clear_inner(0, og.CLEAR_CUTOFF, ips, body.nx, body.ny, body.idx,
                                                      x, y, s, r)
    # the kernel and the oracle both round every product and sum as written: bit for bit
    np.testing.assert_array_equal(p.x, ox)
    np.testing.assert_array_equal(p.y, oy)
    np.testing.assert_array_equal(p.s, os_)
    assert nc == onc
    assert abs(lost - olost) < 1e-4 * max(1.0, abs(olost))
    # every particle ends at or above the layer's inner edge
    assert np.min(np.hypot(p.x, p.y)) > 0.5


def test_clear_inner_layer_shared_node_and_tiles_vs_oracle(ctx, restatement):
    """Two triangles joined at one node (four panels meet there: its normal is summed in panel
    order, as in the reference) and a 5000-panel circle (several shared-memory tiles of panel
    records per sweep): the kernel equals the oracle bit for bit."""
    rng = np.random.default_rng(31)
    nx = np.array([0.0, 0.4, 0.4, -0.4, -0.4], np.float32)
    ny = np.array([0.0, -0.2, 0.2, 0.2, -0.2], np.float32)
    idx = np.array([0, 1, 1, 2, 2, 0, 0, 3, 3, 4, 4, 0], np.uint32)       # clockwise bow tie
    bowtie = og.Surfaces(nx, ny, idx)
    big = og.circle_panels(5000)
    for body, n, lo, hi in ((bowtie, 3000, 0.0, 0.45), (big, 8000, 0.3, 0.6)):
        rad = rng.uniform(lo, hi, n)
        a = rng.uniform(0, 2 * np.pi, n)
        x, y = (rad * np.cos(a)).astype(np.float32), (rad * np.sin(a)).astype(np.float32)
        s = rng.normal(0, 1, n).astype(np.float32)
        r = np.full(n, 0.01, np.float32)
        for method in (0, 1):
            p = og.Points(x, y, r, s)
            lost, nc = og.clear_inner_layer(p, body, 0.01, method=method, env=og.ExecEnv(context=ctx))
            ox, oy, os_, olost, onc = restatement.clear_inner(method, og.CLEAR_CUTOFF, 0.01, body.nx, body.ny,
                                                              body.idx, x, y, s, r)
            np.testing.assert_array_equal(p.x, ox)
            np.testing.assert_array_equal(p.y, oy)
            np.testing.assert_array_equal(p.s, os_)
            assert nc == onc and nc > 0


def _two_rotating_bodies(golden):
    g = golden("bodies_aug")
    bodies = [og.Surfaces(g[f"nx{k}"], g[f"ny{k}"], g[f"idx{k}"]) for k in range(2)]
    n0, n1 = bodies[0].npan, bodies[1].npan
    npu = 2 * (n0 + n1)
    # reference order: body 0's panel unknowns, its rotation; body 1's, its rotation
    perm = np.concatenate([np.arange(2 * n0), [npu], np.arange(2 * n0, npu), [npu + 1]])
    return g, bodies, perm


def test_bodies_augmented_matrix_matches_reference(ctx, golden):
    """Two rotating bodies in one system against the reference's own block assembly
    (src/BEMHelper.h:166-221, each block from src/Coefficients.h:155-572; golden
    bodies_aug.npz), after permuting the engine's order (panels first, rotations last)."""
    g, bodies, perm = _two_rotating_bodies(golden)
    A, geom = og.panels_on_panels_coeff_bodies(bodies, [True, True], context=ctx)
    R = g["A"].astype(np.float64)
    B = A[np.ix_(perm, perm)]
    for k in range(2):
        assert abs(geom[k, 0] - g[f"vol{k}"][0]) < 1e-6 * abs(geom[k, 0])
    rot = [2 * bodies[0].npan, R.shape[0] - 1]
    pan = np.setdiff1d(np.arange(R.shape[0]), rot)
    # the reference forms every block in FP32; on this pair of bodies its float assembly is
    # 1.2e-5 off FP64 (test_two_bodies_matrix_matches_reference_block_assembly)
    assert rel_err(R[np.ix_(pan, pan)], B[np.ix_(pan, pan)]) < 2e-5
    assert rel_err(R[np.ix_(pan, rot)], B[np.ix_(pan, rot)]) < 2e-5           # unit-rotation columns
    np.testing.assert_allclose(B[rot, :], R[rot, :], rtol=0, atol=1e-6 * np.max(np.abs(R[rot, :])))


@pytest.mark.parametrize("augmented", [(True, True), (True, False)])
def test_bodies_augmented_solve(ctx, golden, restatement, augmented):
    """The solve of two bodies, one or both rotating, against an FP64 solve of the reference's
    matrix (golden; a non-rotating body drops its rotation row and column) with the right-hand
    side from the FP64 restatement and the prescribed circulations."""
    g, bodies, perm = _two_rotating_bodies(golden)
    rng = np.random.default_rng(41)
    n = 5000
    r = np.sqrt(rng.uniform(0.55 ** 2, 4.0, n))
    t = rng.uniform(0, 2 * np.pi, n)
    x, y = r * np.cos(t), r * np.sin(t)
    keep = np.hypot(x - 1.3, y - 0.4) > 0.45
    x, y = x[keep].astype(np.float32), y[keep].astype(np.float32)
    s = rng.normal(0, 1e-2, x.size).astype(np.float32)
    circ = [0.3, -0.2]
    rel = og.solve_bem_bodies(og.Points(x, y, np.full(x.size, 0.01, np.float32), s), bodies, fs=(1.0, 0.0),
                              nunk=2, env=og.ExecEnv(accum=og.COMPENSATED, context=ctx), augmented=list(augmented),
                              circ_rhs=circ)
    assert rel < 1e-12
    joined, offs = og.join_surfaces([og.Surfaces(b.nx, b.ny, b.idx) for b in bodies])
    pu, pv = restatement.points_affect_panels(x, y, s, joined.nx, joined.ny, joined.idx, fp64=True)
    pu, pv = 1.0 + pu / (2 * np.pi), pv / (2 * np.pi)
    rhs_p = restatement.vels_to_rhs_panels(2, joined.nx, joined.ny, joined.idx, pu, pv, fp64=True)
    npu = rhs_p.size
    rhs = np.concatenate([rhs_p, circ])[perm]
    R = g["A"].astype(np.float64)
    keep_rows = np.array([not (p >= npu and not augmented[p - npu]) for p in perm])
    xr = np.linalg.solve(R[np.ix_(keep_rows, keep_rows)], rhs[keep_rows])
    full = np.full(perm.size, np.nan)
    full[keep_rows] = xr
    unperm = np.empty_like(full)
    unperm[perm] = full
    got = np.stack([np.concatenate([b.vs for b in bodies]), np.concatenate([b.ss for b in bodies])], 1).ravel()
    assert rel_err(unperm[:npu], got) < 3e-4
    for k in range(2):
        if augmented[k]:
            assert abs(bodies[k].omega - unperm[npu + k]) < 3e-4 * max(1.0, abs(unperm[npu + k]))
        else:
            assert bodies[k].omega is None


def test_bodies_augmented_matrix_vortex_only(ctx, golden):
    """The vortex-only system (one unknown per panel, src/Coefficients.h:366-385) of the two
    rotating bodies: its panel block is the vortex-on-tangential part of the two-unknown
    matrix, its rotation rows the panel lengths under the vortex unknowns, its rotation
    columns the tangential components -- the even rows and columns of the reference's
    two-unknown assembly (golden bodies_aug.npz)."""
    g, bodies, _ = _two_rotating_bodies(golden)
    n0, n1 = bodies[0].npan, bodies[1].npan
    A1, _ = og.panels_on_panels_coeff_bodies(bodies, [True, True], nunk=1, context=ctx)
    # engine order: panels of body 0, of body 1, rotation 0, rotation 1 -> reference order
    ref_idx = np.concatenate([2 * np.arange(n0), 2 * n0 + 1 + 2 * np.arange(n1), [2 * n0, 2 * n0 + 1 + 2 * n1]])
    R = g["A"].astype(np.float64)[np.ix_(ref_idx, ref_idx)]
    pan = np.arange(n0 + n1)
    rot = np.array([n0 + n1, n0 + n1 + 1])
    assert rel_err(R[np.ix_(pan, pan)], A1[np.ix_(pan, pan)]) < 2e-5
    assert rel_err(R[np.ix_(pan, rot)], A1[np.ix_(pan, rot)]) < 2e-5
    np.testing.assert_allclose(A1[rot, :], R[rot, :], rtol=0, atol=1e-6 * np.max(np.abs(R[rot, :])))


def test_bodies_augmented_three_bodies_solve(ctx, restatement):
    """Three bodies, the first and last rotating: the rotation unknowns follow the body order
    of the rotating bodies only; the solve equals an FP64 solve of the engine's own augmented
    matrix with the restated FP64 right-hand side and the prescribed circulations, and the
    middle body gets no rotation rate."""
    bodies = [og.circle_panels(40, 0.8, center=(0.0, 0.0)), og.circle_panels(24, 0.5, center=(1.6, 0.3)),
              og.circle_panels(30, 0.6, center=(-0.4, 1.5))]
    aug = [True, False, True]
    A, geom = og.panels_on_panels_coeff_bodies(bodies, aug, nunk=2, context=ctx)
    npu = 2 * sum(b.npan for b in bodies)
    assert A.shape == (npu + 2, npu + 2)
    # rotation rows: each rotating body's panel lengths under its own vortex unknowns only
    offs = np.cumsum([0] + [b.npan for b in bodies])
    for r, k in ((npu, 0), (npu + 1, 2)):
        b = bodies[k]
        L = np.hypot(np.diff(np.append(b.nx, b.nx[0])), np.diff(np.append(b.ny, b.ny[0])))
        row = A[r, :npu]
        np.testing.assert_allclose(row[2 * offs[k]:2 * offs[k + 1]:2], L, rtol=1e-6)
        others = np.ones(npu, bool)
        others[2 * offs[k]:2 * offs[k + 1]:2] = False
        assert not row[others].any()
        assert abs(A[r, r] - 2 * geom[k, 0]) < 1e-9 * abs(A[r, r])
    rng = np.random.default_rng(43)
    n = 3000
    x, y = rng.uniform(-2.0, 3.0, (2, n))
    inside = np.zeros(n, bool)
    for b, c, d in zip(bodies, ((0.0, 0.0), (1.6, 0.3), (-0.4, 1.5)), (0.8, 0.5, 0.6)):
        inside |= np.hypot(x - c[0], y - c[1]) < 0.5 * d + 0.08
    x, y = x[~inside].astype(np.float32), y[~inside].astype(np.float32)
    s = rng.normal(0, 1e-2, x.size).astype(np.float32)
    circ = [0.25, 0.0, -0.4]
    rel = og.solve_bem_bodies(og.Points(x, y, np.full(x.size, 0.01, np.float32), s), bodies, fs=(1.0, 0.0),
                              nunk=2, env=og.ExecEnv(accum=og.COMPENSATED, context=ctx), augmented=aug, circ_rhs=circ)
    assert rel < 1e-12
    joined, _ = og.join_surfaces([og.Surfaces(b.nx, b.ny, b.idx) for b in bodies])
    pu, pv = restatement.points_affect_panels(x, y, s, joined.nx, joined.ny, joined.idx, fp64=True)
    pu, pv = 1.0 + pu / (2 * np.pi), pv / (2 * np.pi)
    rhs = np.concatenate([restatement.vels_to_rhs_panels(2, joined.nx, joined.ny, joined.idx, pu, pv, fp64=True),
                          [circ[0], circ[2]]])
    xr = np.linalg.solve(A, rhs)
    got = np.stack([np.concatenate([b.vs for b in bodies]), np.concatenate([b.ss for b in bodies])], 1).ravel()
    assert rel_err(xr[:npu], got) < 3e-4
    assert abs(bodies[0].omega - xr[npu]) < 3e-4 * max(1.0, abs(xr[npu]))
    assert abs(bodies[2].omega - xr[npu + 1]) < 3e-4 * max(1.0, abs(xr[npu + 1]))
    assert bodies[1].omega is None


@pytest.mark.parametrize("call", ["panels_on_points", "points_on_panels", "panel_vjp", "rhs"])
def test_device_panel_node_index_out_of_range_is_reported(call):
    """A node index past the node count in a device panel set (the host entry points check
    indices before any launch; device arrays can only be checked on the device): the kernels
    check every index before they read the nodes, take that panel as a far panel of zero
    strength and record the failure, which the next synchronizing call reports (OBS_ERR_ARG,
    record code 301); the context then computes a correct sum."""
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    ctx = og.Context()
    bd = og.circle_panels(256)
    good = torch.from_numpy(bd.idx.astype(np.int32)).to(dev)
    bad = good.clone()
    bad[2 * 17 + 1] = bd.nnodes + 5
    NX, NY = torch.from_numpy(bd.nx).to(dev), torch.from_numpy(bd.ny).to(dev)
    rng = np.random.default_rng(11)
    px, py = rng.uniform(-2.0, 2.0, (2, 5000)).astype(np.float32)
    ps = rng.normal(0.0, 1e-2, 5000).astype(np.float32)
    PX, PY, PS = [torch.from_numpy(a).to(dev) for a in (px, py, ps)]
    VS = torch.ones(bd.npan, device=dev)
    TU, TV = torch.zeros(5000, device=dev), torch.zeros(5000, device=dev)
    PU, PV = torch.zeros(bd.npan, device=dev), torch.zeros(bd.npan, device=dev)
    RHS = torch.zeros(2 * bd.npan, dtype=torch.float64, device=dev)

    def run(idx):
        if call == "panels_on_points":
            og.panels_affect_points_dev(ctx, og.COMPENSATED, NX, NY, idx, VS, None, PX, PY, TU, TV)
        elif call == "points_on_panels":
            og.points_affect_panels_dev(ctx, og.COMPENSATED, PX, PY, PS, NX, NY, idx, PU, PV, finalize=True)
        elif call == "panel_vjp":
            og.panels_affect_points_vjp_dev(ctx, og.COMPENSATED, NX, NY, idx, PX, PY, PS, PS, PU, PV)
        else:
            og.vels_to_rhs_panels_dev(ctx, 2, NX, NY, idx, PU, PV, None, None, RHS)

    run(bad)
    with pytest.raises(og.EngineError) as ei:
        ctx.synchronize()
    assert ei.value.status == -1
    bits, code, _, _ = ctx.last_failure()
    assert bits & 4 and code == 301
    # the same context afterwards: a valid call completes and reports nothing
    for t in (TU, TV, PU, PV, RHS):
        t.zero_()
    run(good)
    ctx.synchronize()
    ctx.close()
