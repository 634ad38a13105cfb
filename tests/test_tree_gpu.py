"""GPU tests of the treecode (obs_points_affect_points_tree, csrc/tree.cu): the reference's
Barnes-Hut summation slot (summation_t barneshut, src/ExecEnv.h:26-31), reached in the
reference only through the external solver hook (src/Influence.h:31-38, 74-98).  Checked
against the FP64 restatement of the direct sum (the oracle) for every core, thick targets and
field points, and against the engine's compensated direct sum at a size where the tree is deep.

Tolerance: normwise max relative error 2e-6 at the default acceptance (theta 0.5) and order
(24 terms), whose truncation bound per node is 0.5^24/0.5 = 1.2e-7 of that node's summed
|strength|/distance."""
import ctypes

import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

TOL = 2e-6
CORES = [og.CORE_GAUSSIAN, og.CORE_SINGULAR, og.CORE_COMPACT_EXP, og.CORE_RM, og.CORE_V2, og.CORE_WL, og.CORE_V3]


def patch(rng, n, sigma=0.25, core_r=0.005):
    x, y = rng.normal(0.0, sigma, (2, n)).astype(np.float32)
    g = np.exp(-(x.astype(np.float64) ** 2 + y.astype(np.float64) ** 2) / (2 * sigma ** 2))
    s = (g / g.sum()).astype(np.float32)
    return x, y, np.full(n, core_r, np.float32), s


@pytest.mark.parametrize("core", CORES)
@pytest.mark.parametrize("thick", [True, False])
def test_tree_matches_fp64_direct_sum(ctx, restatement, core, thick):
    rng = np.random.default_rng(100 + core)
    ns, nt = 12000, 3000
    sx, sy, sr, ss = patch(rng, ns)
    sr = (sr * rng.uniform(0.8, 1.25, ns)).astype(np.float32)     # varying radii
    tx, ty, tr, _ = patch(rng, nt)
    tx[:100], ty[:100], tr[:100] = sx[:100], sy[:100], sr[:100]    # coincident pairs
    src = og.Points(sx, sy, sr, ss)
    targ = og.Points(tx, ty, tr if thick else None, None)
    og.points_affect_points_tree(src, targ, og.ExecEnv(core, og.COMPENSATED, ctx))
    u, v, _ = restatement.points_affect_points(core, po.VELONLY, sx, sy, sr, ss, tx, ty, tr if thick else None,
                                               fp64=True)
    assert np.isfinite(targ.u).all() and np.isfinite(targ.v).all()
    assert rel_err(u, targ.u) < TOL and rel_err(v, targ.v) < TOL


@pytest.mark.parametrize("thick", [True, False])
def test_tree_gaussian_uniform_radii_fp64(ctx, restatement, thick):
    """Every source (and target) with one radius: the Gaussian's near leaf sums take the packed
    uniform form (cut-offs x > 16 and x < 0.001 on t = -x log2 e); coincident pairs exercise
    the small-x branch."""
    rng = np.random.default_rng(321 + thick)
    sx, sy, sr, ss = patch(rng, 12000)
    tx, ty, tr, _ = patch(rng, 3000)
    tx[:100], ty[:100] = sx[:100], sy[:100]
    src = og.Points(sx, sy, sr, ss)
    targ = og.Points(tx, ty, tr if thick else None, None)
    og.points_affect_points_tree(src, targ, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    u, v, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, po.VELONLY, sx, sy, sr, ss, tx, ty,
                                               tr if thick else None, fp64=True)
    assert np.isfinite(targ.u).all() and np.isfinite(targ.v).all()
    assert rel_err(u, targ.u) < TOL and rel_err(v, targ.v) < TOL


def test_tree_self_interaction_against_direct_engine(ctx):
    """200,000 particles of the Gaussian patch on themselves (a seven-level tree): the treecode
    against the engine's compensated direct sum (itself within 1e-7 of FP64)."""
    rng = np.random.default_rng(7)
    x, y, r, s = patch(rng, 200_000)
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    a = og.Points(x, y, r, s)
    og.points_affect_points(a, a, og.VELONLY, env)
    b = og.Points(x, y, r, s)
    og.points_affect_points_tree(b, b, env)
    assert rel_err(a.u, b.u) < TOL and rel_err(a.v, b.v) < TOL
    c = og.Points(x, y, r, s)
    og.points_affect_points_tree(c, c, env)
    np.testing.assert_array_equal(b.u, c.u)                        # deterministic
    np.testing.assert_array_equal(b.v, c.v)


@pytest.mark.parametrize("ns", [0, 1, 31, 33, 1000])
@pytest.mark.parametrize("nt", [0, 1, 33, 257])
def test_tree_edge_sizes(ctx, restatement, ns, nt):
    rng = np.random.default_rng(ns * 131 + nt)
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = np.full(ns, 0.05, np.float32)
    ss = rng.normal(0, 0.1, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tr = np.full(nt, 0.05, np.float32)
    targ = og.Points(tx, ty, tr, None, u=np.ones(nt, np.float32), v=-np.ones(nt, np.float32))
    og.points_affect_points_tree(og.Points(sx, sy, sr, ss), targ, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    u, v, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True,
                                               tu=np.ones(nt), tv=-np.ones(nt))
    if nt:
        assert rel_err(u, targ.u) < TOL and rel_err(v, targ.v) < TOL


def test_tree_accumulates_and_finalizes(ctx, restatement):
    rng = np.random.default_rng(12)
    sx, sy, sr, ss = patch(rng, 5000)
    tx, ty = rng.uniform(-0.5, 0.5, (2, 700)).astype(np.float32)
    u0, v0 = rng.normal(0, 1, (2, 700)).astype(np.float32)
    targ = og.Points(tx, ty, None, None, u=u0.copy(), v=v0.copy())
    og.points_affect_points_tree(og.Points(sx, sy, sr, ss), targ, og.ExecEnv(og.CORE_V2, og.COMPENSATED, ctx),
                                 finalize=True, fs=(1.0, -0.5))
    u, v, _ = restatement.points_affect_points(og.CORE_V2, 1, sx, sy, sr, ss, tx, ty, None, fp64=True,
                                               tu=u0.astype(np.float64), tv=v0.astype(np.float64))
    assert rel_err(1.0 + u / (2 * np.pi), targ.u) < TOL and rel_err(-0.5 + v / (2 * np.pi), targ.v) < TOL


def test_tree_error_falls_with_order(ctx, restatement):
    """The truncation error shrinks with the number of terms (theta 0.5): order 4, 8, 16."""
    rng = np.random.default_rng(13)
    sx, sy, sr, ss = patch(rng, 30_000, core_r=0.001)
    tx, ty, tr, _ = patch(rng, 2000, core_r=0.001)
    u, v, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True)
    errs = []
    for order in (4, 8, 16):
        targ = og.Points(tx, ty, tr, None)
        og.points_affect_points_tree(og.Points(sx, sy, sr, ss), targ, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx),
                                     order=order)
        errs.append(max(rel_err(u, targ.u), rel_err(v, targ.v)))
    assert errs[0] > errs[1] > errs[2] and errs[0] > 1e-5 and errs[2] < 1e-5


def test_tree_device_entry_point(ctx):
    torch = pytest.importorskip("torch")
    dev = torch.device("cuda:0")
    rng = np.random.default_rng(14)
    x, y, r, s = patch(rng, 20_000)
    X, Y, R, S = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    U, V = torch.zeros(20_000, device=dev), torch.zeros(20_000, device=dev)
    og.points_affect_points_tree_dev(ctx, og.CORE_GAUSSIAN, X, Y, R, S, X, Y, R, U, V)
    ctx.synchronize()
    p = og.Points(x, y, r, s)
    og.points_affect_points_tree(p, p, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    np.testing.assert_array_equal(U.cpu().numpy(), p.u)
    np.testing.assert_array_equal(V.cpu().numpy(), p.v)


def test_external_hook_through_the_tree(restatement):
    """external_vel_solver_tr_f_ (the reference's external-solver hook, which reaches onbody's
    treecode in the reference) routed through the treecode."""
    L = og.lib()
    rng = np.random.default_rng(15)
    x, y, r, s = patch(rng, 8000)
    u = np.zeros(8000, np.float32)
    v = np.zeros(8000, np.float32)
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    n = ctypes.c_int(8000)
    assert L.obs_external_configure(og.CORE_GAUSSIAN, og.COMPENSATED) == 0
    assert L.obs_external_configure_summation(og.SUMMATION_TREE, ctypes.c_double(0.0), 0) == 0
    try:
        fl = L.external_vel_solver_tr_f_(ctypes.byref(n), P(x), P(y), P(s), P(r), ctypes.byref(n), P(x), P(y), P(r),
                                         P(u), P(v))
    finally:
        L.obs_external_configure_summation(og.SUMMATION_DIRECT, ctypes.c_double(0.0), 0)
        L.obs_external_configure(og.CORE_V2, og.COMPENSATED)
    assert fl > 0
    ru, rv, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, x, y, r, s, x, y, r, fp64=True)
    assert rel_err(ru, u) < TOL and rel_err(rv, v) < TOL
