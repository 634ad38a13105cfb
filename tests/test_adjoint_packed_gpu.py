"""GPU tests of the packed-FP32 VJP gathers (Gaussian core) against the generic kernels and the
FP64 reference adjoints of the oracle, in every processing order."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err

pytestmark = pytest.mark.gpu

ORDERS = [og.ORDER_INPUT, og.ORDER_BINNED_TARGETS, og.ORDER_BINNED]


def _with(ctx, variant, order, fn):
    try:
        ctx.set_kernel_variant(variant)
        ctx.set_target_order(order)
        return fn()
    finally:
        ctx.set_kernel_variant(og.VARIANT_AUTO)
        ctx.set_target_order(og.ORDER_AUTO)


def _sources(rng, n, sigma, uniform=True):
    sx, sy = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    sr = (np.full(n, sigma, np.float32) if uniform
          else rng.uniform(0.5 * sigma, 2 * sigma, n).astype(np.float32))
    ss = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    return sx, sy, sr, ss


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("sigma", [0.002, 0.01, 0.2])
@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_probe_vjp_packed_vs_fp64(ctx, restatement, order, sigma, accum):
    """Field-point probes (config-4 shape at reduced size): dL/d(x, y, G) of the sources."""
    rng = np.random.default_rng(int(sigma * 1e4) + order + accum)
    sx, sy, sr, ss = _sources(rng, 12000, sigma)
    g = np.linspace(-0.5, 0.5, 40)
    px, py = [a.ravel().astype(np.float32) for a in np.meshgrid(g, g)]
    px[:50], py[:50] = sx[:50], sy[:50]                           # probes on sources: x < 0.001
    px[50:100], py[50:100] = sx[50:100] + 2 * sigma, sy[50:100]    # the exponential branch
    lu, lv = rng.normal(size=(2, px.size)).astype(np.float32)
    src, probes = og.Points(sx, sy, sr, ss), og.Points(px, py)
    gx, gy, gs = _with(ctx, og.VARIANT_AUTO, order, lambda: og.points_affect_points_vjp(
        src, probes, lu, lv, og.ExecEnv(og.CORE_GAUSSIAN, accum, ctx)))
    rx, ry, rs = restatement.probe_vjp(og.CORE_GAUSSIAN, sx, sy, sr, ss, px, py, lu, lv)
    tol = 1e-5 if accum == og.COMPENSATED else 1e-4
    assert rel_err(rs, gs) < tol and rel_err(rx, gx) < tol and rel_err(ry, gy) < tol


@pytest.mark.parametrize("order", ORDERS)
@pytest.mark.parametrize("uniform", [True, False])
@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_self_vjp_packed_vs_fp64(ctx, restatement, order, uniform, accum):
    rng = np.random.default_rng(3 + order + 2 * uniform + accum)
    n = 9000
    x, y, r, s = _sources(rng, n, 0.01, uniform)
    x[:40], y[:40] = x[40:80], y[40:80] + 1e-4                       # near-coincident pairs
    lu, lv = rng.normal(size=(2, n)).astype(np.float32)
    gx, gy, gs = _with(ctx, og.VARIANT_AUTO, order, lambda: og.points_affect_points_vjp_self(
        og.Points(x, y, r, s), lu, lv, og.ExecEnv(og.CORE_GAUSSIAN, accum, ctx)))
    rx, ry, rs = restatement.self_vjp(og.CORE_GAUSSIAN, x, y, r, s, lu, lv)
    tol = 2e-5 if accum == og.COMPENSATED else 1e-4
    assert rel_err(rx, gx) < tol and rel_err(ry, gy) < tol and rel_err(rs, gs) < tol


@pytest.mark.parametrize("uniform", [True, False])
@pytest.mark.parametrize("accum", [og.COMPENSATED, og.PLAIN_F32])
def test_thick_target_vjp_packed_vs_generic(ctx, uniform, accum):
    """Thick targets (a separate particle set): no FP64 oracle for this form, so the packed
    gather is checked against the generic kernel."""
    rng = np.random.default_rng(17 + uniform + accum)
    sx, sy, sr, ss = _sources(rng, 7000, 0.01, uniform)
    tx, ty, tr, _ = _sources(rng, 5001, 0.01, uniform)
    tx[:30], ty[:30] = sx[:30], sy[:30]
    lu, lv = rng.normal(size=(2, tx.size)).astype(np.float32)
    src, targ = og.Points(sx, sy, sr, ss), og.Points(tx, ty, tr)
    env = og.ExecEnv(og.CORE_GAUSSIAN, accum, ctx)
    a = _with(ctx, og.VARIANT_GENERIC, og.ORDER_INPUT, lambda: og.points_affect_points_vjp(src, targ, lu, lv, env))
    b = _with(ctx, og.VARIANT_AUTO, og.ORDER_BINNED, lambda: og.points_affect_points_vjp(src, targ, lu, lv, env))
    tol = 1e-5 if accum == og.COMPENSATED else 1e-4
    for ga, gb in zip(a, b):
        assert np.isfinite(gb).all()
        assert rel_err(ga, gb) < tol


def test_probe_vjp_binned_reproducible(ctx):
    rng = np.random.default_rng(23)
    sx, sy, sr, ss = _sources(rng, 20000, 0.005)
    px, py = rng.uniform(-0.5, 0.5, (2, 6000)).astype(np.float32)
    lu, lv = rng.normal(size=(2, px.size)).astype(np.float32)
    src, probes = og.Points(sx, sy, sr, ss), og.Points(px, py)
    env = og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx)
    a = _with(ctx, og.VARIANT_AUTO, og.ORDER_BINNED, lambda: og.points_affect_points_vjp(src, probes, lu, lv, env))
    b = _with(ctx, og.VARIANT_AUTO, og.ORDER_BINNED, lambda: og.points_affect_points_vjp(src, probes, lu, lv, env))
    for ga, gb in zip(a, b):
        assert np.array_equal(ga, gb)
