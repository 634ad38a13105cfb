"""GPU tests of the packed-FP32 velocity kernels against the generic kernels and the oracle."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err

pytestmark = pytest.mark.gpu


def cloud(rng, n, uniform):
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = np.full(n, 0.02, np.float32) if uniform else rng.uniform(0.01, 0.04, n).astype(np.float32)
    s = rng.normal(0, 1 / np.sqrt(max(n, 1)), n).astype(np.float32)
    return x, y, r, s


@pytest.mark.parametrize("core", [og.CORE_GAUSSIAN, og.CORE_RM])
@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("uniform", [True, False])
@pytest.mark.parametrize("variant", [og.VARIANT_PACKED2, og.VARIANT_PACKED4])
def test_packed_matches_generic_and_fp64(ctx, restatement, core, thick, accum, uniform, variant):
    rng = np.random.default_rng(core * 100 + thick * 10 + accum + 2 * uniform + variant)
    ns, nt = 5000, 3001
    sx, sy, sr, ss = cloud(rng, ns, uniform)
    tx, ty, tr, _ = cloud(rng, nt, uniform)
    tx[:100], ty[:100], tr[:100] = sx[:100], sy[:100], sr[:100]          # coincident pairs
    outs = {}
    try:
        for v in (og.VARIANT_GENERIC, variant):
            ctx.set_kernel_variant(v)
            t = og.Points(tx, ty, tr if thick else None, None, u=np.full(nt, 0.5, np.float32))
            og.points_affect_points(og.Points(sx, sy, sr, ss), t, og.VELONLY, og.ExecEnv(core, accum, ctx),
                                    finalize=True, fs=(1.0, -0.25))
            outs[v] = (t.u, t.v)
    finally:
        ctx.set_kernel_variant(og.VARIANT_AUTO)
    u64, v64, _ = restatement.points_affect_points(core, 1, sx, sy, sr, ss, tx, ty, tr if thick else None, fp64=True,
                                                   tu=np.full(nt, 0.5), tv=np.zeros(nt))
    u64, v64 = 1.0 + u64 / (2 * np.pi), -0.25 + v64 / (2 * np.pi)
    tol = 2e-6 if accum == og.COMPENSATED else 2e-5
    for v, (u, w) in outs.items():
        assert np.isfinite(u).all() and np.isfinite(w).all()
        assert rel_err(u64, u) < tol and rel_err(v64, w) < tol, v
    assert rel_err(outs[og.VARIANT_GENERIC][0], outs[variant][0]) < tol


@pytest.mark.parametrize("ns,nt", [(1, 1), (255, 33), (257, 1025), (4097, 2049)])
def test_packed_edge_sizes(ctx, restatement, ns, nt):
    rng = np.random.default_rng(ns + nt)
    sx, sy, sr, ss = cloud(rng, ns, True)
    tx, ty, tr, _ = cloud(rng, nt, True)
    t = og.Points(tx, ty, tr, None)
    og.points_affect_points(og.Points(sx, sy, sr, ss), t, og.VELONLY, og.ExecEnv(og.CORE_GAUSSIAN, og.COMPENSATED, ctx))
    u, v, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True)
    assert rel_err(u, t.u) < 2e-6 and rel_err(v, t.v) < 2e-6
