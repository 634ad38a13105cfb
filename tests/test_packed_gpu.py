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


# every core with every variant (PACKED3 means 3 target pairs for the Gaussian core, 2 for the
# others): the host sizes target blocks and the kernel covers them from one table
CORE_VARIANTS = [(c, v) for c in (og.CORE_GAUSSIAN, og.CORE_RM, og.CORE_V2, og.CORE_WL, og.CORE_V3,
                                  og.CORE_SINGULAR, og.CORE_COMPACT_EXP)
                 for v in (og.VARIANT_PACKED2, og.VARIANT_PACKED3, og.VARIANT_PACKED4, og.VARIANT_AUTO)]


@pytest.mark.parametrize("core,variant", CORE_VARIANTS)
@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("uniform", [True, False])
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


def _vel(ctx, src, tx, ty, tr, core, accum, order, variant):
    try:
        ctx.set_kernel_variant(variant)
        ctx.set_target_order(order)
        t = og.Points(tx, ty, tr, None, u=np.full(tx.size, 0.5, np.float32))
        og.points_affect_points(src, t, og.VELONLY, og.ExecEnv(core, accum, ctx), finalize=True, fs=(1.0, -0.25))
    finally:
        ctx.set_kernel_variant(og.VARIANT_AUTO)
        ctx.set_target_order(og.ORDER_AUTO)
    return t.u, t.v


# the far radius of each masked core and an offset that lands in its exponential branch
MASKED = {og.CORE_GAUSSIAN: 3.0, og.CORE_COMPACT_EXP: 1.5}


@pytest.mark.parametrize("core", list(MASKED))
@pytest.mark.parametrize("sigma", [1e-4, 2e-3, 0.05])
@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("variant", [og.VARIANT_PACKED2, og.VARIANT_PACKED3, og.VARIANT_PACKED4])
def test_binned_order_identities(ctx, core, sigma, thick, accum, variant):
    """Binned target order gives the same bits as the caller's order: the far-block fast form and
    the full form agree pair by pair, and each target's sum runs over the sources in one order."""
    rng = np.random.default_rng(int(sigma * 1e5) + 7 * thick + accum + variant + core)
    ns, nt = 9000, 7001
    sx, sy = rng.normal(0, 0.3, (2, ns)).astype(np.float32)
    ss = rng.normal(0, 1e-3, ns).astype(np.float32)
    sr = np.full(ns, sigma, np.float32)
    tx, ty = rng.normal(0, 0.3, (2, nt)).astype(np.float32)
    tx[:300], ty[:300] = sx[:300], sy[:300]                        # coincident pairs: x < 0.001
    tx[300:600] = sx[300:600] + MASKED[core] * sigma               # the exponential branch
    ty[300:600] = sy[300:600]
    tr = np.full(nt, sigma, np.float32) if thick else None
    src = og.Points(sx, sy, sr, ss)
    a = _vel(ctx, src, tx, ty, tr, core, accum, og.ORDER_INPUT, variant)
    b = _vel(ctx, src, tx, ty, tr, core, accum, og.ORDER_BINNED_TARGETS, variant)
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    # binned sources change the summation order only: reproducible, and equal up to rounding
    c = _vel(ctx, src, tx, ty, tr, core, accum, og.ORDER_BINNED, variant)
    d = _vel(ctx, src, tx, ty, tr, core, accum, og.ORDER_BINNED, variant)
    assert np.array_equal(c[0], d[0]) and np.array_equal(c[1], d[1])
    tol = 1e-6 if accum == og.COMPENSATED else 2e-5
    assert rel_err(a[0], c[0]) < tol and rel_err(a[1], c[1]) < tol


@pytest.mark.parametrize("core", list(MASKED))
@pytest.mark.parametrize("sigma", [1e-4, 2e-3])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_binned_targets_vs_fp64(ctx, restatement, core, sigma, accum):
    rng = np.random.default_rng(11 + accum + core)
    ns, nt = 6000, 5003
    sx, sy = rng.normal(0, 0.3, (2, ns)).astype(np.float32)
    ss = rng.normal(0, 1e-3, ns).astype(np.float32)
    sr = np.full(ns, sigma, np.float32)
    tx, ty = rng.normal(0, 0.3, (2, nt)).astype(np.float32)
    tx[:200], ty[:200] = sx[:200], sy[:200]
    tx[200:400], ty[200:400] = sx[200:400] + 2.5 * sigma, sy[200:400]
    tr = np.full(nt, sigma, np.float32)
    u, v = _vel(ctx, og.Points(sx, sy, sr, ss), tx, ty, tr, core, accum, og.ORDER_BINNED, og.VARIANT_AUTO)
    u64, v64, _ = restatement.points_affect_points(core, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True,
                                                   tu=np.full(nt, 0.5), tv=np.zeros(nt))
    u64, v64 = 1.0 + u64 / (2 * np.pi), -0.25 + v64 / (2 * np.pi)
    tol = 2e-6 if accum == og.COMPENSATED else 2e-5
    assert rel_err(u64, u) < tol and rel_err(v64, v) < tol


@pytest.mark.parametrize("nt", [1, 31, 4097])
def test_binned_targets_degenerate(ctx, restatement, nt):
    """All targets on one point, or on one line: the bounding box has zero width."""
    rng = np.random.default_rng(nt)
    ns = 3000
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    ss = rng.normal(0, 1e-2, ns).astype(np.float32)
    sr = np.full(ns, 0.01, np.float32)
    for tx, ty in ((np.full(nt, 0.25, np.float32), np.full(nt, -0.5, np.float32)),
                   (np.linspace(-1, 1, nt).astype(np.float32), np.zeros(nt, np.float32))):
        tr = np.full(nt, 0.01, np.float32)
        u, v = _vel(ctx, og.Points(sx, sy, sr, ss), tx, ty, tr, og.CORE_GAUSSIAN, og.COMPENSATED,
                    og.ORDER_BINNED, og.VARIANT_AUTO)
        u64, v64, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True,
                                                       tu=np.full(nt, 0.5), tv=np.zeros(nt))
        u64, v64 = 1.0 + u64 / (2 * np.pi), -0.25 + v64 / (2 * np.pi)
        assert rel_err(u64, u) < 2e-6 and rel_err(v64, v) < 2e-6


@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_binned_self_interaction_shared_order(ctx, accum):
    """Self-interaction on one set of device arrays reuses the target order for the sources;
    the result equals that of separate copies, whose orders are computed independently."""
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(5 + accum)
    n = 20000
    x, y = rng.normal(0, 0.25, (2, n)).astype(np.float32)
    g = rng.normal(0, 1e-4, n).astype(np.float32)
    r = np.full(n, 0.003, np.float32)
    dev = torch.device("cuda", 0)
    X, Y, R, G = [torch.from_numpy(a).to(dev) for a in (x, y, r, g)]
    outs = []
    try:
        ctx.set_target_order(og.ORDER_BINNED)
        for same in (True, False):
            TU = torch.zeros(n, device=dev)
            TV = torch.zeros(n, device=dev)
            tx, ty, tr = (X, Y, R) if same else (X.clone(), Y.clone(), R.clone())
            og.points_affect_points_dev(ctx, og.CORE_GAUSSIAN, og.VELONLY, accum, X, Y, R, G, tx, ty, tr, TU, TV)
            ctx.synchronize()
            outs.append((TU.cpu().numpy(), TV.cpu().numpy()))
    finally:
        ctx.set_target_order(og.ORDER_AUTO)
    assert np.array_equal(outs[0][0], outs[1][0]) and np.array_equal(outs[0][1], outs[1][1])
    assert np.isfinite(outs[0][0]).all()


def _morton_ref(x, y):
    """Host restatement of the engine's order: float32 cell arithmetic, stable sort."""
    x = np.asarray(x, np.float32)
    y = np.asarray(y, np.float32)

    def cells(v):
        lo, hi = v.min(), v.max()
        w = np.float32(hi - lo)
        sc = np.float32(256.0) / w if w > 0 else np.float32(0.0)
        c = np.minimum(np.maximum((v - lo) * sc, np.float32(0.0)), np.float32(255.0))
        return c.astype(np.uint32)

    def spread(v):
        v = (v | (v << 4)) & 0x0F0F
        v = (v | (v << 2)) & 0x3333
        return (v | (v << 1)) & 0x5555

    key = spread(cells(x)) | (spread(cells(y)) << 1)
    return np.argsort(key, kind="stable")


@pytest.mark.parametrize("n,dist", [(1, "u"), (1000, "u"), (300_001, "n"), (65536, "line"), (5000, "dup")])
def test_morton_order_matches_host_stable_sort(ctx, n, dist):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(n)
    if dist == "u":
        x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    elif dist == "n":
        x, y = rng.normal(0, 0.25, (2, n)).astype(np.float32)
    elif dist == "line":
        x = np.linspace(-3, 5, n).astype(np.float32)
        y = np.full(n, 0.5, np.float32)
    else:
        x, y = rng.integers(0, 4, (2, n)).astype(np.float32)       # many equal keys: stability
    dev = torch.device("cuda", 0)
    X, Y = torch.from_numpy(x).to(dev), torch.from_numpy(y).to(dev)
    P = torch.full((n,), -1, dtype=torch.int32, device=dev)
    og.morton_order_dev(ctx, X, Y, P)
    ctx.synchronize()
    assert np.array_equal(P.cpu().numpy(), _morton_ref(x, y))


@pytest.mark.parametrize("result", [og.VELANDGRAD, og.VELANDVORT, og.VELANDSHEAR])
@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("uniform", [True, False])
@pytest.mark.parametrize("order", [og.ORDER_INPUT, og.ORDER_BINNED])
def test_packed_gradient_results_vs_generic_and_fp64(ctx, restatement, result, thick, accum, uniform, order):
    """Gaussian velocity + gradient / vorticity / shear: the packed kernel (far blocks without the
    exponential) against the generic kernel and the FP64 oracle."""
    rng = np.random.default_rng(result * 10 + thick + 2 * accum + 4 * uniform + order)
    ns, nt = 7000, 4001
    sigma = 0.004
    sx, sy = rng.normal(0, 0.3, (2, ns)).astype(np.float32)
    sr = np.full(ns, sigma, np.float32) if uniform else rng.uniform(0.5 * sigma, 2 * sigma, ns).astype(np.float32)
    ss = rng.normal(0, 1e-3, ns).astype(np.float32)
    tx, ty = rng.normal(0, 0.3, (2, nt)).astype(np.float32)
    tx[:100], ty[:100] = sx[:100], sy[:100]
    tx[100:300], ty[100:300] = sx[100:300] + 4.5 * sigma, sy[100:300]     # between the 16 and 25 cut-offs
    tr = (np.full(nt, sigma, np.float32) if uniform else rng.uniform(0.5 * sigma, 2 * sigma, nt).astype(np.float32))
    outs = {}
    try:
        ctx.set_target_order(order)
        for v in (og.VARIANT_GENERIC, og.VARIANT_AUTO):
            ctx.set_kernel_variant(v)
            t = og.Points(tx, ty, tr if thick else None, None)
            og.points_affect_points(og.Points(sx, sy, sr, ss), t, result, og.ExecEnv(og.CORE_GAUSSIAN, accum, ctx))
            ex = t.grad if result == og.VELANDGRAD else [t.vort if result == og.VELANDVORT else t.shear]
            outs[v] = [t.u, t.v] + list(ex)
    finally:
        ctx.set_kernel_variant(og.VARIANT_AUTO)
        ctx.set_target_order(og.ORDER_AUTO)
    u64, v64, ex64 = restatement.points_affect_points(og.CORE_GAUSSIAN, result, sx, sy, sr, ss, tx, ty,
                                                      tr if thick else None, fp64=True)
    ref = [u64, v64] + list(ex64)
    tol = 2e-6 if accum == og.COMPENSATED else 3e-5
    for v, got in outs.items():
        for k, (a, b) in enumerate(zip(ref, got)):
            ok = np.isfinite(a)
            assert rel_err(a[ok], b[ok]) < tol, (v, k)


@pytest.mark.parametrize("ns,nt", [(300_000, 300_001), (200_000, 1000), (20_000, 70_001)])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("variant", [og.VARIANT_PACKED2, og.VARIANT_PACKED4])
def test_split_reduce_in_kernel_is_deterministic(ctx, restatement, ns, nt, accum, variant):
    """Many source splits per target block.  At 300k x 300k the partials exceed 64 MB and are
    reduced inside the velocity kernel: the block's last split to finish sums them in split
    order, so repeated calls give the same bits whichever split arrives last; the smaller
    shapes take the separate reduction launch.  The sums match FP64, ragged last block
    included."""
    rng = np.random.default_rng(ns + nt + 10 * accum + variant)
    sx, sy, sr, ss = cloud(rng, ns, True)
    tx, ty, tr, _ = cloud(rng, nt, True)
    src = og.Points(sx, sy, sr, ss)
    runs = [_vel(ctx, src, tx, ty, tr, og.CORE_GAUSSIAN, accum, og.ORDER_INPUT, variant) for _ in range(3)]
    for u, v in runs[1:]:
        np.testing.assert_array_equal(u, runs[0][0])
        np.testing.assert_array_equal(v, runs[0][1])
    pick = np.unique(np.concatenate([rng.choice(nt, min(nt, 1500), replace=False), np.arange(max(0, nt - 40), nt)]))
    u64, v64, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx[pick], ty[pick], tr[pick],
                                                   fp64=True, tu=np.full(pick.size, 0.5), tv=np.zeros(pick.size))
    u64, v64 = 1.0 + u64 / (2 * np.pi), -0.25 + v64 / (2 * np.pi)
    tol = 2e-6 if accum == og.COMPENSATED else 5e-5
    assert rel_err(u64, runs[0][0][pick]) < tol and rel_err(v64, runs[0][1][pick]) < tol
