"""GPU parity tests of the particle-on-particle engine (points_affect_points) through the C ABI,
against the golden vectors from the reference's compiled code and against the oracle."""
import ctypes

import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err
from oracle import pyoracle as po

pytestmark = pytest.mark.gpu

REF_CORES = {"rm": og.CORE_RM, "exp": og.CORE_GAUSSIAN, "v2": og.CORE_V2, "wl": og.CORE_WL, "v3": og.CORE_V3}
# Tolerances (normwise max relative error vs the reference's float-pair/double-accumulator
# results).  Pair math differs from the reference only by the rounding of the hardware
# reciprocal/rsqrt/exp2/log2 approximations (<= 2 ulp); accumulation order differs as well.
TOL = {og.PLAIN_F32: 2e-5, og.COMPENSATED: 3e-6}


def run(ctx, core, restype, accum, src, targ, finalize=False, fs=(0.0, 0.0)):
    env = og.ExecEnv(core=core, accum=accum, context=ctx)
    return og.points_affect_points(src, targ, restype, env, finalize=finalize, fs=fs)


@pytest.mark.parametrize("name", list(REF_CORES))
@pytest.mark.parametrize("restype", [og.VELONLY, og.VELANDVORT, og.VELANDSHEAR])
@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_p2p_matches_reference_golden(ctx, golden, name, restype, thick, accum):
    g = golden("p2p")
    key = f"{name}_r{restype}_{'b' if thick else 'p'}"
    src = og.Points(g["sx"], g["sy"], g["sr"], g["ss"])
    targ = og.Points(g["tx"], g["ty"], g["tr"] if thick else None, None, u=g["tu0"].copy(), v=g["tv0"].copy())
    if restype == og.VELANDVORT:
        targ.vort = g["ex0"].copy()
    if restype == og.VELANDSHEAR:
        targ.shear = g["ex0"].copy()
    run(ctx, REF_CORES[name], restype, accum, src, targ)
    outs = [(g[key + "_u"], targ.u), (g[key + "_v"], targ.v)]
    if restype == og.VELANDVORT:
        outs.append((g[key + "_e"], targ.vort))
    if restype == og.VELANDSHEAR:
        outs.append((g[key + "_e"], targ.shear))
    for ref, got in outs:
        ok = np.isfinite(ref)     # reference NaN: Gaussian gradient form on coincident pairs
        assert np.isfinite(got).all()
        assert rel_err(ref[ok], got[ok]) < TOL[accum]


@pytest.mark.parametrize("name", list(REF_CORES))
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_p2p_gradients_match_reference_golden(ctx, golden, name, accum):
    g = golden("p2p")
    src = og.Points(g["sx"], g["sy"], g["sr"], g["ss"])
    targ = og.Points(g["tx"], g["ty"], g["tr"], None)
    run(ctx, REF_CORES[name], og.VELANDGRAD, accum, src, targ)
    got = [targ.u, targ.v] + targ.grad
    for k, nm in enumerate(["u", "v", "ux", "vx", "uy", "vy"]):
        ref = g[f"{name}_grad_{nm}"]
        ok = np.isfinite(ref)
        assert rel_err(ref[ok], got[k][ok]) < TOL[accum], nm


@pytest.mark.parametrize("core", [og.CORE_SINGULAR, og.CORE_COMPACT_EXP])
@pytest.mark.parametrize("restype", [og.VELONLY, og.VELANDGRAD, og.VELANDVORT])
@pytest.mark.parametrize("thick", [True, False])
def test_p2p_builder_cores_match_fp64_restatement(ctx, restatement, core, restype, thick):
    """Cores the reference lacks: pinned only to the FP64 restatement."""
    rng = np.random.default_rng(7 + core)
    ns, nt = 1000, 700
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = rng.uniform(0.02, 0.06, ns).astype(np.float32)
    ss = rng.normal(0, 0.03, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tx[:50], ty[:50] = sx[:50], sy[:50]
    tr = rng.uniform(0.02, 0.06, nt).astype(np.float32)
    src = og.Points(sx, sy, sr, ss)
    targ = og.Points(tx, ty, tr if thick else None, None)
    run(ctx, core, restype, og.COMPENSATED, src, targ)
    u, v, ex = restatement.points_affect_points(core, restype, sx, sy, sr, ss, tx, ty, tr if thick else None, fp64=True)
    assert rel_err(u, targ.u) < 2e-5 and rel_err(v, targ.v) < 2e-5
    if restype == og.VELANDGRAD:
        for k in range(4):
            assert rel_err(ex[k], targ.grad[k]) < 5e-5
    if restype == og.VELANDVORT:
        if core == og.CORE_SINGULAR:
            # point vortices are irrotational away from the centres: the exact value is 0 and
            # the engine's value is rounding noise of b d^2 + 2K; bound it by the gradient scale
            _, _, gx = restatement.points_affect_points(core, og.VELANDGRAD, sx, sy, sr, ss, tx, ty,
                                                        tr if thick else None, fp64=True)
            assert np.max(np.abs(targ.vort - ex[0])) < 1e-5 * np.max(np.abs(gx[2]))
        else:
            assert rel_err(ex[0], targ.vort) < 5e-5


@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_p2p_streamfunction(ctx, restatement, thick, accum):
    rng = np.random.default_rng(21)
    ns, nt = 900, 400
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = rng.uniform(0.02, 0.06, ns).astype(np.float32)
    ss = rng.normal(0, 0.03, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tr = rng.uniform(0.02, 0.06, nt).astype(np.float32)
    src = og.Points(sx, sy, sr, ss)
    targ = og.Points(tx, ty, tr if thick else None, None)
    u0 = targ.u.copy()
    run(ctx, og.CORE_V2, og.PSIONLY, accum, src, targ)
    _, _, ex = restatement.points_affect_points(og.CORE_V2, po.PSIONLY, sx, sy, sr, ss, tx, ty,
                                                tr if thick else None, fp64=True)
    assert rel_err(ex[0], targ.psi) < 2e-5
    np.testing.assert_array_equal(targ.u, u0)   # psionly leaves the velocity untouched


@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
@pytest.mark.parametrize("core", [og.CORE_V2, og.CORE_GAUSSIAN])
def test_p2p_streamfunction_matches_reference_golden(ctx, golden, thick, accum, core):
    """psionly against the reference's kernelp_0v_0b / kernelp_0v_0p (src/Kernels.h:52-74);
    the kernel is the same for every core (radius term sr^2 + tr^2), 30 coincident pairs."""
    g = golden("pins")
    src = og.Points(g["sx"], g["sy"], g["sr"], g["ss"])
    targ = og.Points(g["tx"], g["ty"], g["tr"] if thick else None, None)
    targ.psi = g["tp0"].copy()
    run(ctx, core, og.PSIONLY, accum, src, targ)
    assert np.isfinite(targ.psi).all()
    assert rel_err(g["psi_b" if thick else "psi_p"], targ.psi) < TOL[accum]


@pytest.mark.parametrize("thick", [True, False])
@pytest.mark.parametrize("accum", [og.PLAIN_F32, og.COMPENSATED])
def test_p2p_singular_matches_reference_golden(ctx, golden, thick, accum):
    """The singular core against the reference's Rosenhead-Moore core with zero radii
    (src/CoreFunc.h:42-82) on targets off the sources; the singular core ignores radii."""
    g = golden("pins")
    k = "b" if thick else "p"
    for sr in (np.zeros_like(g["sr"]), g["sr"]):
        src = og.Points(g["sx"], g["sy"], sr, g["ss"])
        targ = og.Points(g["qx"], g["qy"], np.full(g["qx"].size, 0.03, np.float32) if thick else None, None)
        run(ctx, og.CORE_SINGULAR, og.VELONLY, accum, src, targ)
        assert rel_err(g[f"sing_{k}_u"], targ.u) < TOL[accum] and rel_err(g[f"sing_{k}_v"], targ.v) < TOL[accum]
    src = og.Points(g["sx"], g["sy"], g["sr"], g["ss"])
    targ = og.Points(g["qx"], g["qy"], np.full(g["qx"].size, 0.03, np.float32), None)
    run(ctx, og.CORE_SINGULAR, og.VELANDGRAD, accum, src, targ)
    for ref, got in zip([g[f"sing_grad_{nm}"] for nm in ("u", "v", "ux", "vx", "uy", "vy")], [targ.u, targ.v] + targ.grad):
        assert rel_err(ref, got) < TOL[accum]


SIZES = [0, 1, 2, 31, 33, 255, 257, 1031]


@pytest.mark.parametrize("ns", SIZES)
@pytest.mark.parametrize("nt", [0, 1, 33, 513, 2049])
def test_p2p_edge_sizes(ctx, restatement, ns, nt):
    rng = np.random.default_rng(ns * 7919 + nt)
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = np.full(ns, 0.05, np.float32)
    ss = rng.normal(0, 0.1, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tr = np.full(nt, 0.05, np.float32)
    for accum in (og.PLAIN_F32, og.COMPENSATED):
        src = og.Points(sx, sy, sr, ss)
        targ = og.Points(tx, ty, tr, None, u=np.ones(nt, np.float32), v=-np.ones(nt, np.float32))
        run(ctx, og.CORE_GAUSSIAN, og.VELONLY, accum, src, targ)
        u, v, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True,
                                                   tu=np.ones(nt), tv=-np.ones(nt))
        if nt:
            assert rel_err(u, targ.u) < 1e-5 and rel_err(v, targ.v) < 1e-5


def test_p2p_finalize_flag(ctx, restatement):
    rng = np.random.default_rng(3)
    n = 3000
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = np.full(n, 0.01, np.float32)
    s = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    p = og.Points(x, y, r, s)
    run(ctx, og.CORE_RM, og.VELONLY, og.COMPENSATED, p, p, finalize=True, fs=(1.0, 0.25))
    u, v, _ = restatement.points_affect_points(og.CORE_RM, 1, x, y, r, s, x, y, r, fp64=True)
    u, v = 1.0 + u / (2 * np.pi), 0.25 + v / (2 * np.pi)
    assert np.max(np.abs(u - p.u)) < 1e-6 and np.max(np.abs(v - p.v)) < 1e-6


def test_p2p_compensated_precision_vs_fp64(ctx, restatement):
    """Gaussian patch (positions N(0, 0.25^2), strength ~ exp(-r^2/0.125) normalised to 1,
    core 0.005): compensated FP32 within 1e-6 of the FP64 oracle; plain FP32 measured beside."""
    rng = np.random.default_rng(2)
    n = 200_000
    x, y = rng.normal(0, 0.25, (2, n)).astype(np.float32)
    s = np.exp(-(x.astype(np.float64) ** 2 + y.astype(np.float64) ** 2) / 0.125)
    s = (s / s.sum()).astype(np.float32)
    r = np.full(n, 0.005, np.float32)
    sub = rng.choice(n, 1024, replace=False)
    u64, v64, _ = restatement.points_affect_points(og.CORE_GAUSSIAN, 1, x, y, r, s, x[sub], y[sub], r[sub], fp64=True)
    errs = {}
    for accum in (og.PLAIN_F32, og.COMPENSATED):
        src = og.Points(x, y, r, s)
        targ = og.Points(x[sub], y[sub], r[sub], None)
        run(ctx, og.CORE_GAUSSIAN, og.VELONLY, accum, src, targ)
        ref = np.concatenate([u64, v64])
        got = np.concatenate([targ.u, targ.v])
        errs[accum] = rel_err(ref, got)
    assert errs[og.COMPENSATED] < 1e-6, errs
    assert errs[og.PLAIN_F32] < 1e-4, errs


def test_p2p_self_interaction_momentum(ctx):
    """sum_i G_i u_i = 0 for equal cores (pairwise antisymmetry), at a size well past one tile."""
    rng = np.random.default_rng(9)
    n = 100_000
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = np.full(n, 0.01, np.float32)
    s = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    p = og.Points(x, y, r, s)
    run(ctx, og.CORE_GAUSSIAN, og.VELONLY, og.COMPENSATED, p, p)
    sd = s.astype(np.float64)
    scale = np.sum(np.abs(sd) * np.hypot(p.u, p.v))
    assert abs(np.sum(sd * p.u)) < 1e-6 * scale and abs(np.sum(sd * p.v)) < 1e-6 * scale


def test_p2p_linearity_in_strength(ctx):
    rng = np.random.default_rng(10)
    n = 50_000
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = np.full(n, 0.01, np.float32)
    s1 = rng.normal(0, 1, n).astype(np.float32)
    s2 = rng.normal(0, 1, n).astype(np.float32)
    outs = []
    for s in (s1, s2, s1 + s2):
        t = og.Points(x[:4096], y[:4096], r[:4096], None)
        run(ctx, og.CORE_V2, og.VELONLY, og.COMPENSATED, og.Points(x, y, r, s), t)
        outs.append(t.u.astype(np.float64))
    assert rel_err(outs[2], outs[0] + outs[1]) < 2e-6


def test_device_entry_point_with_torch_tensors(ctx, restatement):
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(4)
    n = 20_000
    x, y = rng.uniform(-1, 1, (2, n)).astype(np.float32)
    r = np.full(n, 0.01, np.float32)
    s = rng.normal(0, 1 / np.sqrt(n), n).astype(np.float32)
    dev = torch.device("cuda:0")
    T = [torch.from_numpy(a).to(dev) for a in (x, y, r, s)]
    tu = torch.zeros(n, device=dev)
    tv = torch.zeros(n, device=dev)
    stream = torch.cuda.Stream(dev)
    ctx.set_stream(stream.cuda_stream)
    try:
        stream.wait_stream(torch.cuda.current_stream())
        og.points_affect_points_dev(ctx, og.CORE_RM, og.VELONLY, og.COMPENSATED, *T, T[0], T[1], T[2], tu, tv)
        stream.synchronize()
        ctx.synchronize()
    finally:
        ctx.set_stream(None)
    u, v, _ = restatement.points_affect_points(og.CORE_RM, 1, x, y, r, s, x, y, r, fp64=True)
    assert rel_err(u, tu.cpu().numpy()) < 2e-6 and rel_err(v, tv.cpu().numpy()) < 2e-6


def test_external_solver_hooks(restatement):
    """The reference's own FFI (src/Influence.h:31-38): accumulate, unscaled, return flops."""
    L = og.lib()
    rng = np.random.default_rng(6)
    ns, nt = 3000, 1000
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = np.full(ns, 0.02, np.float32)
    ss = rng.normal(0, 0.02, ns).astype(np.float32)
    tx, ty = rng.uniform(-1, 1, (2, nt)).astype(np.float32)
    tr = np.full(nt, 0.02, np.float32)
    assert L.obs_external_configure(og.CORE_V2, og.COMPENSATED) == 0
    P = lambda a: a.ctypes.data_as(ctypes.c_void_p)
    NS, NT = ctypes.c_int(ns), ctypes.c_int(nt)
    tu = np.full(nt, 0.5, np.float32); tv = np.zeros(nt, np.float32)
    fl = L.external_vel_solver_f_(ctypes.byref(NS), P(sx), P(sy), P(ss), P(sr), ctypes.byref(NT), P(tx), P(ty), P(tu), P(tv))
    assert fl == pytest.approx(nt * (2 + 16 * ns), rel=1e-6)
    u, v, _ = restatement.points_affect_points(og.CORE_V2, 1, sx, sy, sr, ss, tx, ty, None, fp64=True,
                                               tu=np.full(nt, 0.5), tv=np.zeros(nt))
    assert rel_err(u, tu) < 2e-6 and rel_err(v, tv) < 2e-6
    tu = np.zeros(nt, np.float32); tv = np.zeros(nt, np.float32)
    L.external_vel_solver_tr_f_(ctypes.byref(NS), P(sx), P(sy), P(ss), P(sr), ctypes.byref(NT), P(tx), P(ty), P(tr), P(tu), P(tv))
    u, v, _ = restatement.points_affect_points(og.CORE_V2, 1, sx, sy, sr, ss, tx, ty, tr, fp64=True)
    assert rel_err(u, tu) < 2e-6 and rel_err(v, tv) < 2e-6
    d = [a.astype(np.float64) for a in (sx, sy, ss, sr, tx, ty)]
    tu = np.zeros(nt); tv = np.zeros(nt)
    L.external_vel_solver_d_(ctypes.byref(NS), *[P(a) for a in d[:4]], ctypes.byref(NT), P(d[4]), P(d[5]), P(tu), P(tv))
    assert rel_err(u * 0 + restatement.points_affect_points(og.CORE_V2, 1, sx, sy, sr, ss, tx, ty, None, fp64=True)[0], tu) < 1e-12
