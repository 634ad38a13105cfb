"""CPU tests of the oracle: the C restatement (oracle/oracle.c) pinned against the golden
vectors produced by the reference's own compiled code, against the live reference build where
it exists, and against analytic known answers."""
import numpy as np
import pytest

from conftest import rel_err
from oracle import pyoracle as po

CORES = {"rm": po.RM, "exp": po.GAUSS, "v2": po.V2, "wl": po.WL, "v3": po.V3}
TOL_F32 = 2e-6   # float pair math vs the reference's float pair math (contraction differences)


@pytest.mark.parametrize("name", list(CORES))
@pytest.mark.parametrize("restype", [po.VELONLY, po.VELANDVORT, po.VELANDSHEAR])
@pytest.mark.parametrize("thick", [True, False])
def test_restatement_p2p_golden(restatement, golden, name, restype, thick):
    g = golden("p2p")
    key = f"{name}_r{restype}_{'b' if thick else 'p'}"
    tu, tv, ex = restatement.points_affect_points(
        CORES[name], restype, g["sx"], g["sy"], g["sr"], g["ss"], g["tx"], g["ty"],
        g["tr"] if thick else None, tu=g["tu0"], tv=g["tv0"],
        extra=None if restype == po.VELONLY else [g["ex0"]])
    outs = [(g[key + "_u"], tu), (g[key + "_v"], tv)]
    if restype != po.VELONLY:
        outs.append((g[key + "_e"], ex[0]))
    for ref, got in outs:
        ok = np.isfinite(ref)
        # the reference's Gaussian gradient-form core is 0*inf = NaN on coincident pairs
        # (src/CoreFunc.h:157-166); the restatement uses the finite limit there
        if name != "exp" or restype == po.VELONLY:
            assert ok.all()
        assert np.isfinite(got).all()
        assert rel_err(ref[ok], got[ok]) < TOL_F32


@pytest.mark.parametrize("name", list(CORES))
def test_restatement_grad_golden(restatement, golden, name):
    g = golden("p2p")
    tu, tv, ex = restatement.points_affect_points(CORES[name], po.VELANDGRAD, g["sx"], g["sy"], g["sr"], g["ss"],
                                                  g["tx"], g["ty"], g["tr"])
    got = [tu, tv] + ex
    for k, nm in enumerate(["u", "v", "ux", "vx", "uy", "vy"]):
        ref = g[f"{name}_grad_{nm}"]
        ok = np.isfinite(ref)
        assert rel_err(ref[ok], got[k][ok]) < TOL_F32, nm
    if name == "exp":   # NaN exactly on the 40 coincident targets in the reference
        assert (~np.isfinite(g["exp_grad_ux"])).sum() == 40


def test_restatement_panels_golden(restatement, golden):
    g = golden("panels")
    u, v = restatement.panels_affect_points(g["nx"], g["ny"], g["idx"], g["vs"], g["ss"], g["tx"], g["ty"])
    assert rel_err(g["p2pt_1vs_u"], u) < 2e-6 and rel_err(g["p2pt_1vs_v"], v) < 2e-6
    u, v = restatement.panels_affect_points(g["nx"], g["ny"], g["idx"], g["vs"], None, g["tx"], g["ty"])
    assert rel_err(g["p2pt_1v_u"], u) < 2e-6 and rel_err(g["p2pt_1v_v"], v) < 2e-6
    pu, pv = restatement.points_affect_panels(g["tx"], g["ty"], g["tg"], g["nx"], g["ny"], g["idx"])
    assert rel_err(g["pt2p_u"], pu) < 2e-6 and rel_err(g["pt2p_v"], pv) < 2e-6
    A = restatement.panels_on_panels_coeff(2, g["nx"], g["ny"], g["idx"])
    assert rel_err(g["coeff"], A) < 1e-6
    rhs = restatement.vels_to_rhs_panels(2, g["nx"], g["ny"], g["idx"], g["pu"], g["pv"], g["bcn"])
    assert rel_err(g["rhs"], rhs) < 1e-6
    fu, fv = restatement.finalize_vels(g["pu"], g["pv"], (1.0, -0.5))
    np.testing.assert_array_equal(fu, g["fin_u"])
    np.testing.assert_array_equal(fv, g["fin_v"])


def test_restatement_advect_golden(restatement, golden):
    g = golden("advect")
    x, y = restatement.advect(1, po.RM, g["x"], g["y"], g["r"], g["s"], (1.0, 0.0), 0.01, 10)
    assert np.max(np.abs(x - g["euler_x"])) < 1e-6 and np.max(np.abs(y - g["euler_y"])) < 1e-6
    x, y = restatement.advect(2, po.GAUSS, g["x"], g["y"], g["r"], g["s"], (0.0, 0.0), 0.01, 4)
    assert np.max(np.abs(x - g["rk2_x"])) < 1e-6 and np.max(np.abs(y - g["rk2_y"])) < 1e-6


def test_reference_flop_counts(golden):
    g = golden("p2p")
    # flopsu_0v_0b, 0v_0p, ug_0v_0b, uw_0v_0b, ue_0v_0b, u_1v_0p, u_1vs_0p, u_1vos_0p
    assert list(g["exp_flops"]) == [19, 17, 41, 35, 39, 39, 47, 45]
    assert list(g["rm_flops"])[:3] == [15, 13, 34]
    assert list(g["v2_flops"])[:3] == [19, 16, 38]


@pytest.mark.skipif(not po.Reference.available(), reason="reference tree not built here")
@pytest.mark.parametrize("seed", [1, 2])
def test_restatement_vs_live_reference(restatement, seed):
    rng = np.random.default_rng(seed)
    ns, nt = 611, 333
    sx, sy = rng.uniform(-1, 1, (2, ns)).astype(np.float32)
    sr = rng.uniform(0.01, 0.1, ns).astype(np.float32)
    ss = rng.normal(0, 0.05, ns).astype(np.float32)
    tx, ty = rng.uniform(-1.2, 1.2, (2, nt)).astype(np.float32)
    tr = rng.uniform(0.01, 0.1, nt).astype(np.float32)
    for name, core in CORES.items():
        ref = po.Reference(core)
        for thick in (True, False):
            a = ref.points_affect_points(po.VELONLY, sx, sy, sr, ss, tx, ty, tr if thick else None)
            b = restatement.points_affect_points(core, po.VELONLY, sx, sy, sr, ss, tx, ty, tr if thick else None)
            assert rel_err(a[0], b[0]) < TOL_F32 and rel_err(a[1], b[1]) < TOL_F32
            a = ref.points_affect_points(po.VELONLY, sx, sy, sr, ss, tx, ty, tr if thick else None, fp64=True)
            b = restatement.points_affect_points(core, po.VELONLY, sx, sy, sr, ss, tx, ty, tr if thick else None,
                                                 fp64=True)
            assert rel_err(a[0], b[0]) < 1e-13 and rel_err(a[1], b[1]) < 1e-13


def test_analytic_single_vortex(restatement):
    """Tangential speed of one vortex of circulation G at distance r (after /(2 pi)):
    singular G/(2 pi r); RM G r/(2 pi (r^2 + s^2)); Gaussian G/(2 pi r)(1 - exp(-r^2/s^2))."""
    G, s = 0.7, 0.1
    r = np.array([0.03, 0.1, 0.25, 1.0, 3.0])
    tx, ty = r, np.zeros_like(r)
    for core, expect in [
        (po.SINGULAR, G / r),
        (po.RM, G * r / (r * r + s * s)),
        (po.GAUSS, G / r * (1 - np.exp(-r * r / (s * s)))),
    ]:
        u, v, _ = restatement.points_affect_points(core, po.VELONLY, [0.0], [0.0], [s], [G], tx, ty, None, fp64=True)
        assert np.max(np.abs(u)) < 1e-15
        np.testing.assert_allclose(v, expect, rtol=1e-12)


def test_self_interaction_antisymmetry(restatement):
    """With equal cores, sum_i G_i u_i = 0 for the self-interaction (linear impulse is
    conserved): each pair contributes G_i G_j K (-dy, dx) + G_j G_i K (dy, -dx) = 0."""
    rng = np.random.default_rng(5)
    n = 800
    x, y = rng.uniform(-1, 1, (2, n))
    r = np.full(n, 0.02)
    s = rng.normal(0, 1, n)
    for core in (po.RM, po.GAUSS, po.V2, po.WL, po.V3, po.CEXP):
        u, v, _ = restatement.points_affect_points(core, po.VELONLY, x, y, r, s, x, y, r, fp64=True)
        scale = np.sum(np.abs(s) * np.hypot(u, v))
        assert abs(np.sum(s * u)) < 1e-12 * scale and abs(np.sum(s * v)) < 1e-12 * scale


def test_probe_vjp_matches_finite_differences(restatement):
    rng = np.random.default_rng(11)
    ns, npb = 60, 40
    sx, sy = rng.uniform(-1, 1, (2, ns))
    sr = np.full(ns, 0.2)
    ss = rng.normal(0, 1, ns)
    px, py = rng.uniform(-0.5, 0.5, (2, npb))

    def loss(sx_, sy_, ss_):
        u, v, _ = restatement.points_affect_points(po.GAUSS, po.VELONLY, sx_, sy_, sr, ss_, px, py, None, fp64=True)
        u, v = u / (2 * np.pi), v / (2 * np.pi)
        return np.sum(u * u + v * v), u, v

    L, u, v = loss(sx, sy, ss)
    gx, gy, gs = restatement.probe_vjp(po.GAUSS, sx, sy, sr, ss, px, py, 2 * u, 2 * v)
    for j in rng.choice(ns, 8, replace=False):
        for arr, g in ((sx, gx), (sy, gy), (ss, gs)):
            h = 1e-6
            a = arr.copy(); a[j] += h
            b = arr.copy(); b[j] -= h
            args_p = [a if arr is q else q for q in (sx, sy, ss)]
            args_m = [b if arr is q else q for q in (sx, sy, ss)]
            fd = (loss(*args_p)[0] - loss(*args_m)[0]) / (2 * h)
            assert abs(fd - g[j]) < 1e-6 * max(1.0, abs(fd))


def test_rk2_centroid_gradient_matches_finite_differences(restatement):
    rng = np.random.default_rng(12)
    n = 80
    lab = (np.arange(n) >= n // 2).astype(np.int32)
    x = np.where(lab == 0, -0.3, 0.3) + rng.normal(0, 0.1, n)
    y = rng.normal(0, 0.1, n)
    r = np.full(n, 0.05)
    s = np.abs(rng.normal(1.0 / (n // 2), 0.3 / n, n))
    args = (po.GAUSS, x, y, r, s, lab, (0.0, 0.0), 0.02, 6)
    L, gs, gx, gy = restatement.rk2_centroid_grad(*args)
    assert abs(L - restatement.rk2_centroid_loss(*args)) < 1e-14
    for j in rng.choice(n, 6, replace=False):
        h = 1e-7
        sp = s.copy(); sp[j] += h
        sm = s.copy(); sm[j] -= h
        fd = (restatement.rk2_centroid_loss(po.GAUSS, x, y, r, sp, lab, (0.0, 0.0), 0.02, 6)
              - restatement.rk2_centroid_loss(po.GAUSS, x, y, r, sm, lab, (0.0, 0.0), 0.02, 6)) / (2 * h)
        assert abs(fd - gs[j]) < 1e-6 * max(1.0, abs(fd)), (j, fd, gs[j])
        xp = x.copy(); xp[j] += h
        xm = x.copy(); xm[j] -= h
        fd = (restatement.rk2_centroid_loss(po.GAUSS, xp, y, r, s, lab, (0.0, 0.0), 0.02, 6)
              - restatement.rk2_centroid_loss(po.GAUSS, xm, y, r, s, lab, (0.0, 0.0), 0.02, 6)) / (2 * h)
        assert abs(fd - gx[j]) < 1e-6 * max(1.0, abs(fd)), (j, fd, gx[j])


def test_restatement_blob_vorticity_golden(restatement, golden):
    g = golden("extras")
    w = restatement.points_affect_points_vorticity(g["sx"], g["sy"], g["sr"], g["ss"], g["tx"], g["ty"], g["tw0"])
    assert rel_err(g["vort_w"], w) < 1e-6


def test_restatement_panels_on_panels_golden(restatement, golden):
    g = golden("extras")
    pu, pv = restatement.panels_affect_panels(g["snx"], g["sny"], g["sidx"], g["vs"], g["sss"],
                                              g["tnx"], g["tny"], g["tidx"], g["pu0"], g["pv0"])
    # collocation points sit 1e-4 off the panels: FP32 atan2/log rounding is amplified there
    assert rel_err(g["pap_u"], pu) < 5e-6 and rel_err(g["pap_v"], pv) < 5e-6


@pytest.mark.parametrize("order,key,core,fs", [(3, "rk3", 2, (0.5, 0.0)), (4, "heun", 1, (0.0, 0.25))])
def test_restatement_rk3_heun_golden(restatement, golden, order, key, core, fs):
    g = golden("extras")
    x, y = restatement.advect(order, core, g["x"], g["y"], g["r"], g["s"], fs, 0.01, 4)
    disp = np.max(np.hypot(g[key + "_x"] - g["x"], g[key + "_y"] - g["y"]))
    assert np.max(np.hypot(x - g[key + "_x"], y - g[key + "_y"])) < 2e-5 * disp


@pytest.mark.parametrize("thick", [True, False])
def test_restatement_streamfunction_golden(restatement, golden, thick):
    """psionly against the reference's kernelp_0v_0b / kernelp_0v_0p (src/Kernels.h:52-74)."""
    g = golden("pins")
    _, _, ex = restatement.points_affect_points(po.V2, po.PSIONLY, g["sx"], g["sy"], g["sr"], g["ss"], g["tx"],
                                                g["ty"], g["tr"] if thick else None, extra=[g["tp0"]])
    assert np.isfinite(ex[0]).all()
    assert rel_err(g["psi_b" if thick else "psi_p"], ex[0]) < TOL_F32


@pytest.mark.parametrize("thick", [True, False])
def test_restatement_singular_golden(restatement, golden, thick):
    """The singular core against the reference's Rosenhead-Moore core with zero radii
    (src/CoreFunc.h:42-82) on targets off the sources; the singular core ignores the radii."""
    g = golden("pins")
    k = "b" if thick else "p"
    for sr in (np.zeros_like(g["sr"]), g["sr"]):
        tu, tv, _ = restatement.points_affect_points(po.SINGULAR, po.VELONLY, g["sx"], g["sy"], sr, g["ss"],
                                                     g["qx"], g["qy"], np.zeros_like(g["qx"]) if thick else None)
        assert rel_err(g[f"sing_{k}_u"], tu) < TOL_F32 and rel_err(g[f"sing_{k}_v"], tv) < TOL_F32
    tu, tv, ex = restatement.points_affect_points(po.SINGULAR, po.VELANDGRAD, g["sx"], g["sy"], g["sr"], g["ss"],
                                                  g["qx"], g["qy"], g["sr"][:g["qx"].size])
    for ref, got in zip([g[f"sing_grad_{nm}"] for nm in ("u", "v", "ux", "vx", "uy", "vy")], [tu, tv] + ex):
        assert rel_err(ref, got) < TOL_F32


@pytest.mark.skipif(not po.Reference.available(po.RM), reason="reference tree not built here")
def test_live_reference_streamfunction_fp64(restatement):
    """FP64: the restatement's psionly equals the reference's kernelp in double to rounding."""
    rng = np.random.default_rng(5)
    sx, sy = rng.uniform(-1, 1, (2, 400))
    sr = rng.uniform(0.01, 0.1, 400)
    ss = rng.normal(0, 0.05, 400)
    tx, ty = rng.uniform(-1.2, 1.2, (2, 150))
    tr = rng.uniform(0.01, 0.1, 150)
    ref = po.Reference(po.RM)
    for thick in (True, False):
        a = ref.psi(sx, sy, sr, ss, tx, ty, tr if thick else None, fp64=True)
        _, _, b = restatement.points_affect_points(po.RM, po.PSIONLY, sx, sy, sr, ss, tx, ty,
                                                   tr if thick else None, fp64=True)
        assert rel_err(a, b[0]) < 1e-13
