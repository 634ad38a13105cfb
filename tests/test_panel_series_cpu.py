"""The series forms of the panel sums (omega2d_gb300/csrc/panels.cu, panel_uv_star_fast2),
restated in FP64 numpy.  The subtended angle of a panel seen from a target is the arctangent of
r = cross/dot, and the half-log 0.5 log(r0^2/r1^2) is atanh(s) with s = (r0^2 - r1^2)/(r0^2 + r1^2)
(src/Kernels.h:256-268, 330-338 form them as a difference of two atan2 values and a log of the
ratio).  Where both |r| and |s| are below 0.05 the kernel ends both odd series at the 5th power,
below 0.2 at the 9th.  CPU only: these pin the identities, the truncation bounds and the claim
that every pair of the BEM coupling workload takes the 5th-power form; the GPU tests pin the
kernels against the oracle."""
import numpy as np
import pytest

import omega2d_gb300 as og


def atan5(r):
    t = r * r
    return r + r * t * (t * 0.2 - 1.0 / 3.0)


def atanh5(s):
    t = s * s
    return s + s * t * (t * 0.2 + 1.0 / 3.0)


def atan9(r):
    t = r * r
    p = ((t / 9.0 - 1.0 / 7.0) * t + 0.2) * t - 1.0 / 3.0
    return r + r * t * p


def atanh9(s):
    t = s * s
    q = ((t / 9.0 + 1.0 / 7.0) * t + 0.2) * t + 1.0 / 3.0
    return s + s * t * q


def test_series_truncation_bounds():
    """5th power: below 2.3e-9 relative for |x| <= 0.05; 9th power: below 1e-8 for |x| <= 0.2
    (the first omitted terms, x^6/7 and x^10/11, bound the error)."""
    x = np.concatenate([np.linspace(-0.05, 0.05, 20001), [-0.05, 0.05]])
    x = x[x != 0.0]
    assert np.max(np.abs(atan5(x) / np.arctan(x) - 1.0)) < 2.3e-9
    assert np.max(np.abs(atanh5(x) / np.arctanh(x) - 1.0)) < 2.3e-9
    y = np.linspace(-0.2, 0.2, 40001)
    y = y[y != 0.0]
    assert np.max(np.abs(atan9(y) / np.arctan(y) - 1.0)) < 1e-8
    assert np.max(np.abs(atanh9(y) / np.arctanh(y) - 1.0)) < 1e-8


def pair_quantities(p0, p1, t):
    """cross, dot, r0^2 - r1^2 and r0^2 + r1^2 of every (panel, target) pair as the kernel forms
    them: d0 = t - p0, d1 = t - p1, cross = d0 x (p1 - p0), dot = d0 . d1."""
    d0x, d0y = t[:, None, 0] - p0[None, :, 0], t[:, None, 1] - p0[None, :, 1]
    d1x, d1y = t[:, None, 0] - p1[None, :, 0], t[:, None, 1] - p1[None, :, 1]
    px, py = (p1 - p0)[:, 0], (p1 - p0)[:, 1]
    cr = d0x * py[None, :] - d0y * px[None, :]
    dt = d0x * d1x + d0y * d1y
    diff = px[None, :] * (d0x + d1x) + py[None, :] * (d0y + d1y)
    r1 = d1x * d1x + d1y * d1y
    return cr, dt, diff, 2.0 * r1 + diff, d0x * d0x + d0y * d0y, r1


def test_identities_on_far_pairs():
    """For dot > 0 the subtended angle atan2(cross, dot) is atan(cross/dot), and the half-log
    0.5 log(r0^2/r1^2) is atanh((r0^2 - r1^2)/(r0^2 + r1^2)); on pairs in the 5th-power tier
    the series reproduce both to 2.3e-9.  The half-log's reference is 0.5 log1p of the exactly
    formed difference over r1^2: the log of the ratio itself loses up to 1e-8 of its relative
    accuracy to cancellation on these pairs, even in FP64."""
    rng = np.random.default_rng(21)
    th = rng.uniform(0, 2 * np.pi, 300)
    p0 = np.stack([np.cos(th), np.sin(th)], 1)
    ang = rng.uniform(0, 2 * np.pi, 300)
    p1 = p0 + 0.01 * np.stack([np.cos(ang), np.sin(ang)], 1)
    t = rng.uniform(-3, 3, (400, 2))
    cr, dt, diff, den, r0, r1 = pair_quantities(p0, p1, t)
    tier = (np.abs(cr) < 0.05 * dt) & (np.abs(diff) < 0.05 * den)
    assert tier.mean() > 0.9
    us, vs = atan5(cr[tier] / dt[tier]), atanh5(diff[tier] / den[tier])
    ang_ref = np.arctan2(cr[tier], dt[tier])
    log_ref = 0.5 * np.log1p(diff[tier] / r1[tier])
    assert np.max(np.abs(us - ang_ref) / np.abs(ang_ref)) < 2.3e-9
    assert np.max(np.abs(vs - log_ref) / np.abs(log_ref)) < 2.3e-9


@pytest.mark.parametrize("seed", [3])
def test_bem_workload_pairs_all_take_the_5th_power_form(seed):
    """The BEM coupling configuration (unit-diameter circle of 2048 panels, particles uniform in
    0.55 < r < 3, drawn as bench.py draws them): on a sample of 20,000 particles every
    (panel, particle) pair has both ratios below 0.05 -- the largest is about L/d = 0.031, the
    panel length over the 0.05 gap to the body."""
    rng = np.random.default_rng(seed)
    npart = 200_000
    rad = np.sqrt(rng.uniform(0.55 ** 2, 3.0 ** 2, npart))
    th = rng.uniform(0.0, 2.0 * np.pi, npart)
    pts = np.stack([rad * np.cos(th), rad * np.sin(th)], 1)
    sub = pts[np.argsort(rad)[:20_000]]          # the particles nearest the body
    bd = og.circle_panels(2048)
    nodes = np.stack([bd.nx, bd.ny], 1).astype(np.float64)
    idx = bd.idx.reshape(-1, 2)
    p0, p1 = nodes[idx[:, 0]], nodes[idx[:, 1]]
    worst = 0.0
    for c in range(0, sub.shape[0], 2000):
        cr, dt, diff, den, _, _ = pair_quantities(p0, p1, sub[c:c + 2000])
        assert np.all(dt > 0.0)
        worst = max(worst, float(np.max(np.abs(cr) / dt)), float(np.max(np.abs(diff) / den)))
    assert worst < 0.05
