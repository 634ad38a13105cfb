"""The oracle's restatement of clear_inner_panp2 (src/Reflect.h:491-729: particles inside a
body's cutoff layer are cropped with the cut tables, or pushed onto the layer) against the
reference's own routine (golden tests/golden/clear.npz, and the live build where present).

The reference is compiled with -march=native, so its float arithmetic fuses multiply-adds; the
oracle is built with portable flags.  Bit-level differences matter at one place only: a fully
cropped particle (strength 0) is shifted exactly onto the layer, and the rounding of that
shift decides whether the next sweep cuts it once more (a further shift of at most 0.12 core
radii, strength still 0).  Everything else is compared tightly."""
import numpy as np
import pytest

from oracle import pyoracle as po

SHAPES = ("circle", "star")


def _check_method0(g_x, g_y, g_s, x, y, s, r):
    cropped = g_s == 0.0
    d = np.hypot(g_x - x, g_y - y)
    assert np.all(d[~cropped] < 1e-5), np.max(d[~cropped])
    assert np.all(d[cropped] <= 0.12 * r[cropped] + 1e-6)
    assert np.all(s[cropped] == 0.0)
    np.testing.assert_allclose(s, g_s, rtol=1e-5, atol=1e-6)


@pytest.mark.parametrize("shape", SHAPES)
@pytest.mark.parametrize("fp64", [False, True])
def test_clear_inner_matches_reference_golden(restatement, golden, shape, fp64):
    g = golden("clear")
    cut, ips = g["cut"][0], g["ips"][0]
    nx, ny, idx = g[shape + "_nx"], g[shape + "_ny"], g[shape + "_idx"]
    x, y, s, r = g[shape + "_x"], g[shape + "_y"], g[shape + "_s"], g[shape + "_r"]
    # method 0: crop with the cut tables
    ox, oy, os_, lost, n0 = restatement.clear_inner(0, cut, ips, nx, ny, idx, x, y, s, r, fp64=fp64)
    _check_method0(g[shape + "_m0_x"], g[shape + "_m0_y"], g[shape + "_m0_s"], ox, oy, os_, r)
    glost = g[shape + "_m0_lost"][0]
    assert abs(lost - glost) < 1e-5 * max(1.0, abs(glost))
    assert n0 > 0
    # the circulation is conserved: what the particles lost is what the routine reports
    assert abs((s.astype(np.float64).sum() - os_.astype(np.float64).sum()) - lost) < 1e-4
    # method 1: push onto the layer, strengths untouched
    px, py, ps, lost1, n1 = restatement.clear_inner(1, cut, ips, nx, ny, idx, x, y, s, r, fp64=fp64)
    assert lost1 == 0.0 and n1 > 0
    np.testing.assert_array_equal(ps, s.astype(ps.dtype))
    assert np.max(np.hypot(px - g[shape + "_m1_x"], py - g[shape + "_m1_y"])) < 1e-5
    # field points (no radius): method 1
    fx, fy, _, _, _ = restatement.clear_inner(1, 0.0, ips, nx, ny, idx, x, y, None, None, fp64=fp64)
    assert np.max(np.hypot(fx - g[shape + "_fld_x"], fy - g[shape + "_fld_y"])) < 1e-5


def test_clear_inner_refuses_cropping_field_points(restatement):
    """Method 0 on field points never ends in the reference (nothing marks them done)."""
    nx, ny = np.array([0.5, -0.5, -0.5], np.float32), np.array([0.0, 0.5, -0.5], np.float32)
    idx = np.array([0, 1, 1, 2, 2, 0], np.uint32)
    _, _, _, lost, _ = restatement.clear_inner(0, 0.2, 0.02, nx, ny, idx, [0.0], [0.0], None, None)
    assert np.isnan(lost)


def test_clear_inner_matches_live_reference(restatement):
    if not po.Reference.available(po.V2):
        pytest.skip("the compiled reference is not available here")
    rng = np.random.default_rng(9)
    k = 14                                             # an irregular, non-convex polygon
    th = -2.0 * np.pi * np.sort(rng.uniform(0, 1, k))
    rad = rng.uniform(0.25, 0.55, k)
    nx, ny = (rad * np.cos(th)).astype(np.float32), (rad * np.sin(th)).astype(np.float32)
    idx = np.stack([np.arange(k), (np.arange(k) + 1) % k], 1).ravel().astype(np.uint32)
    n = 200
    a, rr = rng.uniform(0, 2 * np.pi, n), rng.uniform(0.1, 0.7, n)
    x, y = (rr * np.cos(a)).astype(np.float32), (rr * np.sin(a)).astype(np.float32)
    s = rng.normal(0, 1, n).astype(np.float32)
    r = np.full(n, 0.02, np.float32)
    ref = po.Reference(po.V2)
    cut, ips = np.float32(0.2), np.float32(0.02)
    gx, gy, gs, glost = ref.clear_inner(1, cut, ips, nx, ny, idx, x, y, s, r)
    ox, oy, _, _, _ = restatement.clear_inner(1, cut, ips, nx, ny, idx, x, y, s, r)
    assert np.max(np.hypot(ox - gx, oy - gy)) < 1e-5
    gx, gy, gs, glost = ref.clear_inner(0, cut, ips, nx, ny, idx, x, y, s, r)
    ox, oy, os_, lost, _ = restatement.clear_inner(0, cut, ips, nx, ny, idx, x, y, s, r)
    _check_method0(gx, gy, gs, ox, oy, os_, r)
