"""The oracle's restatement of clear_inner_panp2 (src/Reflect.h:491-729: particles inside a
body's cutoff layer are cropped with the cut tables, or pushed onto the layer) against the
reference's own routine (golden tests/golden/clear.npz, and the live build where present).

The reference is compiled with -march=native, so its float arithmetic fuses multiply-adds; the
oracle is built with portable flags.  Bit-level differences matter at one place only: a fully
cropped particle (strength 0) is shifted exactly onto the layer, and the rounding of that
shift decides whether the next sweep cuts it again, possibly along another closest panel or
node normal (0.113 core radii per cut).  Such particles carry no circulation; their positions
are compared within half a core radius, everything else tightly."""
import numpy as np
import pytest

from oracle import pyoracle as po

SHAPES = ("circle", "star")


def _check_method0(g_x, g_y, g_s, x, y, s, r):
    cropped = g_s == 0.0
    d = np.hypot(g_x - x, g_y - y)
    assert np.all(d[~cropped] < 1e-5), np.max(d[~cropped])
    assert np.all(d[cropped] <= 0.5 * r[cropped])
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


# ------------------------------------------------------------------ the engine's per-point logic
# omega2d_gb300/csrc/clear_inner.cuh is the code the CUDA kernel runs per point; it also compiles
# for the host.  This harness runs it over an array the way clear_points_kernel does.
HARNESS = r"""
#include "clear_inner.cuh"
#include <vector>
extern "C" int host_clear(int method, float cut, float ips, int nnodes, const float* nx, const float* ny, int npan,
                          const unsigned* idx, int n, float* x, float* y, float* s, const float* r, double* lost,
                          long long* ncrop) {
  std::vector<float> pn(2 * (size_t)npan), nn(2 * (size_t)nnodes), ct(3 * obs::clear::CUT_N);
  if (obs::clear::normals(nnodes, nx, ny, npan, idx, pn.data(), pn.data() + npan, nn.data(), nn.data() + nnodes))
    return -1;
  obs::clear::cut_table(ct.data(), ct.data() + obs::clear::CUT_N, ct.data() + 2 * obs::clear::CUT_N);
  const obs::clear::Geo g{nx, ny, idx, npan, pn.data(), pn.data() + npan, nn.data(), nn.data() + nnodes,
                          ct.data(), ct.data() + obs::clear::CUT_N, ct.data() + 2 * obs::clear::CUT_N};
  double tot = 0.0;
  long long crops = 0;
  int fail = 0;
  for (int i = 0; i < n; ++i) {
    float si = s ? s[i] : 0.0f;
    double l = 0.0;
    const int c = obs::clear::clear_point(g, method, cut, ips, r ? r[i] : ips, x[i], y[i], si, l, 64);
    if (s) s[i] = si;
    tot += l;
    if (c < 0) ++fail; else crops += c;
  }
  *lost = tot;
  *ncrop = crops;
  return fail;
}
"""


@pytest.fixture(scope="module")
def engine_logic(tmp_path_factory):
    import ctypes
    import os
    import shutil
    import subprocess
    if shutil.which("g++") is None:
        pytest.skip("needs g++")
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    d = tmp_path_factory.mktemp("clear")
    src = d / "harness.cpp"
    src.write_text(HARNESS)
    lib = d / "libharness.so"
    # built like the CUDA file and the oracle: no fused multiply-adds
    subprocess.run(["g++", "-O2", "-std=c++17", "-shared", "-fPIC", "-ffp-contract=off",
                    "-I", os.path.join(root, "omega2d_gb300", "csrc"),
                    str(src), "-o", str(lib)], check=True)
    L = ctypes.CDLL(str(lib))

    def run(method, cut, ips, nx, ny, idx, x, y, s=None, r=None):
        f32 = lambda a: None if a is None else np.array(a, np.float32)
        nx, ny, x, y, s, r = (f32(a) for a in (nx, ny, x, y, s, r))
        idx = np.ascontiguousarray(idx, np.uint32)
        lost, nc = ctypes.c_double(), ctypes.c_longlong()
        fail = L.host_clear(ctypes.c_int(method), ctypes.c_float(cut), ctypes.c_float(ips), ctypes.c_int(nx.size),
                            po._p(nx), po._p(ny), ctypes.c_int(idx.size // 2), po._p(idx), ctypes.c_int(x.size),
                            po._p(x), po._p(y), po._p(s), po._p(r), ctypes.byref(lost), ctypes.byref(nc))
        assert fail == 0
        return x, y, s, lost.value, nc.value
    return run


@pytest.mark.parametrize("shape", SHAPES)
def test_engine_point_logic_matches_golden_and_oracle(engine_logic, restatement, golden, shape):
    g = golden("clear")
    cut, ips = g["cut"][0], g["ips"][0]
    nx, ny, idx = g[shape + "_nx"], g[shape + "_ny"], g[shape + "_idx"]
    x, y, s, r = g[shape + "_x"], g[shape + "_y"], g[shape + "_s"], g[shape + "_r"]
    ex, ey, es, elost, enc = engine_logic(0, cut, ips, nx, ny, idx, x, y, s, r)
    _check_method0(g[shape + "_m0_x"], g[shape + "_m0_y"], g[shape + "_m0_s"], ex, ey, es, r)
    glost = g[shape + "_m0_lost"][0]
    assert abs(elost - glost) < 1e-5 * max(1.0, abs(glost))
    # the oracle sweeps all points per pass, the engine repeats each point: the same per-point
    # result, bit for bit (both built without fused multiply-adds)
    ox, oy, os_, olost, onc = restatement.clear_inner(0, cut, ips, nx, ny, idx, x, y, s, r)
    np.testing.assert_array_equal(ex, ox)
    np.testing.assert_array_equal(ey, oy)
    np.testing.assert_array_equal(es, os_)
    assert enc == onc
    px, py, ps, plost, pnc = engine_logic(1, cut, ips, nx, ny, idx, x, y, s, r)
    assert plost == 0.0 and pnc > 0
    np.testing.assert_array_equal(ps, s)
    assert np.max(np.hypot(px - g[shape + "_m1_x"], py - g[shape + "_m1_y"])) < 1e-5
    fx, fy, _, _, _ = engine_logic(1, 0.0, ips, nx, ny, idx, x, y)
    assert np.max(np.hypot(fx - g[shape + "_fld_x"], fy - g[shape + "_fld_y"])) < 1e-5


def test_engine_point_logic_guards(engine_logic):
    """A point on a panel and one on a node are pushed out along the panel / node normal; one far
    outside is untouched; the centre of the diamond ties all four panels, whose normals cancel,
    and stays put (as in the reference: its normal is NaN, so the test never fires); a NaN point
    ends without a closest panel."""
    nx = np.array([0.5, 0.0, -0.5, 0.0], np.float32)
    ny = np.array([0.0, -0.5, 0.0, 0.5], np.float32)                  # clockwise diamond
    idx = np.array([0, 1, 1, 2, 2, 3, 3, 0], np.uint32)
    x = np.array([0.25, 0.5, 10.0, 0.0, np.nan], np.float32)
    y = np.array([-0.25, 0.0, 0.0, 0.0, 0.0], np.float32)
    px, py, _, _, nc = engine_logic(1, 0.2, 0.02, nx, ny, idx, x, y)
    # the reference's own result for the first four (src/Reflect.h:491-729, its float build)
    np.testing.assert_allclose(px[:4], [0.25282842, 0.504, 10.0, 0.0], rtol=0, atol=1e-7)
    np.testing.assert_allclose(py[:4], [-0.25282842, 0.0, 0.0, 0.0], rtol=0, atol=1e-7)
    assert np.isnan(px[4]) and nc == 2
