"""CPU tests of the Python mirror of the reference containers (no GPU calls)."""
import numpy as np

import omega2d_gb300 as og


def test_points_own_their_arrays():
    x = np.linspace(0, 1, 5).astype(np.float32)
    p = og.Points(x, x, np.full(5, 0.1, np.float32), np.ones(5, np.float32))
    p.x[:] = 7.0
    assert x[0] == 0.0          # the caller's array is untouched (src/Points.h copies its input)
    assert p.is_inert() is False and og.Points(x, x).is_inert() is True


def test_points_zero_and_finalize():
    p = og.Points(np.zeros(3), np.zeros(3), np.ones(3), np.ones(3))
    p.u[:] = 2 * np.pi
    p.v[:] = -2 * np.pi
    p.finalize_vels((1.0, 0.5))
    np.testing.assert_allclose(p.u, 2.0, rtol=1e-7)
    np.testing.assert_allclose(p.v, -0.5, rtol=1e-7)
    p.zero_vels()
    assert not p.u.any() and not p.v.any()


def test_circle_panels_are_clockwise_with_fluid_outside():
    s = og.circle_panels(64, 1.0)
    assert s.npan == 64 and s.nnodes == 64
    i0, i1 = s.idx[0::2], s.idx[1::2]
    tx, ty = s.nx[i1] - s.nx[i0], s.ny[i1] - s.ny[i0]
    mx, my = 0.5 * (s.nx[i1] + s.nx[i0]), 0.5 * (s.ny[i1] + s.ny[i0])
    # normal to the left of node0 -> node1 (src/Surfaces.h:713-716) points away from the centre
    nx, ny = -ty, tx
    assert np.all(nx * mx + ny * my > 0)
    np.testing.assert_allclose(np.hypot(mx, my), 0.5 * np.cos(np.pi / 64), rtol=1e-6)
