"""Several bodies in one BEM system (src/BEMHelper.h:43-260 over a list of boundary
collections): the reference assembles the matrix block by block, block (t, s) being
panels_on_panels_coeff of body s on body t with the self term only on diagonal blocks.  The
golden fixture tests/golden/bodies.npz holds that block assembly from the reference's own code
for a circle and an irregular polygon; these CPU tests pin og.join_surfaces and the claim that
the joined panel set has the same matrix."""
import numpy as np
import pytest

import omega2d_gb300 as og
from conftest import rel_err
from oracle import pyoracle as po


def _bodies(g):
    return [og.Surfaces(g["nx0"], g["ny0"], g["idx0"]), og.Surfaces(g["nx1"], g["ny1"], g["idx1"])]


def test_join_surfaces_offsets_and_indices():
    a = og.circle_panels(12)
    b = og.circle_panels(7, 0.4, center=(2.0, 0.0))
    b.vs = np.arange(7, dtype=np.float32)
    a.vs = -np.arange(12, dtype=np.float32)
    j, offs = og.join_surfaces([a, b])
    assert list(offs) == [0, 12, 19]
    assert j.npan == 19 and j.nnodes == 19
    np.testing.assert_array_equal(j.idx[:24], a.idx)
    np.testing.assert_array_equal(j.idx[24:], b.idx + 12)
    np.testing.assert_array_equal(j.nx[12:], b.nx)
    np.testing.assert_array_equal(j.vs, np.concatenate([a.vs, b.vs]))
    assert j.ss is None                                  # only carried when every body has it
    with pytest.raises(ValueError):
        og.join_surfaces([])
    # panel k of the joined set is panel k - offs[body] of its body
    for k in (0, 11, 12, 18):
        body, local = (a, k) if k < 12 else (b, k - 12)
        p0, p1 = j.idx[2 * k], j.idx[2 * k + 1]
        assert (j.nx[p0], j.ny[p1]) == (body.nx[body.idx[2 * local]], body.ny[body.idx[2 * local + 1]])


def test_reference_joined_matrix_equals_block_assembly(golden):
    """The reference's coefficients of the joined panel set are its block assembly, bit for bit."""
    if not po.Reference.available(po.V2):
        pytest.skip("the compiled reference is not available here")
    g = golden("bodies")
    j, offs = og.join_surfaces(_bodies(g))
    C = po.Reference(po.V2).panels_on_panels_coeff(j.nx, j.ny, j.idx)
    np.testing.assert_array_equal(C, g["A"])
    assert list(offs) == [0, 36, 60]


def test_restatement_joined_matrix_vs_block_golden(restatement, golden):
    g = golden("bodies")
    j, _ = og.join_surfaces(_bodies(g))
    A32 = restatement.panels_on_panels_coeff(2, j.nx, j.ny, j.idx)
    A64 = restatement.panels_on_panels_coeff(2, j.nx, j.ny, j.idx, fp64=True)
    assert rel_err(g["A"], A32) < 1e-5          # the same float algorithm
    assert rel_err(g["A"], A64) < 1e-4          # the reference's own float error
    # off-diagonal blocks: the restatement's pair block of body s on body t
    b = _bodies(g)
    R = restatement.panels_on_panels_coeff(2, b[0].nx, b[0].ny, b[0].idx, fp64=True, self_block=False,
                                           tnx=b[1].nx, tny=b[1].ny, tidx=b[1].idx)
    assert rel_err(g["A"][72:, :72], R) < 1e-4


def test_solve_bem_bodies_splits_strengths_by_body(monkeypatch):
    """Host logic of solve_bem_bodies: one solve over the joined set, then each body receives its
    own slice (the solve is replaced by one that writes the joined panel index)."""
    calls = []

    def fake_solve(vort, joined, fs=(0.0, 0.0), nunk=2, env=None, reuse_matrix=False, direct_lu=False):
        calls.append((joined.npan, nunk, reuse_matrix, direct_lu))
        joined.vs = np.arange(joined.npan, dtype=np.float32)
        if nunk == 2:
            joined.ss = -np.arange(joined.npan, dtype=np.float32)
        return 1e-14
    monkeypatch.setattr(og, "solve_bem", fake_solve)
    a, b, c = og.circle_panels(10), og.circle_panels(6, 0.3, center=(2.0, 0.0)), og.circle_panels(4, 0.2, (0, 3))
    vort = og.Points(np.zeros(0), np.zeros(0), np.zeros(0), np.zeros(0))
    assert og.solve_bem_bodies(vort, [a, b, c], nunk=2, reuse_matrix=True) == 1e-14
    assert calls == [(20, 2, True, False)]
    np.testing.assert_array_equal(a.vs, np.arange(10))
    np.testing.assert_array_equal(b.vs, np.arange(10, 16))
    np.testing.assert_array_equal(c.ss, -np.arange(16, 20))
    og.solve_bem_bodies(vort, [a, b], nunk=1, direct_lu=True)
    assert calls[-1] == (16, 1, False, True)
    np.testing.assert_array_equal(b.vs, np.arange(10, 16))


def _geom_center(nx, ny, idx):
    """Area and centroid of a closed body from the triangles (origin, node j, node j+1)
    (src/Surfaces.h:623-677), in FP64."""
    x0, y0 = nx[idx[0::2]].astype(np.float64), ny[idx[0::2]].astype(np.float64)
    x1, y1 = nx[idx[1::2]].astype(np.float64), ny[idx[1::2]].astype(np.float64)
    px, py = x1 - x0, y1 - y0
    a, b, c = np.hypot(x0, y0), np.hypot(px, py), np.hypot(x1, y1)
    hs = 0.5 * (a + b + c)
    ar = np.sqrt(np.maximum(hs * (hs - a) * (hs - b) * (hs - c), 0.0))
    ar = np.where(y0 * px - x0 * py < 0.0, -ar, ar)
    return ar.sum(), (ar * (x0 + x1) / 3.0).sum() / ar.sum(), (ar * (y0 + y1) / 3.0).sum() / ar.sum()


def test_restatement_rotating_bodies_vs_golden(restatement, golden):
    """The rotation rows and columns of two rotating bodies in one system (golden bodies_aug.npz,
    the reference's block assembly, src/BEMHelper.h:166-221 with src/Coefficients.h:429-572),
    restated: column s is body s's unit-rotation sheet (src/Surfaces.h:570-620) acting on each
    body's panels through that body's own collocation points (src/Influence.h:775-795: the
    target's represent_as_particles spaces them by the target's first panel), over 2 pi,
    projected on tangent and normal; row t is body t's panel lengths under its vortex unknowns;
    the corner is 2 * area on the diagonal, zero across bodies."""
    g = golden("bodies_aug")
    bodies = [(g[f"nx{k}"], g[f"ny{k}"], g[f"idx{k}"]) for k in range(2)]
    sizes = [b[2].size // 2 for b in bodies]
    start = [0, 2 * sizes[0] + 1]                            # reference order: panels, then rotation
    R = g["A"].astype(np.float64)
    for s, (snx, sny, sidx) in enumerate(bodies):
        vol, cx, cy = _geom_center(snx, sny, sidx)
        assert abs(vol - g[f"vol{s}"][0]) < 1e-6 * abs(vol)
        x0, y0, x1, y1 = snx[sidx[0::2]], sny[sidx[0::2]], snx[sidx[1::2]], sny[sidx[1::2]]
        L = np.hypot(x1 - x0, y1 - y0)
        ui, vi = -(0.5 * (y0 + y1) - cy), 0.5 * (x0 + x1) - cx
        tx, ty = (x1 - x0) / L, (y1 - y0) / L
        vs, ss = -(ui * tx + vi * ty), -(ui * ty - vi * tx)
        col = start[s] + 2 * sizes[s]
        for t, (tnx, tny, tidx) in enumerate(bodies):
            pu, pv = restatement.panels_affect_panels(snx, sny, sidx, vs, ss, tnx, tny, tidx)
            pu, pv = pu / (2 * np.pi), pv / (2 * np.pi)
            ax, ay = tnx[tidx[0::2]], tny[tidx[0::2]]
            bx, by = tnx[tidx[1::2]], tny[tidx[1::2]]
            Lt = np.hypot(bx - ax, by - ay)
            ttx, tty = (bx - ax) / Lt, (by - ay) / Lt
            want = np.stack([pu * ttx + pv * tty, pu * -tty + pv * ttx], 1).ravel()
            got = R[start[t]:start[t] + 2 * sizes[t], col]
            assert rel_err(got, want) < 1e-5, (s, t)
            # the rotation row of body t under body s's unknowns
            row = R[start[t] + 2 * sizes[t], start[s]:start[s] + 2 * sizes[s]]
            if s == t:
                np.testing.assert_allclose(row[0::2], L, rtol=1e-6)
                assert not row[1::2].any()
                assert R[col, col] == np.float32(2 * g[f"vol{s}"][0])
            else:
                assert not row.any() and R[start[t] + 2 * sizes[t], col] == 0.0
