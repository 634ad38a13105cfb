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
