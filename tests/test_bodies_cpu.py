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
