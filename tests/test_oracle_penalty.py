"""CPU: the oracle's surface penalty and inflate_sphere against known answers.

The reference ships no fixture for apply_boundary_conditions
(examples/vector3D.jl:175-264); on flat faces its b is the face mass matrix
(h^2/36) [[4,2,1,2],[2,4,2,1],[1,2,4,2],[2,1,2,4]] per displacement
component, which 2x2 Gauss integrates exactly.
"""
import math

import numpy as np
import pytest


def test_flat_face_mass_matrix(oracle):
    ne = 3
    NL, IEN, ID, IT, IB = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, ne, 3)
    b = oracle.csc_to_dense(*oracle.apply_boundary_conditions_loops(ne, NL, IEN, IT, IB, 3, "Q1", ID))
    h2 = (1.0 / ne) ** 2
    ref = h2 / 36 * np.array([[4, 2, 1, 2], [2, 4, 2, 1], [1, 2, 4, 2], [2, 1, 2, 4]], float)
    # the corner node of the first bottom face belongs to that face alone, so
    # every pair (corner, a) of it carries exactly the face's mass entry
    nodes = IB[0] - 1
    for c in range(3):
        for a in range(4):
            got = b[ID[nodes[0], c] - 1, ID[nodes[a], c] - 1]
            assert got == pytest.approx(ref[0, a], rel=1e-14)
    assert b[ID[nodes[0], 0] - 1, ID[nodes[0], 1] - 1] == 0.0     # no coupling between components
    # partition of unity: the penalty's blocks sum to the face areas per component
    total = sum(b[ID[i, 0] - 1, ID[j, 0] - 1] for i in range(NL.shape[1]) for j in range(NL.shape[1])
                if ID[i, 0] - 1 < b.shape[0] and ID[j, 0] - 1 < b.shape[1])
    assert total == pytest.approx(2.0, rel=1e-13)   # bottom + top, unit area each
    assert np.allclose(b, b.T, atol=0)


def test_curved_faces_area(oracle):
    """On the inflated cylinder the top/bottom faces still lie in z = 0 / 1;
    their penalty sums to the discs' polygonal area (< pi/4 each)."""
    ne = 6
    NL, IEN, ID, IT, IB = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, ne, 3)
    cyl = oracle.inflate_sphere(NL, 0, 1, 0, 1)
    b = oracle.csc_to_scipy(*oracle.apply_boundary_conditions_loops(ne, cyl, IEN, IT, IB, 3, "Q1", ID))
    comp0 = ID[:, 0] - 1
    comp0 = comp0[comp0 < b.shape[0]]
    area = b[comp0][:, comp0].sum()
    assert 2 * 0.70 < area < 2 * math.pi / 4


def test_inflate_sphere_known_points(oracle):
    NL = np.array([[0.5, 1.0, 1.0, 0.75], [0.5, 1.0, 0.5, 0.5], [0.0, 0.0, 1.0, 0.3]])
    out = oracle.inflate_sphere(NL, 0, 1, 0, 1)
    assert out[0, 0] == 0.0 and out[1, 0] == 0.0                   # centre
    assert math.hypot(out[0, 1], out[1, 1]) == pytest.approx(0.5)   # corner onto the r = 0.5 circle
    assert out[0, 1] == pytest.approx(0.5 / math.sqrt(2))
    assert out[0, 2] == pytest.approx(0.5) and out[1, 2] == pytest.approx(0.0)
    assert out[0, 3] == pytest.approx(0.25) and np.array_equal(out[2], NL[2])
    assert NL[0, 1] == 1.0                                          # input untouched


def test_penalty_rejects_2d_and_empty_top(oracle):
    NL, IEN, ID, IT, IB = oracle.meshgrid_loops(0, 1, 0, 1, 0, 0, 3, 2)
    with pytest.raises(ValueError):
        oracle.apply_boundary_conditions_loops(3, NL, IEN, IT, IB, 2, "Q1", ID, nDof=2)
    NL, IEN, ID, IT, IB = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, 1, 3)   # ne = 1 leaves IEN_top empty
    with pytest.raises(IndexError):
        oracle.apply_boundary_conditions_loops(1, NL, IEN, IT, IB, 3, "Q1", ID)


def test_meshgen_squeeze_helpers_match_oracle(oracle):
    import __graft_entry__ as GE
    mg = GE.load_package().meshgen
    NL, IEN, ID, IT, IB, cyl, faces = mg.squeeze_problem(5)
    assert np.array_equal(cyl, oracle.inflate_sphere(NL, 0, 1, 0, 1))
    fd, fv = mg.squeeze_increments(NL, [0.001, 0.2])
    for k, d in enumerate((0.001, 0.2)):
        q, rcol = oracle.set_boundary_cond(NL, 5, 3, d, 3)
        assert np.array_equal(np.sort(rcol), fd)
        assert np.array_equal(q[fd - 1], fv[k])
