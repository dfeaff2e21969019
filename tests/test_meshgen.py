"""CPU: the seeded workload generators (input layout of examples/vector3D.jl:10-130)."""
import numpy as np
import pytest


@pytest.mark.parametrize("ndim", [2, 3])
@pytest.mark.parametrize("ne", [1, 2, 5])
def test_meshgrid_matches_loop_restatement(sfem, oracle, ndim, ne):
    a = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, ne, ndim)
    b = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, ndim)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_workloads_are_seeded_and_valid(sfem, oracle):
    for make in (lambda: sfem.meshgen.jittered_cube(ne=8), lambda: sfem.meshgen.contrast_cube(ne=8)):
        p, q = make(), make()
        assert np.array_equal(p.NodeList, q.NodeList) and np.array_equal(p.Young, q.Young)
        assert np.array_equal(p.fixed_vals, q.fixed_vals)
        X = p.NodeList
        # boundary nodes stay exactly on the faces; all Gauss-point Jacobians positive
        on = np.any((X == 0) | (X == 1), axis=0)
        assert on.sum() == (p.ne + 1) ** 3 - (p.ne - 1) ** 3
        pts, _ = oracle.gauss_tables(3)
        for g in range(8):
            _, dN = oracle.basis_function(*pts[g])
            J = np.transpose(X[:, p.IEN - 1], (1, 0, 2)) @ dN
            assert np.linalg.det(J).min() > 0
        assert np.unique(p.fixed_dofs).size == p.fixed_dofs.size


def test_parity_cube20_sizes(sfem):
    p = sfem.meshgen.parity_cube20()
    assert p.n_nodes == 9261 and p.n_dof == 27783
    # bottom face: 441 nodes x 3 DOFs; top face: 441 z-DOFs
    assert p.fixed_dofs.size == 441 * 3 + 441
    assert p.n_dof - p.fixed_dofs.size == 26019


def test_batch_and_stream_generators(sfem):
    sizes = sfem.meshgen.quad_batch_sizes()
    assert sizes.size == 1024 and sizes.min() >= 16 and sizes.max() <= 256
    batch = sfem.meshgen.quad_batch(count=4)
    assert all(p.plane == "strain" and p.ndim == 2 for p in batch)
    stream = list(sfem.meshgen.serving_stream(20))
    t = [a for a, _ in stream]
    assert all(b > a for a, b in zip(t, t[1:]))
    assert {p.ndim for _, p in stream} <= {2, 3}
