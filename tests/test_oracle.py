"""CPU: the oracle pinned against the reference's own known answers and
against analytic results, and the C restatement against the NumPy one.

The reference's tests (test/runtests.jl) pin only basis_function and
gaussian_quadrature; they are restated here exactly (``==``).  Assembly and
solve are pinned by analytic known answers (the reference ships none).
"""
import math
import os

import numpy as np
import pytest

GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


# ---- test/runtests.jl:15-35, verbatim known answers -----------------------

def test_reference_kat_basis(oracle):
    bf = oracle.basis_function
    assert list(bf(-1)[0]) == [1.0, 0.0]
    assert list(bf(1)[0]) == [0.0, 1.0]
    corners2 = [(-1, -1), (1, -1), (1, 1), (-1, 1)]
    for i, c in enumerate(corners2):
        assert list(bf(*c)[0]) == list(np.eye(4)[i])
    corners3 = [(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
                (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]
    for i, c in enumerate(corners3):
        assert list(bf(*c)[0]) == list(np.eye(8)[i])


def test_reference_kat_quadrature(oracle):
    xi, w = oracle.gaussian_quadrature(-1, 1, 2)
    assert list(xi) == [-1 / math.sqrt(3), 1 / math.sqrt(3)] and list(w) == [1.0, 1.0]
    xi, w = oracle.gaussian_quadrature(-1, 1, 3)
    assert list(xi) == [-math.sqrt(3 / 5), 0.0, math.sqrt(3 / 5)]
    assert list(w) == [5 / 9, 8 / 9, 5 / 9]


def test_partition_of_unity_and_gradients(oracle):
    rng = np.random.default_rng(0)
    for _ in range(20):
        x, y, z = rng.uniform(-1, 1, 3)
        for args, fc in (((x, y, z), "Q1"), ((x, y), "Q1"), ((x, y), "Q2")):
            N, dN = oracle.basis_function(*args, FunctionClass=fc)
            assert abs(N.sum() - 1) < 1e-14
            assert np.abs(dN.sum(axis=0)).max() < 1e-14
            h = 1e-6
            for k in range(len(args)):
                a1 = list(args); a1[k] += h
                a0 = list(args); a0[k] -= h
                fd = (oracle.basis_function(*a1, FunctionClass=fc)[0]
                      - oracle.basis_function(*a0, FunctionClass=fc)[0]) / (2 * h)
                assert np.abs(fd - dN[:, k]).max() < 1e-8


# ---- analytic element matrices ----------------------------------------------

def _single(oracle, sfem_meshgen, ndim, nDof, Y=1.0, nu=0.3, plane="stress"):
    NL, IEN, ID, _, _ = sfem_meshgen.meshgrid(0, 1, 0, 1, 0, 1, 1, ndim)
    K = oracle.assemble_system(1, NL, IEN, ndim, "Q1", nDof, ID, Y, nu, plane)
    A = oracle.csc_to_dense(*K)
    if nDof == 1:
        p = IEN[0] - 1
    else:
        p = (nDof * (IEN[0] - 1)[:, None] + np.arange(nDof)).ravel()
    return A[np.ix_(p, p)]                                    # element-local order


@pytest.fixture(scope="module")
def meshgen():
    import __graft_entry__ as GE
    return GE.load_package().meshgen


def test_unit_square_laplace(oracle, meshgen):
    Ke = _single(oracle, meshgen, 2, 1)
    ref = np.array([[4, -1, -2, -1], [-1, 4, -1, -2], [-2, -1, 4, -1], [-1, -2, -1, 4]]) / 6
    assert np.abs(Ke - ref).max() < 1e-15


def test_unit_cube_laplace(oracle, meshgen):
    """Trilinear unit cube: 1/3 on the diagonal, 0 along edges, -1/12 across
    face diagonals and across the body diagonal."""
    Ke = _single(oracle, meshgen, 3, 1)
    corners = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0],
                        [0, 0, 1], [1, 0, 1], [1, 1, 1], [0, 1, 1]])
    d = np.abs(corners[:, None, :] - corners[None, :, :]).sum(axis=2)
    ref = np.select([d == 0, d == 1, d >= 2], [1 / 3, 0.0, -1 / 12])
    assert np.abs(Ke - ref).max() < 1e-15


@pytest.mark.parametrize("nu", [0.0, 0.3, 0.45])
def test_unit_square_plane_stress_closed_form(oracle, meshgen, nu):
    """Bilinear unit square, plane stress, unit thickness: the classical
    closed form E/(1-nu^2) k-matrix (nodes counter-clockwise from (0,0))."""
    E = 2.5
    Ke = _single(oracle, meshgen, 2, 2, E, nu, "stress")
    k = [1 / 2 - nu / 6, 1 / 8 + nu / 8, -1 / 4 - nu / 12, -1 / 8 + 3 * nu / 8,
         -1 / 4 + nu / 12, -1 / 8 - nu / 8, nu / 6, 1 / 8 - 3 * nu / 8]
    idx = [[0, 1, 2, 3, 4, 5, 6, 7], [1, 0, 7, 6, 5, 4, 3, 2], [2, 7, 0, 5, 6, 3, 4, 1],
           [3, 6, 5, 0, 7, 2, 1, 4], [4, 5, 6, 7, 0, 1, 2, 3], [5, 4, 3, 2, 1, 0, 7, 6],
           [6, 3, 4, 1, 2, 7, 0, 5], [7, 2, 1, 4, 3, 6, 5, 0]]
    ref = E / (1 - nu ** 2) * np.array(k)[np.array(idx)]
    assert np.abs(Ke - ref).max() < 1e-14 * np.abs(ref).max()


@pytest.mark.parametrize("ndim,plane", [(3, "stress"), (2, "stress"), (2, "strain")])
def test_rigid_body_modes(oracle, meshgen, ndim, plane):
    ne = 3
    rng = np.random.default_rng(4)
    NL, IEN, ID, _, _ = meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, ndim)
    NL = meshgen.jitter_interior(NL, ne, 0.25, rng)
    Y = np.exp(rng.normal(0, 1, ne ** ndim))
    K = oracle.csc_to_dense(*oracle.assemble_system(ne, NL, IEN, ndim, "Q1", ndim, ID, Y, 0.3, plane))
    modes = [np.tile(e, NL.shape[1]) for e in np.eye(ndim)]
    pairs = [(0, 1)] if ndim == 2 else [(0, 1), (1, 2), (0, 2)]
    for i, j in pairs:
        r = np.zeros((NL.shape[1], ndim))
        r[:, i] = -NL[j]
        r[:, j] = NL[i]
        modes.append(r.ravel())
    for r in modes:
        assert np.abs(K @ r).max() < 1e-13 * np.abs(K).max()
    assert np.abs(K - K.T).max() < 1e-14 * np.abs(K).max()
    w = np.linalg.eigvalsh((K + K.T) / 2)
    assert w.min() > -1e-12 * w.max()                          # positive semi-definite
    assert np.sum(w < 1e-10 * w.max()) == len(modes)           # null space = rigid modes


def test_plane_strain_is_restricted_3d(oracle):
    D2 = oracle.constitutive_matrix(2, 3.0, 0.3, "strain")
    D3 = oracle.constitutive_matrix(3, 3.0, 0.3)
    sel = [0, 1, 5]
    assert np.abs(D2 - D3[np.ix_(sel, sel)]).max() < 1e-15


def test_julia_sparse_semantics(oracle):
    # duplicates folded left in input order, zeros kept, rows sorted, size = max index
    I = [3, 1, 3, 2, 1]
    J = [1, 1, 1, 2, 1]
    V = [1.0, 0.0, 2.0, 0.0, 5.0]
    colptr, rowval, nzval, m, n = oracle.julia_sparse(I, J, V)
    assert (m, n) == (3, 2)
    assert list(colptr) == [1, 3, 4]
    assert list(rowval) == [1, 3, 2]
    assert list(nzval) == [5.0, 3.0, 0.0]


def test_patch_test_oracle(oracle, meshgen):
    ne = 4
    rng = np.random.default_rng(8)
    NL, IEN, ID, _, _ = meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, 3)
    NL = meshgen.jitter_interior(NL, ne, 0.25, rng)
    A = rng.normal(size=(3, 3)) * 0.01
    ulin = (A @ NL).T.ravel()
    bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0))
    dofs = (3 * bnd[:, None] + np.arange(1, 4)).ravel()
    K = oracle.assemble_system(ne, NL, IEN, 3, "Q1", 3, ID, 1.0, 0.3)
    u = oracle.solve_eliminated(K, dofs, ulin[dofs - 1], method="inv")
    assert np.abs(u - ulin).max() < 1e-12


# ---- C restatement vs NumPy restatement -----------------------------------

@pytest.mark.parametrize("ndim,nDof,plane", [(2, 1, "stress"), (3, 1, "stress"), (2, 2, "stress"),
                                             (2, 2, "strain"), (3, 3, "stress")])
def test_c_oracle_matches_numpy(oracle, coracle, meshgen, ndim, nDof, plane):
    ne = 4
    rng = np.random.default_rng(ndim * 10 + nDof)
    NL, IEN, ID, _, _ = meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, ndim)
    NL = meshgen.jitter_interior(NL, ne, 0.2, rng)
    Y = np.exp(rng.normal(0, 0.5, ne ** ndim))
    a = oracle.assemble_system(ne, NL, IEN, ndim, "Q1", nDof, ID, Y, 0.3, plane)
    b = coracle.assemble(ne, NL, IEN, ndim, "Q1", nDof, ID, Y, 0.3, plane, nthreads=2).arrays()
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1]) and a[3:] == b[3:]
    assert np.abs(a[2] - b[2]).max() <= 1e-14 * np.abs(a[2]).max()


def test_c_oracle_pcg_matches_direct(oracle, coracle, meshgen):
    p = meshgen.hex_problem(5, 3, jitter=0.2, e_sigma=0.5, top="modes")
    K = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    uref = oracle.solve_eliminated(K.arrays(), p.fixed_dofs, p.fixed_vals, method="inv")
    assert st["status"] == 0
    assert np.linalg.norm(u - uref) / np.linalg.norm(uref) < 1e-10


# ---- committed fixtures still reproduce -------------------------------------

def test_golden_fixtures_reproduce(oracle):
    from tests.golden import make_golden as MG
    for name in MG.SMALL:
        d = np.load(os.path.join(GOLDEN_DIR, f"{name}.npz"))
        c = MG.small_case(name)
        Y = c["Young"] if c["Young"].size > 1 else float(c["Young"][0])
        colptr, rowval, nzval, m, n = oracle.assemble_system_loops(
            c["ne"], c["NodeList"], c["IEN"], c["ndim"], c["fclass"], c["nDof"], c["ID"], Y,
            float(c["nu"][0]), c["plane"])
        assert np.array_equal(colptr, d["colptr"]) and np.array_equal(rowval, d["rowval"])
        assert np.abs(nzval - d["nzval"]).max() <= 1e-15 * max(1.0, np.abs(nzval).max())


@pytest.mark.skipif(not os.path.exists(os.path.join(GOLDEN_DIR, "cube20_dense_inv.npz")),
                    reason="cube20 fixture not generated")
def test_cube20_fixture_matches_c_oracle(coracle, meshgen):
    """The committed dense-inverse displacement of the 20^3 cube agrees with
    the C oracle's PCG, and the checksums of K match."""
    g = np.load(os.path.join(GOLDEN_DIR, "cube20_dense_inv.npz"))
    p = meshgen.parity_cube20()
    K = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, 1.0, 0.3)
    colptr, rowval, nzval, m, n = K.arrays()
    assert n == int(g["n"]) and len(nzval) == int(g["nnz"])
    assert int(rowval.sum()) == int(g["rowsum"]) and int(colptr.sum()) == int(g["colptr_sum"])
    assert abs(np.abs(nzval).sum() - float(g["nzabs"])) < 1e-12 * float(g["nzabs"])
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    assert np.linalg.norm(u - g["u"]) / np.linalg.norm(g["u"]) < 1e-10
