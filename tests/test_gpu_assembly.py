"""GPU assembly parity: libsmearfem_gpu.so vs the CPU oracle (src/fem.jl:135-256).

Bar: the CSC pattern (colptr, rowval, size) is bit-exact to ``sparse(E,J,V)``
of the oracle; values agree within 1e-12 row-scaled
(|K_ij - K_ij^ref| <= 1e-12 max_k |K_ik^ref|), the tolerance that absorbs
cancellation to ~1e-17 in structured meshes.
"""
import glob
import os

import numpy as np
import pytest

from conftest import rowscaled_err

pytestmark = pytest.mark.gpu

TOL_K = 1e-12
GOLDEN_DIR = os.path.join(os.path.dirname(__file__), "golden")


def _assemble(sfem, ctx, ne, NL, IEN, ndim, fc, nDof, ID, Y, nu, plane="stress"):
    K = sfem.assemble_system(ne, NL, IEN, ndim, fc, nDof, ID, Y, nu, plane=plane, ctx=ctx,
                             as_handle=True)
    try:
        return K.n, K.to_csc_arrays()
    finally:
        K.close()


def _check(oracle, ref, got):
    n, (colptr, rowval, nzval) = got
    rc, rr, rv, m, nr = ref
    assert n == nr
    assert np.array_equal(colptr, rc), "colptr differs"
    assert np.array_equal(rowval, rr), "rowval differs"
    assert rowscaled_err(ref, nzval, rowval) <= TOL_K


@pytest.mark.parametrize("path", sorted(glob.glob(os.path.join(GOLDEN_DIR, "*_*.npz"))),
                         ids=lambda p: os.path.basename(p)[:-4])
def test_golden_fixtures(sfem, ctx, path):
    d = np.load(path)
    if "colptr" not in d:
        pytest.skip("not an assembly fixture")
    ndim, ne, nDof = (int(v) for v in d["meta"])
    Y = d["Young"] if d["Young"].size > 1 else float(d["Young"][0])
    got = _assemble(sfem, ctx, ne, d["NodeList"], d["IEN"], ndim, str(d["fclass"]), nDof, d["ID"],
                    Y, float(d["nu"][0]), str(d["plane"]))
    ref = (d["colptr"], d["rowval"], d["nzval"], int(d["m"]), int(d["n"]))
    _check(None, ref, got)


CASES = [
    # ndim, ne, nDof, plane, jitter, per-element E, per-element nu
    (2, 1, 1, "stress", 0.0, False, False),
    (2, 5, 1, "stress", 0.2, False, False),
    (3, 4, 1, "stress", 0.2, False, False),
    (2, 7, 2, "stress", 0.2, True, False),
    (2, 6, 2, "strain", 0.15, True, True),
    (3, 1, 3, "stress", 0.0, False, False),
    (3, 5, 3, "stress", 0.2, True, True),
    (3, 6, 3, "stress", 0.2, True, False),
]


@pytest.mark.parametrize("case", CASES, ids=lambda c: f"{c[0]}d_ne{c[1]}_dof{c[2]}_{c[3]}")
def test_assembly_vs_oracle(sfem, ctx, oracle, case):
    ndim, ne, nDof, plane, jit, pere, pernu = case
    rng = np.random.default_rng(ne * 100 + ndim * 10 + nDof)
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, ndim)
    if jit:
        NL = sfem.meshgen.jitter_interior(NL, ne, jit, rng)
    nEl = ne ** ndim
    Y = np.exp(rng.normal(0, 1.0, nEl)) if pere else 1.0
    nu = rng.uniform(0.25, 0.45, nEl) if pernu else 0.3
    ref = oracle.assemble_system(ne, NL, IEN, ndim, "Q1", nDof, ID, Y, nu, plane)
    got = _assemble(sfem, ctx, ne, NL, IEN, ndim, "Q1", nDof, ID, Y, nu, plane)
    _check(oracle, ref, got)


def test_cube20_vs_c_oracle(sfem, ctx, coracle):
    """The 20^3 unit cube (27,783 DOFs, 2,042,829 nonzeros)."""
    p = sfem.meshgen.parity_cube20()
    ref = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, 1.0, 0.3, nthreads=0).arrays()
    got = _assemble(sfem, ctx, p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, 1.0, 0.3)
    assert len(got[1][2]) == 2042829
    _check(None, ref, got)


def test_jittered_lognormal_vs_c_oracle(sfem, ctx, coracle):
    """A reduced copy of the 128^3 benchmark mesh: 16^3, jitter 0.2h, E ~ lognormal(0, 0.5)."""
    p = sfem.meshgen.jittered_cube(ne=16)
    ref = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3).arrays()
    got = _assemble(sfem, ctx, p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3)
    _check(None, ref, got)


def _q2_mesh(ne):
    """Structured 9-node Q2 mesh of the unit square (node order of src/fem.jl:80-88)."""
    n1 = 2 * ne + 1
    xs = np.linspace(0, 1, n1)
    X, Yg = np.meshgrid(xs, xs, indexing="xy")
    NL = np.stack([X.ravel(), Yg.ravel()])
    IEN = []
    for j in range(ne):
        for i in range(ne):
            def nid(a, b):
                return (2 * j + b) * n1 + (2 * i + a) + 1
            IEN.append([nid(0, 0), nid(2, 0), nid(2, 2), nid(0, 2),
                        nid(1, 0), nid(2, 1), nid(1, 2), nid(0, 1), nid(1, 1)])
    return NL, np.array(IEN, np.int64)


@pytest.mark.parametrize("ne", [1, 3])
def test_q2_scalar_vs_oracle(sfem, ctx, oracle, ne):
    NL, IEN = _q2_mesh(ne)
    rng = np.random.default_rng(5)
    inner = np.all((NL > 0) & (NL < 1), axis=0)
    NL = NL.copy()
    NL[:, inner] += rng.uniform(-0.05, 0.05, (2, int(inner.sum()))) / ne
    ref = oracle.assemble_system(ne, NL, IEN, 2, "Q2", 1)
    got = _assemble(sfem, ctx, ne, NL, IEN, 2, "Q2", 1, None, 1.0, 0.3)
    _check(oracle, ref, got)


def test_general_id_and_unused_nodes(sfem, ctx, oracle):
    """A permuted (non-interleaved) ID, extra IEN rows beyond ne^ndim, and nodes
    no element uses: rows/cols follow ID, size is max referenced DOF."""
    ne = 3
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, 3)
    rng = np.random.default_rng(3)
    NL = sfem.meshgen.jitter_interior(NL, ne, 0.2, rng)
    nN = NL.shape[1]
    NL = np.concatenate([NL, rng.uniform(0, 1, (3, 5))], axis=1)          # 5 unused nodes
    perm = rng.permutation(3 * (nN + 5)) + 1
    ID2 = perm.reshape(nN + 5, 3)
    IEN2 = np.concatenate([IEN, IEN[:4]], axis=0)                          # extra rows ignored
    ref = oracle.assemble_system(ne, NL, IEN2, 3, "Q1", 3, ID2, 1.0, 0.3)
    got = _assemble(sfem, ctx, ne, NL, IEN2, 3, "Q1", 3, ID2, 1.0, 0.3)
    _check(oracle, ref, got)


def test_deterministic_and_symmetric(sfem, ctx):
    p = sfem.meshgen.jittered_cube(ne=12)
    a = _assemble(sfem, ctx, p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3)[1]
    b = _assemble(sfem, ctx, p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3)[1]
    for x, y in zip(a, b):
        assert np.array_equal(x, y)                                        # bitwise repeatable
    import scipy.sparse as sp
    n = len(a[0]) - 1
    K = sp.csc_matrix((a[2], a[1] - 1, a[0] - 1), shape=(n, n))
    D = (K - K.T).tocoo()
    assert np.all(D.data == 0.0)                                           # bitwise symmetric


def test_large_mesh_properties(sfem, ctx):
    """48^3 hex (352,947 DOFs): nnz formula, rigid-body null space, symmetry."""
    ne = 48
    p = sfem.meshgen.jittered_cube(ne=ne)
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3, ctx=ctx)
    assert K.nnz == 9 * (3 * (ne + 1) - 2) ** 3
    X = p.NodeList
    modes = [np.tile(e, X.shape[1]) for e in np.eye(3)]
    for (i, j) in ((0, 1), (1, 2), (0, 2)):                               # infinitesimal rotations
        r = np.zeros((X.shape[1], 3))
        r[:, i] = -X[j]
        r[:, j] = X[i]
        modes.append(r.ravel())
    scale = abs(K).sum(axis=1).max()
    for r in modes:
        assert np.abs(K @ r).max() <= 1e-12 * scale * np.abs(r).max()


def test_empty_mesh(sfem, ctx):
    NL = np.zeros((3, 8))
    IEN = np.zeros((0, 8), np.int64)
    K = sfem.assemble_system(0, NL, IEN, 3, "Q1", 3, np.arange(1, 25).reshape(8, 3), 1.0, 0.3,
                             ctx=ctx)
    assert K.shape == (0, 0) and K.nnz == 0


def test_errors(sfem, ctx):
    from smearfem_gb300._lib import SfemError
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, 2, 3)
    bad = IEN.copy()
    bad[3, 2] = NL.shape[1] + 7
    with pytest.raises(SfemError) as e:
        sfem.assemble_system(2, NL, bad, 3, "Q1", 3, ID, 1.0, 0.3, ctx=ctx)
    assert e.value.code == 2                                              # SFEM_BAD_INDEX
    with pytest.raises(SfemError) as e:
        sfem.assemble_system(3, NL, IEN, 3, "Q1", 3, ID, 1.0, 0.3, ctx=ctx)  # 27 > 8 IEN rows
    assert e.value.code == 2
    dup = ID.copy()
    dup[5] = dup[6]
    with pytest.raises(SfemError) as e:
        sfem.assemble_system(2, NL, IEN, 3, "Q1", 3, dup, 1.0, 0.3, ctx=ctx)
    assert e.value.code == 1                                              # SFEM_BAD_ARG
    flat = NL.copy()
    flat[:, IEN[0] - 1] = 0.0                                             # element 1 collapsed: J == 0 exactly
    with pytest.raises(SfemError) as e:
        sfem.assemble_system(2, flat, IEN, 3, "Q1", 3, ID, 1.0, 0.3, ctx=ctx)
    assert e.value.code == 3                                              # SFEM_SINGULAR_JACOBIAN
    NL1, IEN1 = np.linspace(0, 1, 3)[None], np.array([[1, 2], [2, 3]])
    with pytest.raises(SfemError) as e:
        sfem.assemble_system(2, NL1, IEN1, 1, "Q1", 1, None, ctx=ctx)
    assert e.value.code == 8                                              # 1D: broken in reference
    # the context stays usable after every error
    K = sfem.assemble_system(2, NL, IEN, 3, "Q1", 3, ID, 1.0, 0.3, ctx=ctx)
    assert K.shape == (81, 81)
