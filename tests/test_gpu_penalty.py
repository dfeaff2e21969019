"""GPU: surface penalty K_bar = K + beta*b and the load-increment loop of the
reference's squeeze-flow driver (examples/vector3D.jl:175-264, :266-338).

K_bar must match the oracle's K + beta*b within 1e-12 (row-scaled) on K's
exact pattern; every increment's displacement must match the oracle's
dense-inverse solve of K_bar within 1e-8; with warm starts the steps after
the second start at the answer.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_K = 1e-12
TOL_U = 1e-8
BETA = 100.0


@pytest.fixture(scope="module")
def squeeze(oracle):
    import __graft_entry__ as GE
    mg = GE.load_package().meshgen
    ne = 6
    NL, IEN, ID, IT, IB, cyl, faces = mg.squeeze_problem(ne)
    K = oracle.assemble_system(ne, NL, IEN, 3, "Q1", 3, ID, 40.0, 0.4)
    b = oracle.apply_boundary_conditions_loops(ne, cyl, IEN, IT, IB, 3, "Q1", ID)
    Kbar = oracle.add_scaled(K, BETA, b)
    return dict(ne=ne, NL=NL, IEN=IEN, ID=ID, IT=IT, IB=IB, cyl=cyl, faces=faces, K=K, b=b, Kbar=Kbar)


def _rowscaled(got, ref):
    """max |got_ij - ref_ij| / max_k |ref_ik| over the (shared) stored entries."""
    rowmax = np.asarray(abs(ref).max(axis=1).todense()).ravel()
    rowmax[rowmax == 0] = 1.0
    coo = ref.tocoo()
    return float(np.max(np.abs(got.tocsc()[coo.row, coo.col].A1 - coo.data) / rowmax[coo.row]))


def _csc(A):
    A = A.tocsc()
    A.sort_indices()
    return (A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, A.data.copy(), A.shape[0],
            A.shape[1])


def _gpu_kbar(sfem, ctx, q):
    K = sfem.assemble_system(q["ne"], q["NL"], q["IEN"], 3, "Q1", 3, q["ID"], 40.0, 0.4, ctx=ctx,
                             as_handle=True)
    K.add_penalty(q["cyl"], q["faces"], BETA)
    return K


def test_kbar_matches_oracle(sfem, ctx, squeeze):
    """K_bar keeps K's pattern on the device.  Julia's sparse `+` (like
    scipy's) drops entries that come out exactly 0, so the reference's
    pattern is a subset of it; the entries only the GPU stores are zeros to
    rounding."""
    K = _gpu_kbar(sfem, ctx, squeeze)
    got = K.to_scipy().tocsc()
    K.close()
    ref = squeeze["Kbar"].tocsc()
    rows, cols = ref.nonzero()
    stored = set(zip(*got.tocoo().coords))
    assert all((r, c) in stored for r, c in zip(rows, cols))
    assert _rowscaled(got, ref) <= TOL_K
    rowmax = np.asarray(abs(ref).max(axis=1).todense()).ravel()
    g = got.tocoo()
    ref_set = set(zip(rows, cols))
    only_gpu = np.array([(r, c) not in ref_set for r, c in zip(g.row, g.col)], dtype=bool)
    assert np.all(np.abs(g.data[only_gpu]) <= TOL_K * rowmax[g.row[only_gpu]])


def test_penalty_matrix_alone(sfem, ctx, squeeze, oracle):
    q = squeeze
    got = sfem.apply_boundary_conditions(q["ne"], q["cyl"], q["IEN"], q["IT"], q["IB"], 3, "Q1", q["ID"],
                                         ctx=ctx)
    ref = oracle.csc_to_scipy(*q["b"])
    ref.sort_indices()
    assert got.shape == ref.shape
    assert np.array_equal(got.indptr, ref.indptr) and np.array_equal(got.indices, ref.indices)
    assert np.max(np.abs(got.data - ref.data)) <= 1e-15 * np.max(np.abs(ref.data))


def test_penalty_refreshes_fp32_copies(sfem, ctx, squeeze, oracle):
    """A mixed solve after the penalty sees K_bar, not K (the FP32 copies are refreshed)."""
    q = squeeze
    K = sfem.assemble_system(q["ne"], q["NL"], q["IEN"], 3, "Q1", 3, q["ID"], 40.0, 0.4, ctx=ctx,
                             as_handle=True)
    fd, fv = sfem.meshgen.squeeze_increments(q["NL"], [0.05])
    K.solve(fd, fv[0], precision="mixed", precond="block_jacobi", rtol=1e-12)   # builds the FP32 copies
    K.add_penalty(q["cyl"], q["faces"], BETA)
    u, st = K.solve(fd, fv[0], precision="mixed", precond="block_jacobi", rtol=1e-12)
    K.close()
    ref = oracle.solve_eliminated(_csc(q["Kbar"]), fd, fv[0], method="inv")
    assert np.linalg.norm(u - ref) / np.linalg.norm(ref) <= TOL_U


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_load_increments(sfem, ctx, squeeze, oracle, precision):
    q = squeeze
    deltas = np.arange(0.001, 0.5, 0.01)[:8]               # the driver's 0.001:0.01:0.5, first 8
    fd, fv = sfem.meshgen.squeeze_increments(q["NL"], deltas)
    K = _gpu_kbar(sfem, ctx, q)
    U, st = K.solve_increments(fd, fv, precision=precision, precond="block_jacobi", rtol=1e-12)
    U0, st0 = K.solve_increments(fd, fv, warm_start=False, precision=precision, precond="block_jacobi",
                                 rtol=1e-12)
    K.close()
    Kb = _csc(q["Kbar"])
    for k, d in enumerate(deltas):
        ref = oracle.solve_eliminated(Kb, fd, fv[k], method="inv")
        assert np.linalg.norm(U[k] - ref) / np.linalg.norm(ref) <= TOL_U, (k, st[k])
        assert np.linalg.norm(U0[k] - ref) / np.linalg.norm(ref) <= TOL_U, (k, st0[k])
        assert st[k]["status"] == 0 and st0[k]["status"] == 0
    assert all(s["iterations"] > 0 for s in st0)
    assert all(s["iterations"] == 0 for s in st[2:])       # affine warm start lands on the answer
    assert sum(s["iterations"] for s in st) < sum(s["iterations"] for s in st0) / 3


def test_penalty_errors(sfem, ctx, squeeze):
    q = squeeze
    K = sfem.assemble_system(q["ne"], q["NL"], q["IEN"], 3, "Q1", 3, q["ID"], 40.0, 0.4, ctx=ctx,
                             as_handle=True)
    bad = q["faces"].copy()
    bad[0, 0] = q["NL"].shape[1] + 5
    with pytest.raises(sfem.SfemError):
        K.add_penalty(q["cyl"], bad, BETA)                    # node out of range
    far = q["faces"].copy()
    far[0] = [1, 2, q["NL"].shape[1] - 1, q["NL"].shape[1]]  # couples nodes of no common element
    with pytest.raises(sfem.SfemError):
        K.add_penalty(q["cyl"], far, BETA)
    K.close()
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 0, 3, 2)
    K2 = sfem.assemble_system(3, NL, IEN, 2, "Q1", 2, ID, ctx=ctx, as_handle=True)
    with pytest.raises(sfem.SfemError):
        K2.add_penalty(np.zeros((3, NL.shape[1])), np.array([[1, 2, 6, 5]]), BETA)
    K2.close()
