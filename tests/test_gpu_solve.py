"""GPU Dirichlet solve parity against the reference's solve (examples/vector3D.jl:314-322).

Bar: ||u - u_ref||_2 / ||u_ref||_2 <= 1e-8, with u_ref the oracle's dense
``inv(Matrix(K_free))`` solution (or sparse direct / tight PCG where the dense
inverse does not fit), for the FP64 path and the mixed-precision path.
"""
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_U = 1e-8
GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "cube20_dense_inv.npz")


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _handle(sfem, ctx, p):
    return sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                                p.nu if p.nu.size > 1 else float(p.nu[0]), plane=p.plane,
                                ctx=ctx, as_handle=True)


@pytest.mark.skipif(not os.path.exists(GOLDEN), reason="cube20 dense-inverse fixture not generated")
@pytest.mark.parametrize("precision,precond", [("fp64", "jacobi"), ("fp64", "block_jacobi"),
                                               ("mixed", "jacobi"), ("mixed", "block_jacobi")])
def test_cube20_vs_dense_inverse(sfem, ctx, precision, precond):
    """20^3 unit cube vs the reference's own algorithm: dense inverse of K_free."""
    g = np.load(GOLDEN)
    p = sfem.meshgen.parity_cube20()
    K = _handle(sfem, ctx, p)
    assert K.n == int(g["n"]) and K.nnz == int(g["nnz"])
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision=precision, precond=precond, rtol=1e-12)
    assert st["status"] == 0
    assert _rel(u, g["u"]) <= TOL_U, (st, _rel(u, g["u"]))
    assert np.array_equal(u[p.fixed_dofs - 1], p.fixed_vals)


SMALL = [
    ("hex", dict(ne=4, seed=21, jitter=0.2, e_sigma=0.5, top="modes")),
    ("hex", dict(ne=6, seed=22, jitter=0.2, e_sigma=1.0, nu_range=(0.25, 0.45), top="modes")),
    ("quad", dict(ne=9, seed=23, jitter=0.15, nu_range=(0.2, 0.45), plane="strain")),
    ("quad", dict(ne=7, seed=24, jitter=0.15, nu=0.3, e_sigma=0.5, plane="stress")),
]


@pytest.mark.parametrize("kind,kw", SMALL, ids=lambda x: str(x)[:40])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_small_vs_dense_inverse(sfem, ctx, oracle, kind, kw, precision):
    p = (sfem.meshgen.hex_problem(**kw) if kind == "hex" else sfem.meshgen.quad_problem(**kw))
    Kref = oracle.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                                  p.nu if p.nu.size > 1 else float(p.nu[0]), p.plane)
    uref = oracle.solve_eliminated(Kref, p.fixed_dofs, p.fixed_vals, method="inv")
    K = _handle(sfem, ctx, p)
    for precond in ("jacobi", "block_jacobi"):
        u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision=precision, precond=precond, rtol=1e-12)
        assert _rel(u, uref) <= TOL_U, (precond, st)


def test_load_vector_and_laplace(sfem, ctx, oracle):
    """Scalar Laplace (nDof=1) with a load vector f: C'(f - K q_d)."""
    ne = 8
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, 2)
    rng = np.random.default_rng(9)
    NL = sfem.meshgen.jitter_interior(NL, ne, 0.2, rng)
    bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0)) + 1
    vals = np.sin(NL[0, bnd - 1]) + NL[1, bnd - 1] ** 2
    f = rng.normal(size=NL.shape[1]) / ne ** 2
    Kref = oracle.assemble_system(ne, NL, IEN, 2, "Q1", 1)
    uref = oracle.solve_eliminated(Kref, bnd, vals, f=f, method="inv")
    K = sfem.assemble_system(ne, NL, IEN, 2, "Q1", 1, ctx=ctx, as_handle=True)
    for precision in ("fp64", "mixed"):
        u, st = K.solve(bnd, vals, f=f, precision=precision, rtol=1e-12)
        assert _rel(u, uref) <= TOL_U


def test_patch_test_linear_field(sfem, ctx):
    """A linear displacement prescribed on the boundary of a jittered mesh of
    one homogeneous material is reproduced exactly inside (the Q1 patch test)."""
    p = sfem.meshgen.hex_problem(6, 31, jitter=0.2, e_sigma=None, top="sin")
    X = p.NodeList
    A = np.array([[0.01, -0.02, 0.005], [0.003, 0.02, -0.01], [-0.015, 0.004, 0.01]])
    ulin = (A @ X + np.array([[0.1], [-0.2], [0.05]])).T.ravel()
    bnd = np.flatnonzero(np.any((X == 0) | (X == 1), axis=0))
    dofs = (3 * bnd[:, None] + np.arange(1, 4)).ravel()
    K = _handle(sfem, ctx, p)
    for precision in ("fp64", "mixed"):
        u, st = K.solve(dofs, ulin[dofs - 1], precision=precision, rtol=1e-13)
        assert np.abs(u - ulin).max() <= 1e-9 * np.abs(ulin).max()


def test_medium_vs_c_oracle(sfem, ctx, coracle):
    """24^3 jittered lognormal mesh (46,875 DOFs) vs the C oracle's FP64 PCG at 1e-13."""
    p = sfem.meshgen.jittered_cube(ne=24)
    Kc = coracle.assemble(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, p.Young, 0.3)
    uref, _ = Kc.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    K = _handle(sfem, ctx, p)
    for precision, precond in (("fp64", "jacobi"), ("mixed", "block_jacobi")):
        u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision=precision, precond=precond,
                        rtol=1e-11)
        assert _rel(u, uref) <= TOL_U, (precision, st)
        assert st["relres"] <= 1e-11


def test_solver_status_paths(sfem, ctx):
    from smearfem_gb300._lib import SfemError
    p = sfem.meshgen.hex_problem(4, 41, jitter=0.1, top="sin")
    K = _handle(sfem, ctx, p)
    with pytest.raises(SfemError) as e:
        K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-14, maxit=3)
    assert e.value.code == 5                                              # SFEM_NOT_CONVERGED
    alld = np.arange(1, K.n + 1)
    vals = np.linspace(-1, 1, K.n)
    u, st = K.solve(alld, vals)                                           # nothing free
    assert np.array_equal(u, vals) and st["n_free"] == 0
    with pytest.raises(SfemError) as e:
        K.solve(np.array([K.n + 5]), np.array([0.0]))
    assert e.value.code == 2                                              # bad DOF id
    u, st = K.solve(p.fixed_dofs, np.zeros_like(p.fixed_vals))            # homogeneous -> 0
    assert np.all(u == 0.0)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-10)               # still usable
    assert st["status"] == 0


def test_repeatable_bitwise(sfem, ctx):
    p = sfem.meshgen.jittered_cube(ne=10)
    K = _handle(sfem, ctx, p)
    for precision in ("fp64", "mixed"):
        a, _ = K.solve(p.fixed_dofs, p.fixed_vals, precision=precision)
        b, _ = K.solve(p.fixed_dofs, p.fixed_vals, precision=precision)
        assert np.array_equal(a, b)


@pytest.mark.parametrize("storage", ["upper", "full"])
@pytest.mark.parametrize("precond", ["jacobi", "block_jacobi"])
def test_mixed_fp32_storages(sfem, ctx, storage, precond):
    """The mixed solver's FP32 K as upper-triangle blocks (default) or full
    blocks: both reach the FP64 solution within 1e-8."""
    p = sfem.meshgen.contrast_cube(ne=12)
    K = _handle(sfem, ctx, p)
    ref, _ = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond=precond, rtol=1e-11,
                    fp32_storage=storage)
    assert st["status"] == 0 and st["reliable_updates"] >= 1
    assert _rel(u, ref) <= TOL_U


def test_mixed_upper_storage_general_id(sfem, ctx, oracle):
    """Upper-triangle FP32 storage on a permuted ID with unused nodes."""
    ne = 5
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, 3)
    rng = np.random.default_rng(12)
    NL = sfem.meshgen.jitter_interior(NL, ne, 0.2, rng)
    nN = NL.shape[1]
    NL = np.concatenate([NL, rng.uniform(0, 1, (3, 3))], axis=1)
    ID2 = (rng.permutation(3 * (nN + 3)) + 1).reshape(nN + 3, 3)
    bot = np.flatnonzero(NL[2, :nN] == 0)
    top = np.flatnonzero(NL[2, :nN] == 1)
    fixed = np.concatenate([ID2[bot].ravel(), ID2[top, 2], ID2[nN:].ravel()])
    vals = np.concatenate([np.zeros(3 * bot.size), 0.01 * np.sin(np.pi * NL[0, top]),
                           np.zeros(9)])
    Kref = oracle.assemble_system(ne, NL, IEN, 3, "Q1", 3, ID2, 1.0, 0.3)
    n = Kref[4]
    keep = fixed <= n
    uref = oracle.solve_eliminated(Kref, fixed[keep], vals[keep], method="inv")
    K = sfem.assemble_system(ne, NL, IEN, 3, "Q1", 3, ID2, 1.0, 0.3, ctx=ctx, as_handle=True)
    u, st = K.solve(fixed[keep], vals[keep], precision="mixed", precond="block_jacobi", rtol=1e-12)
    assert _rel(u, uref) <= TOL_U
