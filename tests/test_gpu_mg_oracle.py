"""GPU: the multigrid preconditioner (mixed precision) against the oracle.

The single-mesh solver, the batch kernel and the serving loop each solve
structured meshes with ``precond="multigrid"``; every displacement must be
within 1e-8 (relative 2-norm) of the oracle's solution of the same problem:
the reference's own dense-inverse solve of K_free (examples/vector3D.jl:
315-322, restated in oracle/fem_ref.py) on small meshes, and the C oracle's
FP64 assembly with Jacobi-PCG to 1e-13 on a larger one.  The iteration counts
show that the hierarchy was used (block Jacobi needs several times more).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_U = 1e-8


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _problems(sfem):
    mg = sfem.meshgen
    rng = np.random.default_rng(31)
    quads = [mg.quad_problem(n, 7, jitter=0.15, nu_range=(0.25, 0.45), plane="strain", e_sigma=0.5,
                             rtol=1e-10, rng=rng) for n in (4, 9, 14)]
    hexes = [mg.hex_problem(n, 70 + n, jitter=0.2, e_sigma=0.5, nu=0.35, top="modes") for n in (3, 5)]
    return quads + hexes


def _dense_inverse(oracle, p):
    K = oracle.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                               float(p.nu[0]), p.plane)
    return oracle.solve_eliminated(K, p.fixed_dofs, p.fixed_vals, method="inv")


def _c_oracle(coracle, p):
    K = coracle.assemble(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young, float(p.nu[0]),
                         plane=p.plane)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    assert st["status"] == 0, st
    return u


def _single(sfem, ctx, p, precond):
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                             float(p.nu[0]), plane=p.plane, ctx=ctx, as_handle=True)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond=precond, rtol=1e-12)
    K.close()
    return u, st


@pytest.mark.timeout(600)
def test_single_mesh_multigrid_vs_dense_inverse(sfem, ctx, oracle):
    for p in _problems(sfem):
        u, st = _single(sfem, ctx, p, "multigrid")
        assert st["status"] == 0, (p.name, st)
        assert _rel(u, _dense_inverse(oracle, p)) <= TOL_U, (p.name, st)


@pytest.mark.timeout(600)
def test_single_mesh_multigrid_vs_c_oracle(sfem, ctx, coracle):
    p = sfem.meshgen.hex_problem(16, 77, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes")
    u, st = _single(sfem, ctx, p, "multigrid")
    _, sb = _single(sfem, ctx, p, "block_jacobi")
    assert st["status"] == 0 and st["iterations"] * 5 < sb["iterations"], (st, sb["iterations"])
    assert _rel(u, _c_oracle(coracle, p)) <= TOL_U, st


@pytest.mark.timeout(600)
def test_batch_multigrid_vs_dense_inverse(sfem, ctx, oracle):
    probs = [p for p in _problems(sfem) if p.ndim == 2]
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    nus = np.array([float(p.nu[0]) for p in probs])
    Es = np.concatenate([np.broadcast_to(p.Young, (p.n_elem,)) for p in probs])
    u, st = bt.solve(Es, nus, [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs],
                     plane="strain", precision="mixed", precond="multigrid", rtol=1e-12)
    parts = bt.split(u)
    bt.close()
    for p, x, s in zip(probs, parts, st):
        assert s["status"] == 0, (p.name, s)
        assert _rel(x, _dense_inverse(oracle, p)) <= TOL_U, (p.name, s)


@pytest.mark.timeout(600)
def test_served_multigrid_vs_oracle(sfem, oracle, coracle):
    probs = _problems(sfem)
    big = sfem.meshgen.quad_problem(64, 8, jitter=0.15, nu=0.45, plane="strain", e_sigma=0.5, rtol=1e-10)
    with sfem.Server(cluster=4, rtol=1e-12, precond="multigrid", idle_exit_ms=50.0) as srv:
        ids = [srv.submit(p.NodeList, p.IEN[: p.n_elem], p.ID, p.Young, p.nu, p.fixed_dofs, p.fixed_vals,
                          ndim=p.ndim, nDof=p.ndim, plane=p.plane) for p in probs + [big]]
        outs = [srv.wait(i, timeout_ms=120000) for i in ids]
    for p, (u, res) in zip(probs, outs):
        assert res["status"] == 0, (p.name, res)
        assert _rel(u, _dense_inverse(oracle, p)) <= TOL_U, (p.name, res)
    u, res = outs[-1]
    assert res["status"] == 0 and res["iterations"] < 80, res
    assert _rel(u, _c_oracle(coracle, big)) <= TOL_U, res


@pytest.mark.timeout(600)
def test_single_mesh_multigrid_is_repeatable(sfem, ctx):
    """The single-mesh hierarchy (fine stencil copy, direction-wise Galerkin
    passes, one-CTA coarse levels) and the cycle use no value atomics: two
    solves of the same problem return the same displacements bitwise, on an
    odd-sized hex mesh and a quad mesh."""
    for p in (sfem.meshgen.hex_problem(13, 91, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes"),
              sfem.meshgen.quad_problem(37, 5, jitter=0.15, nu=0.4, plane="strain", e_sigma=0.5, rtol=1e-10)):
        u1, s1 = _single(sfem, ctx, p, "multigrid")
        u2, s2 = _single(sfem, ctx, p, "multigrid")
        assert s1["status"] == 0 and s1["iterations"] == s2["iterations"], (p.name, s1, s2)
        assert np.array_equal(u1, u2), p.name
