"""GPU: the geometric multigrid preconditioner of the serving and batch
solvers (structured meshgrid Q1 meshes, mixed precision).

Each served request or batch mesh must match its single-mesh FP64 solve within 1e-8,
need far fewer iterations than block Jacobi, and stay bitwise the same
alone and in a mix; meshes that are not the structured grid (elements
renumbered) fall back to block Jacobi and stay correct.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_U = 1e-8


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _single(sfem, ctx, p, rtol=1e-13):
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                             float(p.nu[0]), plane=p.plane, ctx=ctx, as_handle=True)
    u, _ = K.solve(p.fixed_dofs, p.fixed_vals, rtol=rtol)
    K.close()
    return u


def _submit(srv, p, IEN=None, key=0):
    IEN = p.IEN[: p.n_elem] if IEN is None else IEN
    return srv.submit(p.NodeList, IEN, p.ID, p.Young, p.nu, p.fixed_dofs, p.fixed_vals,
                      topology_key=key, ndim=p.ndim, nDof=p.ndim, plane=p.plane)


def _problems(sfem):
    mg = sfem.meshgen
    rng = np.random.default_rng(11)
    quads = [mg.quad_problem(n, 5, jitter=0.15, nu_range=(0.25, 0.45), plane="strain", e_sigma=0.5,
                             rtol=1e-10, rng=rng) for n in (3, 4, 17, 33, 64)]
    hexes = [mg.hex_problem(n, 50 + n, jitter=0.2, e_sigma=0.5, nu=0.4, top="modes") for n in (3, 8, 13)]
    return quads + hexes


def _serve(sfem, probs, precond, **kw):
    args = dict(cluster=4, rtol=1e-12, idle_exit_ms=50.0, precond=precond)
    args.update(kw)
    with sfem.Server(**args) as srv:
        ids = [_submit(srv, p) for p in probs]
        return [srv.wait(i, timeout_ms=120000) for i in ids]


@pytest.mark.timeout(600)
def test_multigrid_matches_single_mesh_solves(sfem, ctx):
    probs = _problems(sfem)
    mg = _serve(sfem, probs, "multigrid")
    bj = _serve(sfem, probs, "block_jacobi")
    for p, (u, res), (ub, rb) in zip(probs, mg, bj):
        assert res["status"] == 0, (p.name, res)
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, (p.name, res)
        if p.ne >= 13:  # the hierarchy pays off: far fewer iterations than block Jacobi
            assert res["iterations"] * 5 < rb["iterations"], (p.name, res["iterations"], rb["iterations"])


@pytest.mark.timeout(600)
def test_multigrid_same_alone_and_in_the_mix(sfem):
    probs = _problems(sfem)
    with sfem.Server(cluster=4, rtol=1e-12, precond="multigrid") as srv:
        alone = {k: srv.wait(_submit(srv, probs[k]), timeout_ms=120000)[0] for k in (1, 4, 6)}
        ids = [_submit(srv, p) for p in probs[::-1]]
        mixed = [srv.wait(i, timeout_ms=120000)[0] for i in ids][::-1]
    for k, u in alone.items():
        assert np.array_equal(u, mixed[k]), probs[k].name


@pytest.mark.timeout(600)
def test_multigrid_falls_back_on_unstructured_numbering(sfem, ctx):
    """Elements listed in another order: not the structured grid, so the
    request is solved with block Jacobi (and still correct)."""
    p = sfem.meshgen.quad_problem(24, 9, jitter=0.15, nu=0.3, plane="strain", rtol=1e-10)
    perm = np.random.default_rng(2).permutation(p.n_elem)
    IEN = np.ascontiguousarray(p.IEN[: p.n_elem][perm])
    with sfem.Server(cluster=2, rtol=1e-12, precond="multigrid") as srv:
        u, res = srv.wait(_submit(srv, p, IEN=IEN), timeout_ms=120000)
        us, rs = srv.wait(_submit(srv, p), timeout_ms=120000)
    assert res["status"] == 0 and rs["status"] == 0
    assert _rel(u, _single(sfem, ctx, p)) <= TOL_U
    assert rs["iterations"] * 3 < res["iterations"], (rs["iterations"], res["iterations"])


@pytest.mark.timeout(600)
def test_multigrid_scalar_classes(sfem, ctx):
    """Laplace on structured 2D and 3D grids with boundary values."""
    mg = sfem.meshgen
    cases = []
    for nd, ne in ((2, 40), (3, 12)):
        NL, IEN, _, _, _ = mg.meshgrid(0, 1, 0, 1, 0, 1 if nd == 3 else 0, ne, nd)
        bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0)) + 1
        v = np.sin(3 * NL[0, bnd - 1]) + NL[1, bnd - 1] ** 2
        cases.append((NL, IEN, nd, ne, bnd, v))
    with sfem.Server(cluster=2, rtol=1e-12, precond="multigrid") as srv:
        outs = [srv.wait(srv.submit(NL, IEN, None, 1.0, 0.3, b_, v_, ndim=nd, nDof=1), timeout_ms=120000)
                for NL, IEN, nd, ne, b_, v_ in cases]
    for (NL, IEN, nd, ne, b_, v_), (u, res) in zip(cases, outs):
        assert res["status"] == 0, res
        K = sfem.assemble_system(ne, NL, IEN, nd, "Q1", 1, ctx=ctx, as_handle=True)
        ref = K.solve(b_, v_, rtol=1e-13)[0]
        K.close()
        assert _rel(u, ref) <= TOL_U, (nd, res)
        assert res["iterations"] < 60, (nd, res)


@pytest.mark.timeout(300)
def test_multigrid_needs_mixed_precision_and_known_option(sfem):
    # FP64 servers accept the option and solve with block Jacobi
    p = sfem.meshgen.quad_problem(10, 1, jitter=0.1, nu=0.3, plane="strain", rtol=1e-10)
    with sfem.Server(cluster=2, rtol=1e-12, precision="fp64", precond="multigrid") as srv:
        u, res = srv.wait(_submit(srv, p), timeout_ms=60000)
    assert res["status"] == 0


def _batch(sfem, ctx, probs, precond, launch=None, E=None):
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    if launch:
        bt.set_launch(*launch)
    Ev = 1.0 if E is None else E
    u, st = bt.solve(Ev, np.array([float(p.nu[0]) for p in probs]), [p.fixed_dofs for p in probs],
                     [p.fixed_vals for p in probs], plane=probs[0].plane, precision="mixed",
                     precond=precond, rtol=1e-12)
    parts = bt.split(u)
    bt.close()
    return parts, st


def _unit_E(p):
    p.Young = np.ones(1)
    return p


@pytest.mark.timeout(600)
@pytest.mark.parametrize("launch", [None, (512, 1, 4, 1)])
def test_batch_multigrid_matches_single_mesh_solves(sfem, ctx, launch):
    """Meshes on one CTA each (default shape) or on 4-CTA clusters; a mesh
    too small for a hierarchy (ne = 2) is solved with block Jacobi."""
    mg = sfem.meshgen
    rng = np.random.default_rng(4)
    probs = [mg.quad_problem(n, 4, jitter=0.15, nu_range=(0.25, 0.45), plane="strain", rtol=1e-10, rng=rng)
             for n in (2, 17, 40, 9, 64, 33)]
    parts, st = _batch(sfem, ctx, probs, "multigrid", launch)
    _, stb = _batch(sfem, ctx, probs, "block_jacobi", launch)
    for p, u, s, sb in zip(probs, parts, st, stb):
        assert s["status"] == 0, (p.name, s)
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, (p.name, s)
        if p.ne >= 17:
            assert s["iterations"] * 5 < sb["iterations"], (p.name, s["iterations"], sb["iterations"])


@pytest.mark.timeout(600)
def test_batch_multigrid_hexes_and_determinism(sfem, ctx):
    mg = sfem.meshgen
    probs = [_unit_E(mg.hex_problem(n, 60 + n, jitter=0.2, nu=0.35, top="modes")) for n in (5, 12, 9)]
    parts, st = _batch(sfem, ctx, probs, "multigrid")
    for p, u, s in zip(probs, parts, st):
        assert s["status"] == 0 and s["iterations"] < 80, (p.name, s)
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, (p.name, s)
    alone, _ = _batch(sfem, ctx, [probs[1]], "multigrid")
    assert np.array_equal(alone[0], parts[1])


@pytest.mark.timeout(600)
@pytest.mark.parametrize("kind", ["quad", "hex"])
def test_single_mesh_multigrid(sfem, ctx, kind):
    """The whole-GPU mixed solver with the multigrid preconditioner: same
    answer as the tight FP64 solve, far fewer iterations than block Jacobi;
    FP64 solves with the option use block Jacobi."""
    mg = sfem.meshgen
    if kind == "quad":
        p = mg.quad_problem(45, 3, jitter=0.15, nu=0.4, plane="strain", e_sigma=0.5, rtol=1e-10)
    else:
        p = mg.hex_problem(15, 8, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes")
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young, float(p.nu[0]),
                             plane=p.plane, ctx=ctx, as_handle=True)
    ref, _ = K.solve(p.fixed_dofs, p.fixed_vals, rtol=1e-13)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond="multigrid", rtol=1e-12)
    _, sb = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond="block_jacobi", rtol=1e-12)
    u64, _ = K.solve(p.fixed_dofs, p.fixed_vals, precision="fp64", precond="multigrid", rtol=1e-12)
    u2, st2 = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond="multigrid", rtol=1e-12)
    K.close()
    assert _rel(u, ref) <= TOL_U and _rel(u64, ref) <= TOL_U, st
    assert st["iterations"] * 5 < sb["iterations"], (st["iterations"], sb["iterations"])
    assert np.array_equal(u, u2) and st2["iterations"] == st["iterations"]  # repeatable


@pytest.mark.timeout(600)
def test_single_mesh_multigrid_unstructured_fallback(sfem, ctx):
    p = sfem.meshgen.quad_problem(20, 6, jitter=0.15, nu=0.3, plane="strain", rtol=1e-10)
    perm = np.random.default_rng(5).permutation(p.n_elem)
    IEN = np.ascontiguousarray(p.IEN[: p.n_elem][perm])
    K = sfem.assemble_system(p.ne, p.NodeList, IEN, 2, "Q1", 2, p.ID, p.Young, float(p.nu[0]),
                             plane=p.plane, ctx=ctx, as_handle=True)
    u, st = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond="multigrid", rtol=1e-12)
    _, sb = K.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", precond="block_jacobi", rtol=1e-12)
    K.close()
    assert _rel(u, _single(sfem, ctx, p)) <= TOL_U
    assert st["iterations"] == sb["iterations"]
