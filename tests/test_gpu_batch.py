"""GPU: batches of independent meshes solved by the persistent kernel.

Each mesh of a batch must match its own single-mesh solve (and the oracle's
dense inverse) within 1e-8, and its result must be bitwise the same whether
it is solved alone or in a mix of other meshes.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_U = 1e-8


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _quads(sizes, seed=3):
    rng = np.random.default_rng(seed)
    import __graft_entry__ as GE
    mg = GE.load_package().meshgen
    return [mg.quad_problem(int(n), seed, jitter=0.15, nu_range=(0.2, 0.45), plane="strain",
                            rtol=1e-10, rng=rng) for n in sizes]


def _solve_batch(sfem, ctx, probs, precision="mixed", precond="block_jacobi", rtol=1e-10, **kw):
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    nus = np.array([float(p.nu[0]) for p in probs])
    u, st = bt.solve(1.0, nus, [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs],
                     plane=probs[0].plane, precision=precision, precond=precond, rtol=rtol, **kw)
    parts = bt.split(u)
    bt.close()
    return parts, st


def _single(sfem, ctx, p, rtol=1e-13):
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                             float(p.nu[0]), plane=p.plane, ctx=ctx, as_handle=True)
    u, _ = K.solve(p.fixed_dofs, p.fixed_vals, rtol=rtol)
    K.close()
    return u


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_matches_single_mesh_solves(sfem, ctx, precision):
    probs = _quads([5, 17, 9, 33, 2, 24, 12, 40])
    parts, st = _solve_batch(sfem, ctx, probs, precision=precision)
    for p, u, s in zip(probs, parts, st):
        assert s["status"] == 0, s
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, (p.name, s)


def test_batch_vs_dense_inverse(sfem, ctx, oracle):
    probs = _quads([3, 6, 4], seed=9)
    parts, st = _solve_batch(sfem, ctx, probs, rtol=1e-12)
    for p, u in zip(probs, parts):
        Kref = oracle.assemble_system(p.ne, p.NodeList, p.IEN, 2, "Q1", 2, p.ID, 1.0,
                                      float(p.nu[0]), "strain")
        uref = oracle.solve_eliminated(Kref, p.fixed_dofs, p.fixed_vals, method="inv")
        assert _rel(u, uref) <= TOL_U


def test_same_alone_and_in_the_mix(sfem, ctx):
    """A mesh's result is bitwise identical alone and inside a batch."""
    probs = _quads([30, 7, 19, 26, 11], seed=21)
    mixed_parts, _ = _solve_batch(sfem, ctx, probs)
    for k in (0, 2, 4):
        alone, _ = _solve_batch(sfem, ctx, [probs[k]])
        assert np.array_equal(alone[0], mixed_parts[k])
    # and in a different mix / order
    reordered, _ = _solve_batch(sfem, ctx, [probs[4], probs[2], probs[0]])
    assert np.array_equal(reordered[0], mixed_parts[4])
    assert np.array_equal(reordered[2], mixed_parts[0])


def test_batch_3d_hex_per_element_material(sfem, ctx):
    mg = sfem.meshgen
    probs = [mg.hex_problem(n, 40 + n, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes", rtol=1e-10)
             for n in (3, 7, 5)]
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    E = np.concatenate([p.Young for p in probs])
    u, st = bt.solve(E, 0.3, [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs],
                     precision="mixed", precond="block_jacobi", rtol=1e-10)
    for p, up, s in zip(probs, bt.split(u), st):
        assert s["status"] == 0 and s["refreshes"] >= 1
        assert _rel(up, _single(sfem, ctx, p)) <= TOL_U
    bt.close()


def test_batch_scalar_laplace(sfem, ctx):
    mg = sfem.meshgen
    meshes, fixed, vals, refs = [], [], [], []
    for n in (4, 9, 6):
        NL, IEN, _, _, _ = mg.meshgrid(0, 1, 0, 1, 0, 0, n, 2)
        bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0)) + 1
        v = np.sin(3 * NL[0, bnd - 1]) + NL[1, bnd - 1]
        meshes.append((NL, IEN))
        fixed.append(bnd)
        vals.append(v)
        K = sfem.assemble_system(n, NL, IEN, 2, "Q1", 1, ctx=ctx, as_handle=True)
        refs.append(K.solve(bnd, v, rtol=1e-13)[0])
    bt = sfem.Batch(meshes, 2, 1, ctx=ctx)
    u, st = bt.solve(1.0, 0.3, fixed, vals, precision="mixed", rtol=1e-11)
    for up, r in zip(bt.split(u), refs):
        assert _rel(up, r) <= TOL_U
    bt.close()


def test_batch_errors_and_status(sfem, ctx):
    probs = _quads([4, 6], seed=2)
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    bad = [probs[0].fixed_dofs, np.array([10 ** 6])]
    u, st = bt.solve(1.0, 0.3, bad, [probs[0].fixed_vals, np.zeros(1)], precision="mixed")
    assert st[0]["status"] == 0 and st[1]["status"] == 2      # the bad mesh alone fails
    u, st = bt.solve(1.0, 0.3, [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs],
                     precision="fp64", rtol=1e-14, maxit=2)
    assert all(s["status"] == 5 for s in st)                  # SFEM_NOT_CONVERGED
    bt.close()
    with pytest.raises(sfem.SfemError):
        NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 0, 3, 2)
        IEN = IEN.copy()
        IEN[0, 0] = 99
        sfem.Batch([(NL, IEN, ID)], 2, 2, ctx=ctx)


@pytest.mark.parametrize("cluster", [2, 8])
def test_cluster_mode(sfem, ctx, cluster):
    """Meshes solved by a thread-block cluster (forced for every mesh here)
    match their single-mesh solves, and stay bitwise identical alone vs in
    the mix for a fixed launch shape."""
    probs = _quads([20, 9, 33, 5, 27], seed=31)

    def run(ps):
        bt = sfem.Batch.from_problems(ps, ctx=ctx)
        bt.set_launch(512, 1, cluster, 1)
        u, st = bt.solve(1.0, np.array([float(p.nu[0]) for p in ps]), [p.fixed_dofs for p in ps],
                         [p.fixed_vals for p in ps], plane="strain", precision="mixed",
                         precond="block_jacobi", rtol=1e-10)
        parts = bt.split(u)
        bt.close()
        return parts, st

    parts, st = run(probs)
    for p, u, s in zip(probs, parts, st):
        assert s["status"] == 0
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U
    alone, _ = run([probs[2]])
    assert np.array_equal(alone[0], parts[2])


def test_cluster_mode_3d_fp64(sfem, ctx):
    mg = sfem.meshgen
    probs = [mg.hex_problem(n, 70 + n, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes", rtol=1e-10)
             for n in (6, 4)]
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    bt.set_launch(256, 1, 4, 1)
    E = np.concatenate([p.Young for p in probs])
    u, st = bt.solve(E, 0.3, [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs],
                     precision="fp64", precond="block_jacobi", rtol=1e-11)
    for p, up, s in zip(probs, bt.split(u), st):
        assert s["status"] == 0
        assert _rel(up, _single(sfem, ctx, p)) <= TOL_U
    bt.close()


def test_autotune_picks_a_valid_shape(sfem, ctx):
    probs = _quads([30, 12, 70, 9, 44, 5], seed=51)
    bt = sfem.Batch.from_problems(probs, ctx=ctx)
    nus = np.array([float(p.nu[0]) for p in probs])
    fx, fv = [p.fixed_dofs for p in probs], [p.fixed_vals for p in probs]
    shape, ms = bt.autotune(1.0, nus, fx, fv, plane="strain", precision="mixed",
                            precond="block_jacobi", rtol=1e-10, sample=6)
    assert ms > 0 and shape["threads"] in (256, 512) and shape["cluster"] in (1, 2, 4, 8)
    u, st = bt.solve(1.0, nus, fx, fv, plane="strain", precision="mixed", precond="block_jacobi",
                     rtol=1e-10)
    for p, up, s in zip(probs, bt.split(u), st):
        assert s["status"] == 0 and s["ms"] > 0
        assert _rel(up, _single(sfem, ctx, p)) <= TOL_U
    bt.close()
