"""GPU: the device-resident request loop (sfem_server_*).

Every served request must match its own single-mesh solve within 1e-8 and
be bitwise the same whether it is served alone or among other requests;
admission by HBM budget, the topology cache, the kernel's idle exit and
relaunch, and shutdown with work outstanding are checked on small meshes.
"""
import time

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TOL_U = 1e-8


def _rel(u, v):
    return float(np.linalg.norm(u - v) / np.linalg.norm(v))


def _quads(sizes, seed=3, e_sigma=None):
    rng = np.random.default_rng(seed)
    import __graft_entry__ as GE
    mg = GE.load_package().meshgen
    return [mg.quad_problem(int(n), seed, jitter=0.15, nu_range=(0.2, 0.45), plane="strain",
                            e_sigma=e_sigma, rtol=1e-10, rng=rng) for n in sizes]


def _single(sfem, ctx, p, rtol=1e-13):
    K = sfem.assemble_system(p.ne, p.NodeList, p.IEN, p.ndim, "Q1", p.ndim, p.ID, p.Young,
                             float(p.nu[0]), plane=p.plane, ctx=ctx, as_handle=True)
    u, _ = K.solve(p.fixed_dofs, p.fixed_vals, rtol=rtol)
    K.close()
    return u


def _submit(srv, p, key=0, with_ien=True):
    return srv.submit(p.NodeList, p.IEN[: p.n_elem] if with_ien else None, p.ID if with_ien else None,
                      p.Young, p.nu, p.fixed_dofs, p.fixed_vals, topology_key=key, ndim=p.ndim,
                      nDof=p.ndim, plane=p.plane)


def _server(sfem, **kw):
    args = dict(cluster=4, rtol=1e-12, idle_exit_ms=50.0)
    args.update(kw)
    return sfem.Server(**args)


@pytest.mark.timeout(300)
def test_served_requests_match_single_mesh_solves(sfem, ctx):
    probs = _quads([5, 17, 9, 33, 2, 24, 12, 40, 3, 61], e_sigma=0.5)
    with _server(sfem) as srv:
        ids = [_submit(srv, p) for p in probs]
        for p, rid in zip(probs, ids):
            u, res = srv.wait(rid, timeout_ms=60000)
            assert res["status"] == 0, res
            assert res["ndof"] == p.n_dof and res["gpu_ms"] > 0 and res["total_ms"] >= res["queue_ms"]
            assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, (p.name, res)
        info = srv.info()
        assert info["completed"] == len(probs) and info["pending"] == 0 and info["inflight"] == 0
        assert info["bytes_in_use"] == 0 and info["kernel_launches"] >= 1


@pytest.mark.timeout(300)
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_same_alone_and_in_the_mix(sfem, ctx, precision):
    """A request's displacements are bitwise identical served alone and
    served while other requests share the GPU."""
    probs = _quads([30, 7, 19, 26, 11, 44], seed=21)
    with _server(sfem, precision=precision) as srv:
        alone = {}
        for k in (0, 3, 5):
            alone[k], _ = srv.wait(_submit(srv, probs[k]), timeout_ms=60000)
        ids = [_submit(srv, p) for p in probs]
        mixed = [srv.wait(i, timeout_ms=60000)[0] for i in ids]
    for k, u in alone.items():
        assert np.array_equal(u, mixed[k])
    with _server(sfem, precision=precision) as srv2:   # another server, reversed order
        ids = [_submit(srv2, p) for p in probs[::-1]]
        rev = [srv2.wait(i, timeout_ms=60000)[0] for i in ids][::-1]
    for a, b in zip(rev, mixed):
        assert np.array_equal(a, b)


@pytest.mark.timeout(300)
def test_admission_by_hbm_budget(sfem, ctx):
    """With a budget below one request's footprint, requests still run, one at a time."""
    probs = _quads([12, 20, 8, 16], seed=5)
    with _server(sfem, hbm_budget_bytes=1) as srv:
        ids = [_submit(srv, p) for p in probs]
        outs = [srv.wait(i, timeout_ms=60000) for i in ids]
        info = srv.info()
    assert info["peak_inflight"] == 1 and info["budget_bytes"] == 1
    for p, (u, res) in zip(probs, outs):
        assert res["status"] == 0
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U


@pytest.mark.timeout(300)
def test_topology_cache(sfem, ctx):
    """Requests with one topology key share a pattern; only the first carries IEN/ID."""
    mg = sfem.meshgen
    probs = [mg.quad_problem(14, 100 + k, jitter=0.15, nu_range=(0.2, 0.45), e_sigma=0.3,
                             plane="strain") for k in range(5)]
    with _server(sfem) as srv:
        ids = [_submit(srv, p, key=14, with_ien=(k == 0)) for k, p in enumerate(probs)]
        outs = [srv.wait(i, timeout_ms=60000) for i in ids]
        assert srv.info()["topologies"] == 1
    for p, (u, res) in zip(probs, outs):
        assert res["status"] == 0
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U


@pytest.mark.timeout(300)
def test_idle_exit_and_relaunch(sfem, ctx):
    probs = _quads([9, 13], seed=8)
    with _server(sfem, idle_exit_ms=5.0) as srv:
        u0, r0 = srv.wait(_submit(srv, probs[0]), timeout_ms=60000)
        time.sleep(0.3)                                   # the kernel leaves after 5 ms idle
        u1, r1 = srv.wait(_submit(srv, probs[1]), timeout_ms=60000)
        assert srv.info()["kernel_launches"] >= 2
    assert r0["status"] == 0 and r1["status"] == 0
    assert _rel(u1, _single(sfem, ctx, probs[1])) <= TOL_U


@pytest.mark.timeout(300)
def test_3d_hex_and_scalar_requests(sfem, ctx):
    mg = sfem.meshgen
    probs = [mg.hex_problem(n, 40 + n, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes") for n in (3, 7, 5)]
    with sfem.Server(cluster=2, rtol=1e-12) as srv:
        ids = [_submit(srv, p) for p in probs]
        for p, i in zip(probs, ids):
            u, res = srv.wait(i, timeout_ms=60000)
            assert res["status"] == 0 and res["refreshes"] >= 1
            assert _rel(u, _single(sfem, ctx, p)) <= TOL_U
    NL, IEN, _, _, _ = mg.meshgrid(0, 1, 0, 1, 0, 0, 11, 2)
    bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0)) + 1
    v = np.sin(3 * NL[0, bnd - 1]) + NL[1, bnd - 1]
    K = sfem.assemble_system(11, NL, IEN, 2, "Q1", 1, ctx=ctx, as_handle=True)
    ref = K.solve(bnd, v, rtol=1e-13)[0]
    K.close()
    with sfem.Server(cluster=1, rtol=1e-12) as srv:
        u, res = srv.wait(srv.submit(NL, IEN, None, 1.0, 0.3, bnd, v), timeout_ms=60000)
    assert res["status"] == 0 and _rel(u, ref) <= TOL_U


@pytest.mark.timeout(300)
def test_scalar_classes_3d_and_q2(sfem, ctx):
    """The scalar branches of the serving kernel: 3D Q1 and 2D Q2 Laplace."""
    mg = sfem.meshgen
    cases = []
    NL, IEN, _, _, _ = mg.meshgrid(0, 1, 0, 1, 0, 1, 5, 3)
    bnd = np.flatnonzero(np.any((NL == 0) | (NL == 1), axis=0)) + 1
    cases.append((NL, IEN, 3, "Q1", bnd, NL[0, bnd - 1] * NL[1, bnd - 1] + NL[2, bnd - 1], 5))
    # 2D Q2: 9-node elements on a (2n+1)^2 node grid
    n = 4
    m1 = 2 * n + 1
    xs = np.linspace(0, 1, m1)
    X, Y = np.meshgrid(xs, xs, indexing="xy")
    NL2 = np.stack([X.ravel(), Y.ravel()])
    rows = []
    for j in range(n):
        for i in range(n):
            b0 = 2 * j * m1 + 2 * i + 1
            c = [b0, b0 + 2, b0 + 2 * m1 + 2, b0 + 2 * m1, b0 + 1, b0 + m1 + 2, b0 + 2 * m1 + 1, b0 + m1,
                 b0 + m1 + 1]
            rows.append(c)
    IEN2 = np.array(rows, dtype=np.int64)
    bnd2 = np.flatnonzero(np.any((NL2 == 0) | (NL2 == 1), axis=0)) + 1
    cases.append((NL2, IEN2, 2, "Q2", bnd2, np.cos(2 * NL2[0, bnd2 - 1]) + NL2[1, bnd2 - 1] ** 2, n))
    with sfem.Server(cluster=2, rtol=1e-12) as srv:
        ids = [srv.submit(NLc, IENc, None, 1.0, 0.3, b_, v_, ndim=nd, nDof=1, FunctionClass=fc)
               for NLc, IENc, nd, fc, b_, v_, _ in cases]
        outs = [srv.wait(i, timeout_ms=60000) for i in ids]
    for (NLc, IENc, nd, fc, b_, v_, ne), (u, res) in zip(cases, outs):
        assert res["status"] == 0
        K = sfem.assemble_system(ne, NLc, IENc, nd, fc, 1, ctx=ctx, as_handle=True)
        ref = K.solve(b_, v_, rtol=1e-13)[0]
        K.close()
        assert _rel(u, ref) <= TOL_U, fc


@pytest.mark.timeout(300)
def test_mixed_classes_in_one_stream(sfem, ctx):
    """2D and 3D requests interleaved on one server, each matching its own solve."""
    mg = sfem.meshgen
    probs = []
    for k, n in enumerate((6, 4, 21, 5, 13, 3)):
        if k % 2:
            probs.append(mg.hex_problem(n, 90 + n, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes"))
        else:
            probs.append(_quads([n], seed=60 + n, e_sigma=0.4)[0])
    with _server(sfem) as srv:
        ids = [_submit(srv, p) for p in probs]
        outs = [srv.wait(i, timeout_ms=60000) for i in ids]
    for p, (u, res) in zip(probs, outs):
        assert res["status"] == 0
        assert _rel(u, _single(sfem, ctx, p)) <= TOL_U, p.name


@pytest.mark.timeout(300)
def test_warm_start_state_per_topology(sfem, ctx):
    """With warm starts a request starts from the last solution served on its
    topology key: a repeated request needs no iteration, a nearby one fewer;
    every result stays within the tolerance of its own single-mesh solve."""
    mg = sfem.meshgen
    p = mg.quad_problem(40, 77, jitter=0.15, nu_range=(0.2, 0.45), e_sigma=0.3, plane="strain")
    q = mg.quad_problem(40, 77, jitter=0.15, nu_range=(0.2, 0.45), e_sigma=0.3, plane="strain")
    q.Young = p.Young * 1.02                                   # same mesh and loads, stiffer material
    q.fixed_vals = p.fixed_vals * 1.05
    with _server(sfem, warm_start=True) as srv:
        cold = srv.wait(_submit(srv, p, key=40), timeout_ms=60000)
        again = srv.wait(_submit(srv, p, key=40, with_ien=False), timeout_ms=60000)
        near = srv.wait(_submit(srv, q, key=40, with_ien=False), timeout_ms=60000)
    ref_p, ref_q = _single(sfem, ctx, p), _single(sfem, ctx, q)
    assert cold[1]["status"] == 0 and again[1]["status"] == 0 and near[1]["status"] == 0
    assert again[1]["iterations"] == 0 and near[1]["iterations"] < cold[1]["iterations"]
    assert _rel(cold[0], ref_p) <= TOL_U and _rel(again[0], ref_p) <= TOL_U and _rel(near[0], ref_q) <= TOL_U
    with _server(sfem) as srv:                                  # off: repeats are bitwise identical
        a = srv.wait(_submit(srv, p, key=40), timeout_ms=60000)
        b = srv.wait(_submit(srv, p, key=40, with_ien=False), timeout_ms=60000)
    assert np.array_equal(a[0], b[0]) and a[1]["iterations"] == b[1]["iterations"] == cold[1]["iterations"]


@pytest.mark.timeout(300)
def test_errors_and_shutdown_with_work_outstanding(sfem, ctx):
    probs = _quads([6, 10], seed=2)
    with _server(sfem) as srv:
        bad = srv.submit(probs[0].NodeList, probs[0].IEN, probs[0].ID, 1.0, 0.3,
                         np.array([10 ** 6]), np.zeros(1), plane="strain")
        good = _submit(srv, probs[1])
        _, rb = srv.wait(bad, timeout_ms=60000)
        ug, rg = srv.wait(good, timeout_ms=60000)
        assert rb["status"] == 2 and rg["status"] == 0      # the bad request alone fails
        with pytest.raises(sfem.SfemError):
            srv.submit(probs[0].NodeList, None, None, 1.0, 0.3, [], [], topology_key=77)
        with pytest.raises(sfem.SfemError):                  # elasticity with nDof 3 in 2D
            srv.submit(probs[0].NodeList, probs[0].IEN, probs[0].ID, 1.0, 0.3, [], [], nDof=3)
    srv = _server(sfem)
    for _ in range(3):
        for p in _quads([40, 50, 60], seed=4):
            _submit(srv, p)
    t0 = time.time()
    srv.close()                                            # in-flight ones finish, the rest are dropped
    assert time.time() - t0 < 60
