"""GPU: sfem_reassemble_noalloc, the re-assembly entry point that allocates no
device memory, against the allocating sfem_assemble.

It exists for callers that cannot call cudaMalloc/cudaFree when they refresh
K (device memory owned by another allocator under a budget, latency-bound
update loops where cudaFree's device-wide synchronisation stalls other
streams, no-allocation-after-start-up deployments).  Its scratch is a fixed
64 MiB device array shared by every call.  Two calls in a row must each give
exactly what sfem_assemble gives for the same material data; meshes too big
for the array must be refused.  This file is collected last so that a run
stopping at its first failure has already run every other test.
"""
import ctypes as C

import numpy as np
import pytest

from conftest import rowscaled_err

pytestmark = pytest.mark.gpu

TOL_K = 1e-12


def _csc(K):
    colptr, rowval, nzval = K.to_csc_arrays()
    return colptr, rowval, nzval, K.n, K.n


def _noalloc(sfem, ctx, K, young, nu):
    young = np.ascontiguousarray(np.atleast_1d(young), dtype=np.float64)
    nu = np.ascontiguousarray(np.atleast_1d(nu), dtype=np.float64)
    code = sfem.lib().sfem_reassemble_noalloc(ctx.h, K.h, young.ctypes.data, young.size,
                                              nu.ctypes.data, nu.size, 0)
    return code


def test_noalloc_matches_assemble_twice(sfem, ctx):
    p = sfem.meshgen.jittered_cube(ne=14)                      # 2,744 hex elements: fits the 64 MiB array
    m = sfem.Mesh(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, ctx=ctx)
    rng = np.random.default_rng(77)
    mats = [(p.Young, 0.3), (np.exp(rng.normal(0, 1.0, p.n_elem)), rng.uniform(0.25, 0.45, p.n_elem))]
    refs = [_csc(m.assemble(y, v)) for y, v in mats]     # the existing, allocating entry point
    K = m.assemble(np.ones(1), 0.2)                      # the matrix the no-alloc calls overwrite
    for (y, v), ref in zip(mats, refs):                  # two calls in a row, different data
        assert _noalloc(sfem, ctx, K, y, v) == 0, ctx.error()
        got = _csc(K)
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
        assert rowscaled_err(ref, got[2], got[1]) <= TOL_K


def test_noalloc_scalar_and_fp32_copy(sfem, ctx):
    """Laplace (no material data) and the FP32 copy used by mixed solves."""
    ne = 16
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, ne, 2)
    m = sfem.Mesh(ne, NL, IEN, 2, "Q1", 1, ctx=ctx)
    K = m.assemble()
    ref = _csc(K)
    assert sfem.lib().sfem_reassemble_noalloc(ctx.h, K.h, None, 0, None, 0, 0) == 0
    got = _csc(K)
    assert rowscaled_err(ref, got[2], got[1]) <= TOL_K
    p = sfem.meshgen.hex_problem(8, 5, jitter=0.2, e_sigma=0.5, top="modes")
    mh = sfem.Mesh(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, ctx=ctx)
    Kh = mh.assemble(np.ones(1), 0.3)
    Kh.solve(p.fixed_dofs, p.fixed_vals, precision="mixed")          # builds the FP32 copy
    assert _noalloc(sfem, ctx, Kh, p.Young, 0.3) == 0
    u1, _ = Kh.solve(p.fixed_dofs, p.fixed_vals, precision="mixed", rtol=1e-12)
    u2, _ = mh.assemble(p.Young, 0.3).solve(p.fixed_dofs, p.fixed_vals, precision="mixed",
                                             rtol=1e-12)
    assert np.linalg.norm(u1 - u2) <= 1e-8 * np.linalg.norm(u2)


def test_noalloc_refuses_meshes_beyond_its_scratch(sfem, ctx):
    p = sfem.meshgen.jittered_cube(ne=30)                      # 27,000 hex elements > 64 MiB of blocks
    m = sfem.Mesh(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, ctx=ctx)
    K = m.assemble(p.Young, 0.3)
    assert _noalloc(sfem, ctx, K, p.Young, 0.3) == 1     # SFEM_BAD_ARG
    assert "too large" in ctx.error()
    u, st = K.solve(p.fixed_dofs, p.fixed_vals)          # the context and K are untouched
    assert st["status"] == 0
