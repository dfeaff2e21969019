"""GPU: the on-device mesh generator and inflate_sphere against the oracle's
restatements of examples/vector3D.jl:10-130 and src/PostProcess.jl:30-44.

Index arrays must be identical; coordinates too (the generator rounds like
the linspace the restatement uses), so the boundary planes hold their nodes
exactly.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("ndim,ne", [(2, 1), (2, 7), (3, 1), (3, 5), (3, 12)])
def test_meshgrid_matches_oracle(sfem, ctx, oracle, ndim, ne):
    box = (0.0, 1.0, -0.5, 2.0, 0.25, 1.75)
    got = sfem.meshgrid(*box, ne, ndim, ctx=ctx)
    ref = oracle.meshgrid_loops(*box, ne, ndim)
    for g, r, name in zip(got, ref, ("NodeList", "IEN", "ID", "IEN_top", "IEN_btm")):
        assert g.shape == r.shape, name
        assert np.array_equal(g, r), name


def test_meshgrid_on_device_feeds_assembly(sfem, ctx, oracle):
    """Device-generated inputs go straight into the assembly (no host copy)."""
    import torch
    NL, IEN, ID, IT, IB = sfem.meshgrid(0, 1, 0, 1, 0, 1, 6, 3, device=True, ctx=ctx)
    assert NL.is_cuda and IEN.is_cuda and tuple(NL.shape) == (3, 343)
    K = sfem.assemble_system(6, NL, IEN, 3, "Q1", 3, ID, 40.0, 0.4, ctx=ctx)
    NLh, IENh, IDh, _, _ = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, 6, 3)
    Kh = sfem.assemble_system(6, NLh, IENh, 3, "Q1", 3, IDh, 40.0, 0.4, ctx=ctx)
    assert (K != Kh).nnz == 0
    torch.cuda.synchronize()


def test_inflate_sphere_matches_oracle(sfem, ctx, oracle):
    import torch
    NL, _, _, _, _ = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, 9, 3)
    ref = oracle.inflate_sphere(NL, 0, 1, 0, 1)
    got = sfem.inflate_sphere(NL, 0, 1, 0, 1, ctx=ctx)
    assert np.max(np.abs(got - ref)) <= 1e-15 and np.array_equal(got[2], ref[2])
    assert np.array_equal(NL, oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, 9, 3)[0])   # numpy input untouched
    Xd = sfem.meshgrid(0, 1, 0, 1, 0, 1, 9, 3, device=True, ctx=ctx)[0]
    sfem.inflate_sphere(Xd, 0, 1, 0, 1, ctx=ctx)                                   # in place, like the reference
    assert np.max(np.abs(Xd.cpu().numpy() - ref)) <= 1e-15
    torch.cuda.synchronize()


def test_meshgrid_errors(sfem, ctx):
    with pytest.raises(sfem.SfemError):
        sfem.meshgrid(0, 1, 0, 1, 0, 1, 0, 3, ctx=ctx)
    with pytest.raises(sfem.SfemError):
        sfem.meshgrid(0, 1, 0, 1, 0, 1, 4, 1, ctx=ctx)
