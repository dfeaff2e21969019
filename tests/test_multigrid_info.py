"""CPU: which meshes the multigrid preconditioner builds a hierarchy for, and
its size (sfem_multigrid_info, host only).  The structured-grid check
accepts exactly the reference's meshgrid connectivity; the level count and
the device bytes follow the hierarchy's rules, restated here."""
import numpy as np
import pytest


def _levels(ne):
    if ne < 3:
        return 0
    L, n = 1, ne
    while n > 2:
        n = (n + 1) // 2
        L += 1
    return L


def _bytes(ndim, b, ne):
    """The hierarchy's device layout: its record, then per level the smoother
    and two vectors (level >= 1: also the stencil blocks, free flags and the
    right-hand side), then the coarsest inverse and Gauss-Jordan scratch,
    every array 256-byte aligned."""
    L = _levels(ne)
    off = 0

    def take(nbytes):
        nonlocal off
        off = (off + 255) // 256 * 256
        off += max(nbytes, 1)

    take(8 + 12 * 56 + 16)  # MgMesh: nlev, ndc, 12 levels of 56 bytes, two pointers
    S = 9 if ndim == 2 else 27
    nn0 = (ne + 1) ** ndim
    ndp = (nn0 + 31) // 32 * 32 * b
    n, ndc = ne, 0
    for lvl in range(L):
        nn = (n + 1) ** ndim
        nd = ndp if lvl == 0 else nn * b
        take(4 * nn * b * b)
        take(4 * nd)
        take(4 * nd)
        if lvl > 0:
            take(4 * S * b * b * ((nn + 31) // 32 * 32))  # stencil blocks in tiles of 32 nodes
            take(nn * b)
            take(4 * nd)
        if lvl == L - 1:
            ndc = nn * b
        n = (n + 1) // 2
    take(4 * ndc * ndc)
    take(16 * ndc * ndc)
    return off


@pytest.mark.parametrize("ndim,ne", [(2, 33), (2, 64), (3, 12), (3, 5)])
def test_meshgrid_meshes_get_a_hierarchy(sfem, ndim, ne):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1 if ndim == 3 else 0, ne, ndim)
    info = sfem.multigrid_info(NL.shape[1], IEN, ndim)
    assert info == {"ne": ne, "levels": _levels(ne), "bytes": _bytes(ndim, ndim, ne)}
    scalar = sfem.multigrid_info(NL.shape[1], IEN, ndim, nDof=1)
    assert scalar["levels"] == info["levels"] and 0 < scalar["bytes"] < info["bytes"]
    assert scalar["bytes"] == _bytes(ndim, 1, ne)


def test_other_meshes_get_none(sfem):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 0, 20, 2)
    perm = np.random.default_rng(0).permutation(IEN.shape[0])
    assert sfem.multigrid_info(NL.shape[1], IEN[perm], 2) == {"ne": 0, "levels": 0, "bytes": 0}
    swapped = IEN.copy()
    swapped[:, [1, 3]] = swapped[:, [3, 1]]  # clockwise node order
    assert sfem.multigrid_info(NL.shape[1], swapped, 2)["ne"] == 0
    assert sfem.multigrid_info(NL.shape[1] + 1, IEN, 2)["ne"] == 0  # node count off the grid
    NL2, IEN2, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, 2, 3)
    assert sfem.multigrid_info(NL2.shape[1], IEN2, 3) == {"ne": 2, "levels": 0, "bytes": 0}  # too small
    q2 = np.ones((4, 9), dtype=np.int64)
    assert sfem.multigrid_info(25, q2, 2, nDof=1, FunctionClass="Q2")["ne"] == 0


def test_bad_arguments_raise(sfem):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 0, 4, 2)
    with pytest.raises(sfem.SfemError):
        sfem.multigrid_info(NL.shape[1], IEN, 1)
    with pytest.raises(sfem.SfemError):
        sfem.multigrid_info(NL.shape[1], IEN, 2, nDof=3)
