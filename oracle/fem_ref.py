"""CPU oracle for the smearFEM.jl hot path -- TEST INFRASTRUCTURE ONLY.

This module is a faithful NumPy restatement of the reference's Julia code.
Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU-baseline leg of
``bench.py`` may use it, and always as the checker: the GPU product never
imports it and has no CPU fallback through it.

What it restates (reference paths are relative to the smearFEM.jl project):

  gaussian_quadrature     src/fem.jl:21-31
  basis_function          src/fem.jl:48-114   (Q1 1D/2D/3D, Q2 2D)
  assemble_system         src/fem.jl:135-256  (COO triplets, ``V[inz] +=`` per
                                               Gauss point, then ``sparse``)
  julia_sparse            ``SparseArrays.sparse(I,J,V)`` as called at
                          src/fem.jl:253: duplicates folded left in input
                          order, explicit zeros kept, rows sorted per column,
                          size ``maximum(I) x maximum(J)``
  meshgrid_loops          examples/vector3D.jl:10-130
  set_boundary_cond       examples/vector3D.jl:133-173
  solve_eliminated        examples/vector3D.jl:315-322 (dense ``inv`` of
                          ``K_free = C' K C``, ``q = q_d + C q_f``)
  apply_boundary_conditions_loops
                          examples/vector3D.jl:175-264 (surface penalty b)
  add_scaled              examples/vector3D.jl:308 (K_bar = K + beta*b)
  inflate_sphere          src/PostProcess.jl:30-44

Parity pinning.  ``gaussian_quadrature`` and ``basis_function`` are pinned by
the reference's own known-answer tests (test/runtests.jl:15-35; restated in
tests/test_oracle.py).  The reference ships no assembly or solve fixture and
its Julia code cannot run in this environment (no Julia toolchain), so the
assembled K and the displacement u are pinned only by analytic known answers
(unit-square Laplace element, closed-form plane-stress element, rigid-body
null space, linear patch test).  Beyond those the K/u parity is unpinned.

Julia's ``det``/``inv`` of a small Float64 matrix go through LAPACK LU, and so
do NumPy's; the matrix products may round differently from OpenBLAS.  Results
therefore agree with the reference to rounding (~1e-16 relative), which is far
inside the 1e-12 (K) and 1e-8 (u) tolerances used by the parity tests.
"""
from __future__ import annotations

import math

import numpy as np

# --------------------------------------------------------------------------
# src/fem.jl:21-31
# --------------------------------------------------------------------------


def gaussian_quadrature(a, b, nGaussPoints=2):
    """Gauss-Legendre nodes and weights on [a, b] (src/fem.jl:21-31).

    The expressions are evaluated exactly as written in the reference so the
    known-answer test ``gaussian_quadrature(-1,1,2) == ([-1/sqrt3, 1/sqrt3],
    [1,1])`` (test/runtests.jl:34) holds bit for bit.
    """
    if nGaussPoints == 2:
        xi = [-(b - a) / (2 * math.sqrt(3)) + (b + a) / 2,
              (b - a) / (2 * math.sqrt(3)) + (b + a) / 2]
        w = [(b - a) / 2, (b - a) / 2]
    elif nGaussPoints == 3:
        xi = [-(b - a) / (2 * math.sqrt(5 / 3)) + (b + a) / 2, 0.0,
              (b - a) / (2 * math.sqrt(5 / 3)) + (b + a) / 2]
        w = [(b - a) / 2 * 5 / 9, (b - a) / 2 * 8 / 9, (b - a) / 2 * 5 / 9]
    else:
        raise ValueError("nGaussPoints must be 2 or 3")
    return np.array(xi, dtype=np.float64), np.array(w, dtype=np.float64)


# --------------------------------------------------------------------------
# src/fem.jl:48-114
# --------------------------------------------------------------------------


def basis_function(xi, eta=None, zeta=None, FunctionClass="Q1"):
    """Shape functions N and reference gradients dN (src/fem.jl:48-114).

    Returns ``(N, dN)`` with ``dN`` of shape (nen, ndim) -- column k is
    dN/d(xi_k), the reference's ``hcat`` layout.  1D returns the 1x2 row the
    reference returns (src/fem.jl:75), which is what breaks 1D assembly.
    """
    if FunctionClass == "Q1":
        if zeta is not None:
            x, y, z = xi, eta, zeta
            N = [(1 - x) * (1 - y) * (1 - z) / 8,
                 (1 + x) * (1 - y) * (1 - z) / 8,
                 (1 + x) * (1 + y) * (1 - z) / 8,
                 (1 - x) * (1 + y) * (1 - z) / 8,
                 (1 - x) * (1 - y) * (1 + z) / 8,
                 (1 + x) * (1 - y) * (1 + z) / 8,
                 (1 + x) * (1 + y) * (1 + z) / 8,
                 (1 - x) * (1 + y) * (1 + z) / 8]
            dx = [-(1 - y) * (1 - z) / 8, (1 - y) * (1 - z) / 8,
                  (1 + y) * (1 - z) / 8, -(1 + y) * (1 - z) / 8,
                  -(1 - y) * (1 + z) / 8, (1 - y) * (1 + z) / 8,
                  (1 + y) * (1 + z) / 8, -(1 + y) * (1 + z) / 8]
            dy = [-(1 - x) * (1 - z) / 8, -(1 + x) * (1 - z) / 8,
                  (1 + x) * (1 - z) / 8, (1 - x) * (1 - z) / 8,
                  -(1 - x) * (1 + z) / 8, -(1 + x) * (1 + z) / 8,
                  (1 + x) * (1 + z) / 8, (1 - x) * (1 + z) / 8]
            dz = [-(1 - x) * (1 - y) / 8, -(1 + x) * (1 - y) / 8,
                  -(1 + x) * (1 + y) / 8, -(1 - x) * (1 + y) / 8,
                  (1 - x) * (1 - y) / 8, (1 + x) * (1 - y) / 8,
                  (1 + x) * (1 + y) / 8, (1 - x) * (1 + y) / 8]
            dN = np.array([dx, dy, dz], dtype=np.float64).T
        elif eta is not None:
            x, y = xi, eta
            N = [(1 - x) * (1 - y) / 4, (x + 1) * (1 - y) / 4,
                 (1 + x) * (y + 1) / 4, (1 - x) * (1 + y) / 4]
            dx = [-(1 - y) / 4, (1 - y) / 4, (y + 1) / 4, -(1 + y) / 4]
            dy = [-(1 - x) / 4, -(x + 1) / 4, (1 + x) / 4, (1 - x) / 4]
            dN = np.array([dx, dy], dtype=np.float64).T
        else:
            N = [0.5 - 0.5 * xi, 0.5 + 0.5 * xi]
            dN = np.array([[-0.5, 0.5]], dtype=np.float64)
        return np.array(N, dtype=np.float64), dN
    if FunctionClass == "Q2":
        if eta is None:
            raise ValueError("Q2 is defined for 2D only (src/fem.jl:77-111)")
        x, y = xi, eta
        N = [(1 - x) * x * (1 - y) * y / 4,
             -x * (1 + x) * (1 - y) * y / 4,
             x * (1 + x) * y * (1 + y) / 4,
             -(1 - x) * x * y * (1 + y) / 4,
             -(1 - x) * (1 + x) * (1 - y) * y / 2,
             x * (1 + x) * (1 - y) * (1 + y) / 2,
             (1 - x) * (1 + x) * y * (1 + y) / 2,
             -(1 - x) * x * (1 - y) * (1 + y) / 2,
             (1 - x) * (1 + x) * (1 - y) * (1 + y)]
        dx = [(1 - 2 * x) * (1 - y) * y / 4,
              -(1 + 2 * x) * (1 - y) * y / 4,
              (1 + 2 * x) * y * (1 + y) / 4,
              -(1 - 2 * x) * y * (1 + y) / 4,
              x * (1 - y) * y,
              (1 + 2 * x) * (1 - y) * (1 + y) / 2,
              -x * y * (1 + y),
              -(1 - 2 * x) * (1 - y) * (1 + y) / 2,
              -2 * x * (1 - y) * (1 + y)]
        dy = [(1 - x) * x * (1 - 2 * y) / 4,
              -x * (1 + x) * (1 - 2 * y) / 4,
              x * (1 + x) * (1 + 2 * y) / 4,
              -(1 - x) * x * (1 + 2 * y) / 4,
              -(1 - x) * (1 + x) * (1 - 2 * y) / 2,
              -x * (1 + x) * y,
              (1 - x) * (1 + x) * (1 + 2 * y) / 2,
              (1 - x) * x * y,
              -(1 - x) * (1 + x) * 2 * y]
        return (np.array(N, dtype=np.float64),
                np.array([dx, dy], dtype=np.float64).T)
    raise ValueError("FunctionClass must be 'Q1' or 'Q2'")


def gauss_tables(ndim):
    """Gauss points and weights in the reference's order (src/fem.jl:149-177).

    Points run counter-clockwise in (xi, eta): (-,-), (+,-), (+,+), (-,+),
    first at zeta = -1/sqrt3 and then at zeta = +1/sqrt3 in 3D.
    """
    xi, w = gaussian_quadrature(-1, 1)
    if ndim == 1:
        return np.array([[xi[0]], [xi[1]]]), np.array([w[0], w[1]])
    if ndim == 2:
        wp = [w[0] * w[0], w[1] * w[0], w[1] * w[1], w[0] * w[1]]
        x = [xi[0], xi[1], xi[1], xi[0]]
        y = [xi[0], xi[0], xi[1], xi[1]]
        return np.array([x, y]).T, np.array(wp)
    wp = [w[0] * w[0] * w[0], w[1] * w[0] * w[0], w[1] * w[1] * w[0],
          w[0] * w[1] * w[0], w[0] * w[0] * w[1], w[1] * w[0] * w[1],
          w[1] * w[1] * w[1], w[0] * w[1] * w[1]]
    x = [xi[0], xi[1], xi[1], xi[0], xi[0], xi[1], xi[1], xi[0]]
    y = [xi[0], xi[0], xi[1], xi[1], xi[0], xi[0], xi[1], xi[1]]
    z = [xi[0], xi[0], xi[0], xi[0], xi[1], xi[1], xi[1], xi[1]]
    return np.array([x, y, z]).T, np.array(wp)


def constitutive_matrix(ndim, Young, nu, plane="stress"):
    """Constitutive matrix D of src/fem.jl:217 (2D) and :230 (3D).

    The reference's 2D matrix is plane stress.  ``plane="strain"`` is this
    project's extension: the 3D matrix restricted to the [xx, yy, xy] rows and
    columns.
    """
    if ndim == 2:
        if plane == "stress":
            return np.array([[Young / (1 - nu ** 2), nu * Young / (1 - nu ** 2), 0.0],
                             [nu * Young / (1 - nu ** 2), Young / (1 - nu ** 2), 0.0],
                             [0.0, 0.0, Young / (2 * (1 + nu))]])
        c = Young / ((1 + nu) * (1 - 2 * nu))
        return np.array([[1 - nu, nu, 0.0], [nu, 1 - nu, 0.0],
                         [0.0, 0.0, (1 - 2 * nu) / 2]]) * c
    return np.array([[1 - nu, nu, nu, 0, 0, 0],
                     [nu, 1 - nu, nu, 0, 0, 0],
                     [nu, nu, 1 - nu, 0, 0, 0],
                     [0, 0, 0, (1 - 2 * nu) / 2, 0, 0],
                     [0, 0, 0, 0, (1 - 2 * nu) / 2, 0],
                     [0, 0, 0, 0, 0, (1 - 2 * nu) / 2]],
                    dtype=np.float64) * (Young / ((1 + nu) * (1 - 2 * nu)))


def strain_displacement(dNdX, nDof):
    """B matrix of src/fem.jl:211-228 (DOFs interleaved per node)."""
    nen = dNdX.shape[0]
    if nDof == 2:
        B = np.zeros((3, 2 * nen))
        B[0, 0::2] = dNdX[:, 0]
        B[1, 1::2] = dNdX[:, 1]
        B[2, 0::2] = dNdX[:, 1]
        B[2, 1::2] = dNdX[:, 0]
        return B
    B = np.zeros((6, 3 * nen))
    B[0, 0::3] = dNdX[:, 0]
    B[1, 1::3] = dNdX[:, 1]
    B[2, 2::3] = dNdX[:, 2]
    B[3, 1::3] = dNdX[:, 2]
    B[3, 2::3] = dNdX[:, 1]
    B[4, 0::3] = dNdX[:, 2]
    B[4, 2::3] = dNdX[:, 0]
    B[5, 0::3] = dNdX[:, 1]
    B[5, 1::3] = dNdX[:, 0]
    return B


# --------------------------------------------------------------------------
# SparseArrays.sparse(I, J, V) as used at src/fem.jl:253
# --------------------------------------------------------------------------


def julia_sparse(I, J, V, m=None, n=None):
    """COO -> CSC with Julia's ``sparse`` semantics.

    * size ``maximum(I) x maximum(J)`` unless given,
    * duplicates combined with ``+`` as a left fold in input order
      (``SparseArrays.sparse!`` compresses each row in input order),
    * explicit zeros kept as stored entries,
    * row indices sorted inside each column.

    Returns 1-based ``(colptr, rowval, nzval, m, n)`` like ``SparseMatrixCSC``.
    """
    I = np.asarray(I, dtype=np.int64)
    J = np.asarray(J, dtype=np.int64)
    V = np.asarray(V, dtype=np.float64)
    if I.size == 0:
        m = 0 if m is None else m
        n = 0 if n is None else n
        return (np.ones(n + 1, np.int64), np.zeros(0, np.int64),
                np.zeros(0, np.float64), m, n)
    if I.min() < 1 or J.min() < 1:
        raise IndexError("row and column indices must be >= 1")
    m = int(I.max()) if m is None else m
    n = int(J.max()) if n is None else n
    key = (J - 1) * m + (I - 1)
    order = np.argsort(key, kind="stable")          # keeps input order among duplicates
    ks = key[order]
    vs = V[order]
    first = np.r_[True, ks[1:] != ks[:-1]]
    seg = np.cumsum(first) - 1
    starts = np.flatnonzero(first)
    pos = np.arange(ks.size) - starts[seg]
    acc = np.zeros(starts.size)
    for k in range(int(pos.max()) + 1):             # left fold: ((v1 + v2) + v3) + ...
        sel = pos == k
        acc[seg[sel]] += vs[sel]
    uk = ks[starts]
    cols = uk // m
    rows = uk % m
    colptr = np.zeros(n + 1, np.int64)
    np.add.at(colptr, cols + 1, 1)
    colptr = np.cumsum(colptr) + 1
    return colptr, rows + 1, acc, m, n


# --------------------------------------------------------------------------
# src/fem.jl:135-256
# --------------------------------------------------------------------------


def _element_count(ne, ndim):
    # src/fem.jl:139-145,179: the element loop runs over 1:ne^ndim, not size(IEN,1)
    return int(ne) ** int(ndim)


def assemble_system_loops(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1,
                          ID=None, Young=1, nu=0.3, plane="stress"):
    """Line-by-line restatement of ``assemble_system`` (src/fem.jl:135-256).

    Pure-Python loops: use on small meshes only.  ``NodeList`` is (ndim, nN),
    ``IEN`` (nEl, nen) and ``ID`` (nN, nDof), all with the reference's 1-based
    indices.  ``Young``/``nu`` may be scalars or per-element arrays (per-
    element values extend the reference, which takes scalars).
    """
    NodeList = np.asarray(NodeList, dtype=np.float64)
    IEN = np.asarray(IEN, dtype=np.int64)
    if ndim == 1:
        raise ValueError("1D assembly is broken in the reference "
                         "(coords*dN dimension mismatch, src/fem.jl:75,192)")
    nEl = _element_count(ne, ndim)
    if IEN.shape[0] < nEl:
        raise IndexError("IEN has fewer rows than ne^ndim")
    Ys = np.broadcast_to(np.asarray(Young, dtype=np.float64), (nEl,)) if np.ndim(Young) else None
    nus = np.broadcast_to(np.asarray(nu, dtype=np.float64), (nEl,)) if np.ndim(nu) else None
    if nDof == 1:
        L = nEl * IEN.shape[1] ** 2
    else:
        ID = np.asarray(ID, dtype=np.int64)
        L = nEl * (ID.shape[1] * 2 ** ndim) ** 2
    E = np.zeros(L, np.int64)
    J = np.zeros(L, np.int64)
    V = np.zeros(L, np.float64)
    pts, wpoints = gauss_tables(ndim)
    for e in range(nEl):
        coords = NodeList[:, IEN[e, :] - 1]
        Ye = Young if Ys is None else Ys[e]
        nue = nu if nus is None else nus[e]
        for gp in range(2 ** ndim):
            if ndim == 2:
                N, dN = basis_function(pts[gp, 0], pts[gp, 1], None, FunctionClass)
            else:
                N, dN = basis_function(pts[gp, 0], pts[gp, 1], pts[gp, 2], FunctionClass)
            Jac = coords @ dN
            w = wpoints[gp] * abs(np.linalg.det(Jac))
            invJ = np.linalg.inv(Jac)
            dNdX = dN @ invJ
            if nDof == 1:
                szN = N.shape[0]
                for i in range(szN):
                    for j in range(szN):
                        inz = szN * szN * e + szN * i + j
                        E[inz] = IEN[e, i]
                        J[inz] = IEN[e, j]
                        V[inz] += w * np.dot(dNdX[i, :], dNdX[j, :])
            else:
                B = strain_displacement(dNdX, nDof)
                cMat = constitutive_matrix(ndim, Ye, nue, plane)
                Ke = ((B.T @ cMat) @ B) * w
                nk = Ke.shape[0]
                for iNode in range(nk // nDof):
                    for jNode in range(nk // nDof):
                        for iDof in range(ID.shape[1]):
                            for jDof in range(ID.shape[1]):
                                i = iNode * nDof + iDof
                                j = jNode * nDof + jDof
                                inz = (Ke.size * e + iNode * nDof * nk
                                       + jNode * nDof * nDof + iDof * nDof + jDof)
                                E[inz] = ID[IEN[e, iNode] - 1, iDof]
                                J[inz] = ID[IEN[e, jNode] - 1, jDof]
                                V[inz] += Ke[i, j]
    return julia_sparse(E, J, V)


def assemble_system(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1,
                    ID=None, Young=1, nu=0.3, plane="stress"):
    """Element-vectorised restatement of ``assemble_system`` (src/fem.jl:135-256).

    Same arithmetic per element and Gauss point as the loop form: ``Jac =
    coords*dN``, ``w = wgp*|det Jac|``, ``dNdX = dN*inv(Jac)``, ``Ke =
    ((B'*D)*B)*w`` accumulated into the element's COO slots in Gauss-point
    order, COO index layout of src/fem.jl:203,242, then ``julia_sparse``.
    Returns 1-based ``(colptr, rowval, nzval, m, n)``.
    """
    NodeList = np.asarray(NodeList, dtype=np.float64)
    IEN = np.asarray(IEN, dtype=np.int64)
    if ndim == 1:
        raise ValueError("1D assembly is broken in the reference "
                         "(coords*dN dimension mismatch, src/fem.jl:75,192)")
    nEl = _element_count(ne, ndim)
    if IEN.shape[0] < nEl:
        raise IndexError("IEN has fewer rows than ne^ndim")
    if nEl == 0:
        return julia_sparse([], [], [])
    ien = IEN[:nEl] - 1
    nen = ien.shape[1]
    coords = np.transpose(NodeList[:, ien], (1, 0, 2))        # (nEl, ndim, nen)
    pts, wpoints = gauss_tables(ndim)
    Y = np.broadcast_to(np.asarray(Young, dtype=np.float64), (nEl,))
    NU = np.broadcast_to(np.asarray(nu, dtype=np.float64), (nEl,))
    if nDof == 1:
        Vloc = np.zeros((nEl, nen, nen))
    else:
        if nDof != ndim:
            raise ValueError("vector assembly needs nDof == ndim (src/fem.jl:210-231)")
        nk = nDof * nen
        Vloc = np.zeros((nEl, nk, nk))
        if Young is not None and np.ndim(Young) == 0 and np.ndim(nu) == 0:
            Ds = constitutive_matrix(ndim, float(Young), float(nu), plane)[None]
        else:
            Ds = np.stack([constitutive_matrix(ndim, Y[e], NU[e], plane) for e in range(nEl)])
    for gp in range(2 ** ndim):
        if ndim == 2:
            N, dN = basis_function(pts[gp, 0], pts[gp, 1], None, FunctionClass)
        else:
            N, dN = basis_function(pts[gp, 0], pts[gp, 1], pts[gp, 2], FunctionClass)
        Jac = coords @ dN                                      # (nEl, ndim, ndim)
        w = wpoints[gp] * np.abs(np.linalg.det(Jac))
        invJ = np.linalg.inv(Jac)
        dNdX = dN[None] @ invJ                                 # (nEl, nen, ndim)
        if nDof == 1:
            Vloc += w[:, None, None] * np.einsum("eik,ejk->eij", dNdX, dNdX)
        else:
            B = np.zeros((nEl, 3 if nDof == 2 else 6, nk))
            if nDof == 2:
                B[:, 0, 0::2] = dNdX[:, :, 0]
                B[:, 1, 1::2] = dNdX[:, :, 1]
                B[:, 2, 0::2] = dNdX[:, :, 1]
                B[:, 2, 1::2] = dNdX[:, :, 0]
            else:
                B[:, 0, 0::3] = dNdX[:, :, 0]
                B[:, 1, 1::3] = dNdX[:, :, 1]
                B[:, 2, 2::3] = dNdX[:, :, 2]
                B[:, 3, 1::3] = dNdX[:, :, 2]
                B[:, 3, 2::3] = dNdX[:, :, 1]
                B[:, 4, 0::3] = dNdX[:, :, 2]
                B[:, 4, 2::3] = dNdX[:, :, 0]
                B[:, 5, 0::3] = dNdX[:, :, 1]
                B[:, 5, 1::3] = dNdX[:, :, 0]
            Vloc += ((np.transpose(B, (0, 2, 1)) @ Ds) @ B) * w[:, None, None]
    if nDof == 1:
        rows = np.repeat(IEN[:nEl], nen, axis=1)               # E[inz] = IEN[e,i]
        cols = np.tile(IEN[:nEl], (1, nen))                    # J[inz] = IEN[e,j]
        return julia_sparse(rows.ravel(), cols.ravel(), Vloc.ravel())
    ID = np.asarray(ID, dtype=np.int64)
    # COO order (iNode, jNode, iDof, jDof) of src/fem.jl:242
    V4 = Vloc.reshape(nEl, nen, nDof, nen, nDof).transpose(0, 1, 3, 2, 4)
    dof = ID[ien]                                              # (nEl, nen, nDof)
    R = np.broadcast_to(dof[:, :, None, :, None], (nEl, nen, nen, nDof, nDof))
    C = np.broadcast_to(dof[:, None, :, None, :], (nEl, nen, nen, nDof, nDof))
    return julia_sparse(R.ravel(), C.ravel(), V4.ravel())


def csc_to_dense(colptr, rowval, nzval, m, n):
    A = np.zeros((m, n))
    for j in range(n):
        for k in range(colptr[j] - 1, colptr[j + 1] - 1):
            A[rowval[k] - 1, j] += nzval[k]
    return A


def csc_to_scipy(colptr, rowval, nzval, m, n):
    import scipy.sparse as sp
    return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=(m, n))


# --------------------------------------------------------------------------
# examples/vector3D.jl:10-130
# --------------------------------------------------------------------------


def meshgrid_loops(x0, x1, y0, y1, z0, z1, ne, ndim):
    """Loop restatement of ``meshgrid`` (examples/vector3D.jl:10-130).

    Returns ``NodeList (ndim, nN)``, ``IEN (ne^ndim, 2^ndim)``, ``ID (nN,
    ndim)`` (interleaved: ID[m,l] = ndim*(m-1)+l), ``IEN_top``, ``IEN_btm``,
    all 1-based.
    """
    nN = (ne + 1) ** ndim
    NodeList = np.zeros((ndim, nN))
    IEN = np.zeros((ne ** ndim, 2 ** ndim), np.int64)
    IEN_top = np.zeros((ne ** (ndim - 1), 2 ** (ndim - 1)), np.int64)
    IEN_btm = np.zeros((ne ** (ndim - 1), 2 ** (ndim - 1)), np.int64)
    ID = np.zeros((nN, ndim), np.int64)
    x = np.linspace(x0, x1, ne + 1)
    y = np.linspace(y0, y1, ne + 1)
    if ndim == 2:
        m = 1
        for j in range(1, ne + 2):
            for i in range(1, ne + 2):
                NodeList[0, m - 1] = x[i - 1]
                NodeList[1, m - 1] = y[j - 1]
                for l in range(1, ndim + 1):
                    ID[m - 1, l - 1] = ndim * (m - 1) + l
                m += 1
        n = 1
        for j in range(1, ne + 1):
            for i in range(1, ne + 1):
                IEN[n - 1] = [(j - 1) * (ne + 1) + i, (j - 1) * (ne + 1) + i + 1,
                              j * (ne + 1) + i + 1, j * (ne + 1) + i]
                if j == 1:
                    IEN_btm[i - 1] = IEN[n - 1, [0, 1]]
                elif j == ne:
                    IEN_top[i - 1] = IEN[n - 1, [3, 2]]
                n += 1
        return NodeList, IEN, ID, IEN_top, IEN_btm
    z = np.linspace(z0, z1, ne + 1)
    m = 1
    for k in range(1, ne + 2):
        for j in range(1, ne + 2):
            for i in range(1, ne + 2):
                NodeList[:, m - 1] = [x[i - 1], y[j - 1], z[k - 1]]
                for l in range(1, ndim + 1):
                    ID[m - 1, l - 1] = ndim * (m - 1) + l
                m += 1
    n = nt = nb = 1
    p = (ne + 1) ** 2
    for k in range(1, ne + 1):
        for j in range(1, ne + 1):
            for i in range(1, ne + 1):
                IEN[n - 1] = [(k - 1) * p + (j - 1) * (ne + 1) + i,
                              (k - 1) * p + (j - 1) * (ne + 1) + i + 1,
                              (k - 1) * p + j * (ne + 1) + i + 1,
                              (k - 1) * p + j * (ne + 1) + i,
                              k * p + (j - 1) * (ne + 1) + i,
                              k * p + (j - 1) * (ne + 1) + i + 1,
                              k * p + j * (ne + 1) + i + 1,
                              k * p + j * (ne + 1) + i]
                if k == 1:
                    IEN_btm[nb - 1] = IEN[n - 1, :4]
                    nb += 1
                elif k == ne:
                    IEN_top[nt - 1] = IEN[n - 1, 4:]
                    nt += 1
                n += 1
    return NodeList, IEN, ID, IEN_top, IEN_btm


# --------------------------------------------------------------------------
# examples/vector3D.jl:133-173 and :315-322
# --------------------------------------------------------------------------


def set_boundary_cond(NodeList, ne, ndim, d, nDof=1):
    """``setboundaryCond`` for Q1 (examples/vector3D.jl:133-173).

    z-DOF of every node with ``z == 0`` is fixed to 0 and of every node with
    ``z == 1`` to ``-d`` (exact float compares, :161,:164).  Returns ``q_d``
    (length nDof*(ne+1)^ndim) and the 1-based list of constrained DOFs
    (``rCol``); ``C = I[:, setdiff(1:n, rCol)]``.
    """
    n = nDof * (ne + 1) ** ndim
    q_d = np.zeros(n)
    rcol = []
    for nNode in range(1, NodeList.shape[1] + 1):
        coord = NodeList[:, nNode - 1]
        if coord[2] == 0:
            q_d[3 * nNode - 1] = 0
            rcol.append(3 * nNode)
        elif coord[2] == 1:
            q_d[3 * nNode - 1] = -d
            rcol.append(3 * nNode)
    return q_d, np.array(rcol, dtype=np.int64)


def solve_eliminated(K_csc, fixed_dofs, fixed_vals, f=None, method="inv"):
    """Dirichlet elimination and solve of examples/vector3D.jl:315-322.

    ``K_free = C' K C``; ``q_f = inv(Matrix(K_free)) * C' * (f - K q_d)``;
    ``q = q_d + C q_f``.  The reference has no load vector (f = 0); a given
    ``f`` enters the right-hand side as ``C' f``.  ``method="inv"`` follows
    the reference's dense inverse (O(n_f^3): small/medium systems only);
    ``method="splu"`` is a sparse-direct cross-check for larger systems.
    """
    colptr, rowval, nzval, m, n = K_csc
    K = csc_to_scipy(colptr, rowval, nzval, m, n)
    q_d = np.zeros(n)
    fixed = np.asarray(fixed_dofs, dtype=np.int64) - 1
    q_d[fixed] = np.asarray(fixed_vals, dtype=np.float64)
    free = np.setdiff1d(np.arange(n), fixed)
    rhs = -(K @ q_d)
    if f is not None:
        rhs = rhs + np.asarray(f, dtype=np.float64)
    rhs = rhs[free]
    Kff = K[free][:, free]
    if method == "inv":
        invK = np.linalg.inv(Kff.toarray())
        qf = invK @ rhs
    else:
        import scipy.sparse.linalg as spla
        qf = spla.splu(Kff.tocsc()).solve(rhs)
    q = q_d.copy()
    q[free] += qf
    return q


# --------------------------------------------------------------------------
# examples/vector3D.jl:175-264 (surface penalty), :306-308 (K_bar = K + beta b)
# and src/PostProcess.jl:30-44 (inflate_sphere)
# --------------------------------------------------------------------------


def apply_boundary_conditions_loops(ne, NodeList, IEN, IEN_top, IEN_btm, ndim, FunctionClass="Q1",
                                    ID=None, nDof=3):
    """Line-by-line restatement of ``apply_boundary_conditions``
    (examples/vector3D.jl:175-264): the penalty ("slip") matrix ``b`` of the
    top and bottom surfaces, b = sum over surface quads and their 2x2 Gauss
    points of w |dx/dxi x dx/deta| M'M with M = [N_1 I, ..., N_4 I] (3 x 12).

    COO layout as the reference: bottom faces first (inz_btm), then top faces
    (inz_top), each face a 4x4 grid of 3x3 blocks (iNode, jNode, iDof, jDof);
    ``V[inz] +=`` per Gauss point; then ``sparse``.  Only 3D exists: the 2D
    branch takes ``cross`` of 2-vectors, which the reference cannot evaluate.
    ``IEN`` is unused, as in the reference.
    """
    if ndim != 3:
        raise ValueError("apply_boundary_conditions: the reference's 2D branch calls cross() on "
                         "2-vectors (examples/vector3D.jl:218), so only ndim = 3 is defined")
    NodeList = np.asarray(NodeList, dtype=np.float64)
    IEN_top = np.asarray(IEN_top, dtype=np.int64)
    IEN_btm = np.asarray(IEN_btm, dtype=np.int64)
    ID = np.asarray(ID, dtype=np.int64)
    nface = int(ne) ** (ndim - 1)
    if min(IEN_top[:nface].min(), IEN_btm[:nface].min()) < 1:
        raise IndexError("surface connectivity holds node 0 (the reference's meshgrid leaves "
                         "IEN_top empty when ne = 1)")
    L = nface * (ID.shape[1] * IEN_btm.shape[1]) ** 2 * 2
    E = np.zeros(L, np.int64)
    J = np.zeros(L, np.int64)
    V = np.zeros(L, np.float64)
    xi, w_xi = gaussian_quadrature(-1, 1)
    eta, w_eta = gaussian_quadrature(-1, 1)
    wpoints = [w_xi[0] * w_eta[0], w_xi[1] * w_eta[0], w_xi[1] * w_eta[1], w_xi[0] * w_eta[1]]
    x = [xi[0], xi[1], xi[1], xi[0]]
    y = [eta[0], eta[0], eta[1], eta[1]]
    for e in range(nface):
        coords_top = NodeList[:, IEN_top[e, :] - 1]
        coords_btm = NodeList[:, IEN_btm[e, :] - 1]
        for gp in range(2 ** (ndim - 1)):
            N, dN = basis_function(x[gp], y[gp], None, FunctionClass)
            dx_top = coords_top @ dN
            dx_btm = coords_btm @ dN
            w_top = wpoints[gp] * np.linalg.norm(np.cross(dx_top[:, 0], dx_top[:, 1]))
            w_btm = wpoints[gp] * np.linalg.norm(np.cross(dx_btm[:, 0], dx_btm[:, 1]))
            M = np.zeros((3, ndim * N.shape[0]))
            M[0, 0::nDof] = N
            M[1, 1::nDof] = N
            M[2, 2::nDof] = N
            be = M.T @ M
            nb = be.shape[0]
            for iNode in range(nb // nDof):
                for jNode in range(nb // nDof):
                    for iDof in range(ID.shape[1]):
                        for jDof in range(ID.shape[1]):
                            i = iNode * nDof + iDof
                            j = jNode * nDof + jDof
                            inz_btm = (be.size * e + iNode * nDof * nb + jNode * nDof ** 2
                                       + iDof * nDof + jDof)
                            inz_top = be.size * nface + inz_btm
                            E[inz_top] = ID[IEN_top[e, iNode] - 1, iDof]
                            J[inz_top] = ID[IEN_top[e, jNode] - 1, jDof]
                            V[inz_top] += w_top * be[i, j]
                            E[inz_btm] = ID[IEN_btm[e, iNode] - 1, iDof]
                            J[inz_btm] = ID[IEN_btm[e, jNode] - 1, jDof]
                            V[inz_btm] += w_btm * be[i, j]
    return julia_sparse(E, J, V)


def add_scaled(K_csc, beta, b_csc):
    """``K + beta * b`` for two CSC matrices (examples/vector3D.jl:308) as a
    scipy CSC matrix: each stored entry of ``beta * b`` is rounded once, then
    added to K's entry."""
    K = csc_to_scipy(*K_csc)
    b = csc_to_scipy(*b_csc)
    b.data = beta * b.data
    if b.shape != K.shape:
        b.resize(K.shape)
    return (K + b).tocsc()


def inflate_sphere(NodeList, x0, x1, y0, y1):
    """``inflate_sphere`` (src/PostProcess.jl:30-44) on a copy: every node's
    (x, y) is moved radially so that the square cross-section becomes a disc
    (scale = max(|dx|, |dy|) about the centre, new radius = scale).  The
    reference mutates its argument; this returns a new array."""
    out = np.array(NodeList, dtype=np.float64, copy=True)
    xc = np.array([0.5 * (x0 + x1), 0.5 * (y0 + y1)])
    for i in range(out.shape[1]):
        d = out[0:2, i] - xc
        scale = np.max(np.abs(d))
        if scale == 0.0:  # Julia's `scale ≈ 0.` (rtol sqrt(eps), atol 0) holds only for exact 0
            out[0:2, i] = [0.0, 0.0]
        else:
            r = math.sqrt((out[0, i] - xc[0]) ** 2 + (out[1, i] - xc[1]) ** 2)
            out[0:2, i] = scale * (out[0:2, i] - xc) / r
    return out
