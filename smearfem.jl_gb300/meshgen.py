"""Structured Q1 meshes and the seeded synthetic workloads.

``meshgrid`` restates ``meshgrid`` of examples/vector3D.jl:10-130 (vectorised):
nodes numbered x fastest, then y, then z; element connectivity ``IEN``
counter-clockwise on the bottom face then the top face (the node order of
``basis_function``, src/fem.jl:53-60); interleaved DOF map ``ID[m,l] =
ndim*(m-1)+l`` (examples/vector3D.jl:73-75).  All indices are 1-based and the
arrays have the reference's shapes: ``NodeList`` (ndim, nN), ``IEN`` (nEl, nen),
``ID`` (nN, ndim).

The workload builders produce the seeded inputs of the five benchmark
workloads (20^3 unit-cube parity case, 128^3 jittered FP64 case, 96^3
high-contrast mixed-precision case, 1024-mesh plane-strain batch, serving
stream).  Every random draw comes from ``numpy.random.default_rng(seed)``.
Boundary nodes are never jittered, so face selection by exact coordinate
compares (examples/vector3D.jl:161,164) stays valid.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def meshgrid(x0, x1, y0, y1, z0, z1, ne, ndim):
    """Vectorised ``meshgrid`` (examples/vector3D.jl:10-130).

    Returns ``(NodeList, IEN, ID, IEN_top, IEN_btm)``.
    """
    ne = int(ne)
    n1 = ne + 1
    x = np.linspace(x0, x1, n1)
    y = np.linspace(y0, y1, n1)
    if ndim == 2:
        X, Y = np.meshgrid(x, y, indexing="xy")               # j (y) outer, i (x) inner
        NodeList = np.stack([X.ravel(), Y.ravel()])
        j, i = np.meshgrid(np.arange(ne), np.arange(ne), indexing="ij")
        base = (j * n1 + i).ravel() + 1
        IEN = np.stack([base, base + 1, base + n1 + 1, base + n1], axis=1).astype(np.int64)
        IEN_btm = IEN[:ne][:, [0, 1]].copy()
        IEN_top = IEN[ne * (ne - 1):][:, [3, 2]].copy()
        if ne == 1:                       # `if j == 1 ... elseif j == ne` never fills the top
            IEN_top[:] = 0
    elif ndim == 3:
        z = np.linspace(z0, z1, n1)
        Z, Y, X = np.meshgrid(z, y, x, indexing="ij")          # k outer, then j, then i
        NodeList = np.stack([X.ravel(), Y.ravel(), Z.ravel()])
        p = n1 * n1
        k, j, i = np.meshgrid(np.arange(ne), np.arange(ne), np.arange(ne), indexing="ij")
        base = (k * p + j * n1 + i).ravel() + 1
        IEN = np.stack([base, base + 1, base + n1 + 1, base + n1,
                        base + p, base + p + 1, base + p + n1 + 1, base + p + n1],
                       axis=1).astype(np.int64)
        IEN_btm = IEN[: ne * ne, :4].copy()
        IEN_top = IEN[ne * ne * (ne - 1):, 4:].copy()
        if ne == 1:                       # `if k == 1 ... elseif k == ne` never fills the top
            IEN_top[:] = 0
    else:
        raise ValueError("ndim must be 2 or 3")
    nN = NodeList.shape[1]
    ID = (ndim * np.arange(nN, dtype=np.int64)[:, None]
          + np.arange(1, ndim + 1, dtype=np.int64)[None, :])
    return NodeList, IEN, ID, IEN_top, IEN_btm


def jitter_interior(NodeList, ne, amp, rng, lo=0.0, hi=1.0):
    """Move every node not on the domain boundary by U(-amp*h, amp*h) per axis."""
    h = (hi - lo) / ne
    interior = np.all((NodeList > lo) & (NodeList < hi), axis=0)
    d = rng.uniform(-amp * h, amp * h, size=(NodeList.shape[0], int(interior.sum())))
    out = NodeList.copy()
    out[:, interior] += d
    return out


@dataclass
class Problem:
    """One assemble-and-solve request: mesh, material, Dirichlet data."""
    name: str
    ndim: int
    ne: int
    NodeList: np.ndarray
    IEN: np.ndarray
    ID: np.ndarray
    Young: np.ndarray
    nu: np.ndarray
    fixed_dofs: np.ndarray            # 1-based global DOF ids
    fixed_vals: np.ndarray
    plane: str = "stress"             # 2D constitutive law: "stress" (reference) or "strain"
    rtol: float = 1e-10
    seed: int = 0
    meta: dict = field(default_factory=dict)

    @property
    def nDof(self):
        return self.ndim

    @property
    def n_nodes(self):
        return self.NodeList.shape[1]

    @property
    def n_dof(self):
        return self.ndim * self.NodeList.shape[1]

    @property
    def n_elem(self):
        return self.ne ** self.ndim


def _face_dofs_3d(NodeList, z, comps):
    nodes = np.flatnonzero(NodeList[2] == z)                   # exact compare, as the reference
    return nodes, np.concatenate([3 * nodes + c + 1 for c in comps])


def hex_problem(ne, seed, jitter=0.0, e_sigma=None, nu=0.3, nu_range=None,
                top="sin", rtol=1e-10, name=None):
    """3D unit-cube elasticity: bottom clamped, top face z-displacement.

    ``top="sin"``: u_z = 0.05 sin(pi x) sin(pi y) (the 20^3 parity case);
    ``top="modes"``: u_z = 0.02 * sum_k a_k sin(p_k pi x) sin(q_k pi y) /
    sum|a_k| with 4 seeded modes.  ``e_sigma`` gives per-element
    E = exp(N(0, e_sigma)); ``nu_range`` per-element nu ~ U(range).
    """
    rng = np.random.default_rng(seed)
    NodeList, IEN, ID, _, _ = meshgrid(0, 1, 0, 1, 0, 1, ne, 3)
    if jitter:
        NodeList = jitter_interior(NodeList, ne, jitter, rng)
    nEl = ne ** 3
    Young = (np.exp(rng.normal(0.0, e_sigma, nEl)) if e_sigma else np.ones(1))
    nus = (rng.uniform(nu_range[0], nu_range[1], nEl) if nu_range else np.array([nu]))
    bot_nodes, bot_dofs = _face_dofs_3d(NodeList, 0.0, (0, 1, 2))
    top_nodes = np.flatnonzero(NodeList[2] == 1.0)
    x, y = NodeList[0, top_nodes], NodeList[1, top_nodes]
    if top == "sin":
        uz = 0.05 * np.sin(np.pi * x) * np.sin(np.pi * y)
    else:
        a = rng.uniform(-1, 1, 4)
        p = rng.integers(1, 5, 4)
        q = rng.integers(1, 5, 4)
        uz = 0.02 * sum(a[k] * np.sin(p[k] * np.pi * x) * np.sin(q[k] * np.pi * y)
                        for k in range(4)) / np.abs(a).sum()
    fixed = np.concatenate([bot_dofs, 3 * top_nodes + 3]).astype(np.int64)
    vals = np.concatenate([np.zeros(bot_dofs.size), uz])
    order = np.argsort(fixed, kind="stable")
    return Problem(name or f"hex{ne}", 3, ne, NodeList, IEN, ID, Young, nus,
                   fixed[order], vals[order], "stress", rtol, seed)


def quad_problem(ne, seed, jitter=0.15, nu=None, nu_range=(0.2, 0.45), e_sigma=None,
                 plane="strain", rtol=1e-8, name=None, rng=None):
    """2D unit-square elasticity: left edge clamped, right edge prescribed u_x.

    u_x = 0.05 * sum_{k=1..3} a_k sin(k pi y) / sum|a_k| on x = 1, u_y free
    there.  One nu per mesh unless ``e_sigma`` asks for per-element E.
    """
    rng = rng if rng is not None else np.random.default_rng(seed)
    NodeList, IEN, ID, _, _ = meshgrid(0, 1, 0, 1, 0, 0, ne, 2)
    if jitter:
        NodeList = jitter_interior(NodeList, ne, jitter, rng)
    nEl = ne * ne
    nus = np.array([nu if nu is not None else rng.uniform(*nu_range)])
    Young = np.exp(rng.normal(0.0, e_sigma, nEl)) if e_sigma else np.ones(1)
    left = np.flatnonzero(NodeList[0] == 0.0)
    right = np.flatnonzero(NodeList[0] == 1.0)
    a = rng.uniform(-1, 1, 3)
    yv = NodeList[1, right]
    ux = 0.05 * sum(a[k] * np.sin((k + 1) * np.pi * yv) for k in range(3)) / np.abs(a).sum()
    fixed = np.concatenate([2 * left + 1, 2 * left + 2, 2 * right + 1]).astype(np.int64)
    vals = np.concatenate([np.zeros(2 * left.size), ux])
    order = np.argsort(fixed, kind="stable")
    return Problem(name or f"quad{ne}", 2, ne, NodeList, IEN, ID, Young, nus,
                   fixed[order], vals[order], plane, rtol, seed)


def inflate_sphere(NodeList, x0, x1, y0, y1):
    """Map every node's (x, y) radially so the square cross-section becomes a
    disc of the same half-width (src/PostProcess.jl:30-44); returns a new
    array (the reference mutates its argument)."""
    out = np.array(NodeList, dtype=np.float64, copy=True)
    d = out[:2] - np.array([[0.5 * (x0 + x1)], [0.5 * (y0 + y1)]])
    scale = np.abs(d).max(axis=0)
    r = np.sqrt(d[0] ** 2 + d[1] ** 2)
    nz = scale != 0.0                      # Julia's `scale ≈ 0.` holds only for exact 0
    out[:2, ~nz] = 0.0
    out[:2, nz] = scale[nz] * d[:, nz] / r[nz]
    return out


def squeeze_increments(NodeList, deltas):
    """Prescribed z-displacements of the squeeze-flow driver
    (examples/vector3D.jl:133-173, :312-313): z-DOF 0 on nodes with z == 0
    and -d on nodes with z == 1 (exact compares), for every d in ``deltas``.
    Returns ``(fixed_dofs, fixed_vals)`` with ``fixed_vals`` (len(deltas), nfix)."""
    z = np.asarray(NodeList)[2]
    nodes = np.flatnonzero((z == 0.0) | (z == 1.0))
    fixed = 3 * nodes + 3
    top = z[nodes] == 1.0
    vals = np.where(top[None, :], -np.asarray(deltas, dtype=np.float64)[:, None], 0.0)
    return fixed.astype(np.int64), vals


def squeeze_problem(ne=8, Young=40.0, nu=0.4):
    """The reference driver's case (examples/vector3D.jl:266-308): unit cube,
    ne^3 hexes, E = 40, nu = 0.4; the penalty faces on the inflated cylinder."""
    NodeList, IEN, ID, IEN_top, IEN_btm = meshgrid(0, 1, 0, 1, 0, 1, ne, 3)
    cyl = inflate_sphere(NodeList, 0, 1, 0, 1)
    faces = np.concatenate([IEN_btm, IEN_top])
    return NodeList, IEN, ID, IEN_top, IEN_btm, cyl, faces


# ---- the five benchmark workloads ------------------------------------------

def parity_cube20():
    """20^3 unit cube, E=1, nu=0.3, no jitter, u_z = 0.05 sin(pi x) sin(pi y) on top."""
    return hex_problem(20, 1001, jitter=0.0, top="sin", rtol=1e-12, name="cube20")


def jittered_cube(ne=128):
    """128^3 jittered (0.2h) cube, E ~ lognormal(0, 0.5), nu=0.3, 4-mode top load, FP64 PCG 1e-10."""
    return hex_problem(ne, 1002, jitter=0.2, e_sigma=0.5, nu=0.3, top="modes",
                       rtol=1e-10, name=f"cube{ne}_jit")


def contrast_cube(ne=96):
    """96^3 jittered cube, E ~ lognormal(0, 1), nu ~ U(0.25, 0.45), 4-mode top load."""
    return hex_problem(ne, 1003, jitter=0.2, e_sigma=1.0, nu_range=(0.25, 0.45),
                       top="modes", rtol=1e-10, name=f"cube{ne}_contrast")


def quad_batch_sizes(count=1024, seed=1004, lo=16, hi=256):
    rng = np.random.default_rng(seed)
    return rng.integers(lo, hi + 1, count)


def quad_batch(count=1024, seed=1004, lo=16, hi=256):
    """``count`` plane-strain unit squares, n ~ U{lo..hi}, jitter 0.15h, E=1, nu_mesh ~ U(0.2, 0.45)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(lo, hi + 1, count)
    return [quad_problem(int(n), seed, jitter=0.15, nu_range=(0.2, 0.45), plane="strain",
                         rtol=1e-8, name=f"batch{b}_q{int(n)}", rng=rng)
            for b, n in enumerate(sizes)]


def serving_stream(count, seed=1005, rate=2000.0, lo2=32, hi2=512, lo3=16, hi3=64):
    """Serving stream: Poisson arrivals at ``rate``/s; 70% 2D quads, 30% 3D hexes.

    Yields ``(arrival_s, Problem)``; E ~ lognormal(0, 0.5) per element,
    nu ~ U(0.25, 0.45) per request.
    """
    rng = np.random.default_rng(seed)
    t = 0.0
    for r in range(count):
        t += rng.exponential(1.0 / rate)
        if rng.uniform() < 0.7:
            n = int(rng.integers(lo2, hi2 + 1))
            nu = float(rng.uniform(0.25, 0.45))
            p = quad_problem(n, seed, jitter=0.15, nu=nu, e_sigma=0.5, plane="strain",
                             rtol=1e-8, name=f"req{r}_q{n}", rng=rng)
        else:
            n = int(rng.integers(lo3, hi3 + 1))
            p = hex_problem(n, int(rng.integers(1 << 30)), jitter=0.2, e_sigma=0.5,
                            nu_range=None, nu=float(rng.uniform(0.25, 0.45)),
                            top="modes", rtol=1e-8, name=f"req{r}_h{n}")
        yield t, p
