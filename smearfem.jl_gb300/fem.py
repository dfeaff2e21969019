"""Host-side mirror of smearFEM.jl's FE API over the GB300 C ABI.

Same names, argument meaning and array shapes as the reference
(src/smearFEM.jl:3 exports ``assemble_system, gaussian_quadrature,
basis_function``), so code written against the reference reads the same:

  gaussian_quadrature(a, b, nGaussPoints=2)                  src/fem.jl:21-31
  basis_function(xi, eta=None, zeta=None, FunctionClass="Q1") src/fem.jl:48-114
  assemble_system(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1,
                  ID=None, Young=1, nu=0.3)                   src/fem.jl:135-256

Arrays use the reference's shapes and 1-based indices: ``NodeList`` (ndim,
nN), ``IEN`` (nEl, nen), ``ID`` (nN, nDof).  ``assemble_system`` returns the
matrix as ``scipy.sparse.csc_matrix`` (the SparseMatrixCSC of the reference)
or, with ``as_handle=True``, a :class:`Matrix` that stays on the GPU.  The
Dirichlet solve of examples/vector3D.jl:314-322 is :func:`solve_dirichlet`.

Errors raise :class:`SfemError` (the reference raises Julia exceptions:
``BoundsError`` for bad indices, ``SingularException`` from ``inv``).
Every numeric step runs in libsmearfem_gpu.so on the GPU; nothing here
computes FE results on the CPU.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib as L
from ._lib import SfemError, check, lib

try:  # device-resident inputs are optional; torch is only plumbing here
    import torch as _torch
except Exception:  # pragma: no cover
    _torch = None


def _is_dev(x):
    return _torch is not None and isinstance(x, _torch.Tensor) and x.is_cuda


class _Buf:
    """Pointer to an argument in Julia (column-major) memory order."""

    def __init__(self, x, dtype, order="F"):
        self.keep = None
        self.space = L.MEM_HOST
        if x is None:
            self.ptr = None
            return
        if _is_dev(x):
            tdt = {np.float64: _torch.float64, np.int64: _torch.int64}[dtype]
            t = x.to(tdt)
            if t.dim() == 2 and order == "F":
                t = t.t()
            t = t.contiguous()
            self.keep = t
            self.ptr = C.c_void_p(t.data_ptr())
            self.space = L.MEM_DEVICE
            self.size = t.numel()
            return
        a = np.asarray(x, dtype=dtype)
        a = np.ascontiguousarray(a.ravel(order=order))
        self.keep = a
        self.size = a.size
        self.ptr = C.c_void_p(a.ctypes.data) if a.size else None


def _to_dev(v, like):
    """A scalar or host array as a float64 CUDA tensor on ``like``'s device."""
    if _is_dev(v):
        return v
    return _torch.as_tensor(np.atleast_1d(np.asarray(v, dtype=np.float64)), device=like.device)


def _space(*bufs):
    spaces = {b.space for b in bufs if b.ptr is not None}
    if len(spaces) > 1:
        raise SfemError(L.SFEM_BAD_ARG, "mix of host and device arrays in one call")
    return spaces.pop() if spaces else L.MEM_HOST


# ---------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------

class Context:
    """One GPU, one CUDA stream (sfem_ctx_create)."""

    def __init__(self, device=0):
        h = C.c_void_p()
        code = lib().sfem_ctx_create(int(device), C.byref(h))
        if code != L.SFEM_OK:
            raise SfemError(code, f"cannot create a context on CUDA device {device}")
        self.h = h
        self.device = device

    def close(self):
        if getattr(self, "h", None):
            lib().sfem_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def sync(self):
        check(lib().sfem_ctx_synchronize(self.h), self.h)

    def error(self):
        return lib().sfem_last_error(self.h).decode()

    @property
    def stream(self):
        """The context's cudaStream_t as an integer handle."""
        return lib().sfem_ctx_stream(self.h) or 0

    def kernel_launches(self):
        return int(lib().sfem_ctx_kernel_launches(self.h))


_contexts = {}


def get_context(device=0):
    ctx = _contexts.get(device)
    if ctx is None or ctx.h is None:
        ctx = _contexts[device] = Context(device)
    return ctx


def version():
    return lib().sfem_version().decode()


# ---------------------------------------------------------------------------
# host helpers (src/fem.jl:21-31, :48-114) -- computed by the library's host code
# ---------------------------------------------------------------------------

def gaussian_quadrature(a, b, nGaussPoints=2):
    """Gauss-Legendre nodes and weights on [a, b] (src/fem.jl:21-31)."""
    xi = np.zeros(max(nGaussPoints, 1))
    w = np.zeros(max(nGaussPoints, 1))
    code = lib().sfem_gaussian_quadrature(float(a), float(b), int(nGaussPoints),
                                          xi.ctypes.data, w.ctypes.data)
    if code != L.SFEM_OK:
        raise SfemError(code, "nGaussPoints must be 2 or 3")
    return xi, w


def basis_function(xi, eta=None, zeta=None, FunctionClass="Q1"):
    """Shape functions and reference gradients (src/fem.jl:48-114).

    Returns ``(N, dN)``; ``dN`` is (nen, ndim) with column k = dN/dxi_k, or
    the 1x2 row of the reference in 1D.
    """
    ndim = 3 if zeta is not None else (2 if eta is not None else 1)
    fc = {"Q1": L.Q1, "Q2": L.Q2}.get(FunctionClass)
    if fc is None:
        raise SfemError(L.SFEM_BAD_ARG, "FunctionClass must be 'Q1' or 'Q2'")
    nen = 9 if fc == L.Q2 else 2 ** ndim
    N = np.zeros(nen)
    dN = np.zeros(nen * ndim)
    code = lib().sfem_basis_function(ndim, fc, float(xi), float(eta or 0.0), float(zeta or 0.0),
                                     N.ctypes.data, dN.ctypes.data)
    if code != L.SFEM_OK:
        raise SfemError(code, f"basis_function: {FunctionClass} is not defined in {ndim}D")
    if ndim == 1:
        return N, dN.reshape(1, 2)
    return N, dN.reshape(ndim, nen).T.copy()


# ---------------------------------------------------------------------------
# mesh / matrix handles
# ---------------------------------------------------------------------------

class Mesh:
    """A mesh uploaded to the GPU (sfem_mesh_create) and its sparsity pattern."""

    def __init__(self, ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1, ID=None, ctx=None,
                 nNodes=None, nen=None, ldIEN=None):
        self.ctx = ctx or get_context()
        self.ndim = int(ndim)
        self.nDof = int(nDof)
        self.ne = int(ne)
        fc = {"Q1": L.Q1, "Q2": L.Q2}.get(FunctionClass)
        if fc is None:
            raise SfemError(L.SFEM_BAD_ARG, "FunctionClass must be 'Q1' or 'Q2'")
        X = _Buf(NodeList, np.float64)
        E = _Buf(IEN, np.int64)
        I = _Buf(ID, np.int64) if nDof > 1 else _Buf(None, np.int64)
        space = _space(X, E, I)
        if nNodes is None:
            nNodes = np.shape(NodeList)[1]
        if ldIEN is None or nen is None:
            rows, cols = np.shape(IEN)[0], np.shape(IEN)[1]
            ldIEN = rows if ldIEN is None else ldIEN
            nen = cols if nen is None else nen
        self.nNodes = int(nNodes)
        h = C.c_void_p()
        code = lib().sfem_mesh_create(self.ctx.h, self.ndim, fc, self.nDof, self.ne, X.ptr,
                                      self.nNodes, E.ptr, int(ldIEN), int(nen), I.ptr, space,
                                      C.byref(h))
        check(code, self.ctx.h)
        self.h = h

    def pattern(self):
        n, nnz = C.c_int64(), C.c_int64()
        check(lib().sfem_pattern_build(self.ctx.h, self.h, C.byref(n), C.byref(nnz)), self.ctx.h)
        return n.value, nnz.value

    def assemble(self, Young=1, nu=0.3, plane="stress"):
        Y = _Buf(np.atleast_1d(Young) if not _is_dev(Young) else Young, np.float64)
        V = _Buf(np.atleast_1d(nu) if not _is_dev(nu) else nu, np.float64)
        h = C.c_void_p()
        code = lib().sfem_assemble(self.ctx.h, self.h, _plane(plane), Y.ptr, Y.size, V.ptr,
                                   V.size, _space(Y, V), C.byref(h))
        check(code, self.ctx.h)
        return Matrix(self.ctx, h)

    def close(self):
        if getattr(self, "h", None):
            lib().sfem_mesh_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _plane(plane):
    if plane in ("stress", L.PLANE_STRESS):
        return L.PLANE_STRESS
    if plane in ("strain", L.PLANE_STRAIN):
        return L.PLANE_STRAIN
    raise SfemError(L.SFEM_BAD_ARG, "plane must be 'stress' or 'strain'")


class Matrix:
    """Assembled K resident on the GPU (sfem_matrix)."""

    def __init__(self, ctx, h):
        self.ctx = ctx
        self.h = h
        n, nnz = C.c_int64(), C.c_int64()
        check(lib().sfem_matrix_info(h, C.byref(n), C.byref(nnz)), ctx.h)
        self.n, self.nnz = n.value, nnz.value

    @property
    def shape(self):
        return (self.n, self.n)

    def to_csc_arrays(self):
        """(colptr, rowval, nzval), 1-based -- SparseMatrixCSC's fields."""
        colptr = np.empty(self.n + 1, np.int64)
        rowval = np.empty(self.nnz, np.int64)
        nzval = np.empty(self.nnz, np.float64)
        check(lib().sfem_matrix_export_csc(self.ctx.h, self.h, colptr.ctypes.data,
                                           rowval.ctypes.data if self.nnz else None,
                                           nzval.ctypes.data if self.nnz else None, L.MEM_HOST),
              self.ctx.h)
        return colptr, rowval, nzval

    def to_scipy(self):
        import scipy.sparse as sp
        colptr, rowval, nzval = self.to_csc_arrays()
        return sp.csc_matrix((nzval, rowval - 1, colptr - 1), shape=self.shape)

    def solve(self, fixed_dofs, fixed_vals, f=None, precision="fp64", precond="jacobi",
              rtol=1e-10, maxit=100000, check_every=32, reliable_delta=0.1, profile=False,
              out=None, fp32_storage="upper"):
        """Dirichlet solve (examples/vector3D.jl:314-322); returns ``(u, stats)``.

        ``fixed_dofs`` are 1-based global DOF ids.  ``out`` may be a device
        tensor (then every array argument must be on the device).
        """
        opts = L.SolveOpts()
        lib().sfem_solve_opts_default(C.byref(opts))
        opts.precision = {"fp64": L.FP64, "mixed": L.MIXED}[precision]
        opts.precond = _PRECOND[precond]
        opts.rtol = rtol
        opts.maxit = maxit
        opts.check_every = check_every
        opts.reliable_delta = reliable_delta
        opts.profile = 1 if profile else 0
        opts.fp32_storage = {"upper": L.FP32_UPPER, "full": L.FP32_FULL}[fp32_storage]
        Fd = _Buf(fixed_dofs, np.int64)
        Fv = _Buf(fixed_vals, np.float64)
        Ff = _Buf(f, np.float64)
        if out is None:
            if _space(Fd, Fv, Ff) == L.MEM_DEVICE:
                out = _torch.empty(self.n, dtype=_torch.float64, device=Fd.keep.device)
            else:
                out = np.empty(self.n)
        U = _Buf.__new__(_Buf)
        if _is_dev(out):
            U.keep, U.ptr, U.space, U.size = out, C.c_void_p(out.data_ptr()), L.MEM_DEVICE, out.numel()
        else:
            U.keep, U.ptr, U.space, U.size = out, C.c_void_p(out.ctypes.data), L.MEM_HOST, out.size
        space = _space(Fd, Fv, Ff, U)
        stats = L.SolveStats()
        code = lib().sfem_solve_dirichlet(self.ctx.h, self.h, Fd.ptr, Fd.size if Fd.ptr else 0,
                                          Fv.ptr, Ff.ptr, U.ptr, space, C.byref(opts),
                                          C.byref(stats))
        check(code, self.ctx.h)
        return out, stats.as_dict()

    def solve_increments(self, fixed_dofs, fixed_vals, f=None, warm_start=True, **kw):
        """The driver's load-increment loop (examples/vector3D.jl:310-338) on
        this K: ``fixed_vals`` is (nsteps, nfix), one row of prescribed
        values per step, for the same ``fixed_dofs``.  Returns ``(U, stats)``
        with ``U`` of shape (nsteps, n).  ``warm_start`` starts each step from
        the best affine combination of earlier solutions."""
        fd = np.ascontiguousarray(np.asarray(fixed_dofs, dtype=np.int64).ravel())
        fv = np.ascontiguousarray(np.atleast_2d(np.asarray(fixed_vals, dtype=np.float64)))
        nsteps = fv.shape[0]
        if fv.shape[1] != fd.size:
            raise SfemError(L.SFEM_BAD_ARG, "fixed_vals must be (nsteps, len(fixed_dofs))")
        F = _Buf(f, np.float64)
        U = np.empty((nsteps, self.n))
        stats = (L.SolveStats * max(nsteps, 1))()
        opts = _solve_opts(**kw)
        check(lib().sfem_solve_increments(self.ctx.h, self.h, fd.ctypes.data if fd.size else None, fd.size,
                                          fv.ctypes.data if fv.size else None, nsteps, F.ptr, U.ctypes.data,
                                          L.MEM_HOST, C.byref(opts), 1 if warm_start else 0, stats),
              self.ctx.h)
        return U, [stats[i].as_dict() for i in range(nsteps)]

    def add_penalty(self, NodeList, IEN_faces, beta):
        """``K <- K + beta * b`` in place on the GPU, b the surface penalty of
        ``apply_boundary_conditions`` (examples/vector3D.jl:175-264,306-308).

        ``NodeList`` (3, nNodes): the coordinates the faces are integrated
        on; ``IEN_faces`` (nFaces, 4), 1-based, in the reference's order
        ``[IEN_btm; IEN_top]``.
        """
        X = _Buf(NodeList, np.float64)
        F = _Buf(IEN_faces, np.int64)
        check(lib().sfem_penalty_add(self.ctx.h, self.h, X.ptr, F.ptr, int(np.shape(IEN_faces)[0]),
                                     int(np.shape(IEN_faces)[1]), float(beta), _space(X, F)), self.ctx.h)
        return self

    def close(self):
        if getattr(self, "h", None):
            lib().sfem_matrix_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# "multigrid": batches and servers, mixed precision; geometric multigrid on
# structured (meshgrid) Q1 meshes, block Jacobi on the others
_PRECOND = {"jacobi": L.PC_JACOBI, "block_jacobi": L.PC_BLOCK_JACOBI, "multigrid": L.PC_MULTIGRID}


def _solve_opts(precision="fp64", precond="jacobi", rtol=1e-10, maxit=100000, check_every=32,
                reliable_delta=0.1, profile=False, fp32_storage="upper"):
    opts = L.SolveOpts()
    lib().sfem_solve_opts_default(C.byref(opts))
    opts.precision = {"fp64": L.FP64, "mixed": L.MIXED}[precision]
    opts.precond = _PRECOND[precond]
    opts.rtol = rtol
    opts.maxit = maxit
    opts.check_every = check_every
    opts.reliable_delta = reliable_delta
    opts.profile = 1 if profile else 0
    opts.fp32_storage = {"upper": L.FP32_UPPER, "full": L.FP32_FULL}[fp32_storage]
    return opts


class Batch:
    """Many independent meshes of one element class (sfem_batch_*).

    ``meshes`` is a list of ``(NodeList, IEN)`` or ``(NodeList, IEN, ID)``
    tuples in the reference's shapes with mesh-local 1-based indices.
    Every mesh is assembled and solved by one persistent kernel launch.
    """

    def __init__(self, meshes, ndim, nDof, FunctionClass="Q1", ctx=None):
        self.ctx = ctx or get_context()
        self.ndim, self.nDof = int(ndim), int(nDof)
        nn = [np.shape(m[0])[1] for m in meshes]
        ne = [np.shape(m[1])[0] for m in meshes]
        self.node_off = np.concatenate([[0], np.cumsum(nn)]).astype(np.int64)
        self.elem_off = np.concatenate([[0], np.cumsum(ne)]).astype(np.int64)
        X = np.concatenate([np.asarray(m[0], dtype=np.float64) for m in meshes], axis=1)
        IEN = np.concatenate([np.asarray(m[1], dtype=np.int64) for m in meshes], axis=0)
        has_id = self.nDof > 1 and all(len(m) > 2 and m[2] is not None for m in meshes)
        ID = np.concatenate([np.asarray(m[2], dtype=np.int64) for m in meshes], axis=0) if has_id else None
        Xb, Eb, Ib = _Buf(X, np.float64), _Buf(IEN, np.int64), _Buf(ID, np.int64)
        fc = {"Q1": L.Q1, "Q2": L.Q2}[FunctionClass]
        h = C.c_void_p()
        check(lib().sfem_batch_create(self.ctx.h, self.ndim, fc, self.nDof, len(meshes),
                                      self.node_off.ctypes.data, self.elem_off.ctypes.data, Xb.ptr,
                                      Eb.ptr, Ib.ptr, L.MEM_HOST, C.byref(h)), self.ctx.h)
        self.h = h
        self.nmesh = len(meshes)
        td = C.c_int64()
        check(lib().sfem_batch_info(h, C.byref(td), None, None), self.ctx.h)
        self.total_dofs = td.value

    @classmethod
    def from_problems(cls, problems, ctx=None):
        p0 = problems[0]
        return cls([(p.NodeList, p.IEN[: p.n_elem], p.ID) for p in problems], p0.ndim, p0.nDof,
                   ctx=ctx)

    def set_launch(self, threads=512, ctas_per_sm=1, cluster=8, cluster_min_nodes=16384):
        check(lib().sfem_batch_set_launch(self.h, int(threads), int(ctas_per_sm), int(cluster),
                                          int(cluster_min_nodes)), self.ctx.h)

    def _pack(self, Young, nu, fixed_dofs, fixed_vals):
        fo = np.concatenate([[0], np.cumsum([len(f) for f in fixed_dofs])]).astype(np.int64)
        fd = np.concatenate([np.asarray(f, dtype=np.int64) for f in fixed_dofs])
        fv = np.concatenate([np.asarray(v, dtype=np.float64) for v in fixed_vals])
        Y = np.ascontiguousarray(np.atleast_1d(np.asarray(Young, dtype=np.float64)).ravel())
        V = np.ascontiguousarray(np.atleast_1d(np.asarray(nu, dtype=np.float64)).ravel())
        return fo, fd, fv, Y, V

    def autotune(self, Young, nu, fixed_dofs, fixed_vals, plane="stress", sample=128, **kw):
        """Pick the persistent kernel's launch shape by timing candidates on a
        sample of this batch; returns (launch shape dict, best sample ms)."""
        fo, fd, fv, Y, V = self._pack(Young, nu, fixed_dofs, fixed_vals)
        opts = _solve_opts(**kw)
        best = C.c_double()
        check(lib().sfem_batch_autotune(self.ctx.h, self.h, _plane(plane), Y.ctypes.data, Y.size,
                                        V.ctypes.data, V.size, fo.ctypes.data, fd.ctypes.data,
                                        fv.ctypes.data, L.MEM_HOST, C.byref(opts), int(sample),
                                        C.byref(best)), self.ctx.h)
        return self.launch(), best.value

    def launch(self):
        t, c, cl, grid = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        mn = C.c_int64()
        check(lib().sfem_batch_get_launch(self.h, C.byref(t), C.byref(c), C.byref(cl), C.byref(mn),
                                          C.byref(grid)), self.ctx.h)
        return {"threads": t.value, "ctas_per_sm": c.value, "cluster": cl.value,
                "cluster_min_nodes": mn.value, "last_grid": grid.value}

    def solve(self, Young, nu, fixed_dofs, fixed_vals, plane="stress", out=None, **kw):
        """``fixed_dofs``/``fixed_vals``: lists (one array per mesh, 1-based local
        DOFs).  ``Young``/``nu``: scalar, per-mesh or per-element arrays.
        Returns ``(u, stats)`` with ``u`` the concatenated displacements (mesh m
        starts at nDof*node_offsets[m]) and ``stats`` a list of dicts."""
        fo, fd, fv, Y, V = self._pack(Young, nu, fixed_dofs, fixed_vals)
        u = np.empty(self.total_dofs) if out is None else out
        stats = (L.BatchStats * self.nmesh)()
        opts = _solve_opts(**kw)
        check(lib().sfem_batch_solve(self.ctx.h, self.h, _plane(plane), Y.ctypes.data, Y.size,
                                     V.ctypes.data, V.size, fo.ctypes.data, fd.ctypes.data,
                                     fv.ctypes.data, u.ctypes.data, L.MEM_HOST, C.byref(opts),
                                     stats), self.ctx.h)
        return u, [{k: getattr(s, k) for k, _ in s._fields_} for s in stats]

    def split(self, u):
        return [u[self.nDof * self.node_off[m]: self.nDof * self.node_off[m + 1]]
                for m in range(self.nmesh)]

    def close(self):
        if getattr(self, "h", None):
            lib().sfem_batch_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Server:
    """A device-resident request loop (sfem_server_*).

    ``submit`` queues one mesh (reference shapes, 1-based indices, host
    arrays) and returns a request id at once; ``wait`` returns its
    displacements.  One persistent kernel takes requests of any element
    class as they arrive and solves many at once; requests sharing a
    ``topology_key`` reuse the sparsity pattern built for the first of them.
    ``solve_kw`` are the solver options (default: mixed precision, block
    Jacobi, rtol 1e-8); ``precond="multigrid"`` gives meshgrid meshes a
    geometric multigrid hierarchy (a smaller ``reliable_delta``, e.g. 0.01,
    then saves FP64 refreshes).
    """

    def __init__(self, cluster=4, threads=512, sm_fraction=0.9, hbm_budget_fraction=0.5,
                 hbm_budget_bytes=0, max_inflight=1024, idle_exit_ms=20.0, warm_start=False, device=0,
                 **solve_kw):
        cfg = L.ServerConfig()
        lib().sfem_server_config_default(C.byref(cfg))
        cfg.cluster, cfg.threads = int(cluster), int(threads)
        cfg.sm_fraction = float(sm_fraction)
        cfg.hbm_budget_fraction = float(hbm_budget_fraction)
        cfg.hbm_budget_bytes = int(hbm_budget_bytes)
        cfg.max_inflight = int(max_inflight)
        cfg.idle_exit_ms = float(idle_exit_ms)
        cfg.warm_start = 1 if warm_start else 0
        kw = {"precision": "mixed", "precond": "block_jacobi", "rtol": 1e-8}
        kw.update(solve_kw)
        cfg.solve = _solve_opts(**kw)
        h = C.c_void_p()
        check(lib().sfem_server_create(int(device), C.byref(cfg), C.byref(h)))
        self.h = h
        self._ndof = {}
        self._nel_of_key = {}

    def submit(self, NodeList, IEN=None, ID=None, Young=1.0, nu=0.3, fixed_dofs=(), fixed_vals=(),
               topology_key=0, ndim=None, nDof=None, FunctionClass="Q1", plane="stress"):
        """``ndim`` defaults to the rows of ``NodeList``; ``nDof`` to ``ndim``
        when ``ID`` is given (elasticity), else 1."""
        ndim = int(ndim if ndim is not None else np.shape(NodeList)[0])
        nDof = int(nDof if nDof is not None else (ndim if ID is not None else 1))
        X = _Buf(NodeList, np.float64)
        E = np.ascontiguousarray(np.atleast_1d(np.asarray(Young, dtype=np.float64)).ravel())
        V = np.ascontiguousarray(np.atleast_1d(np.asarray(nu, dtype=np.float64)).ravel())
        fd = np.ascontiguousarray(np.asarray(fixed_dofs, dtype=np.int64).ravel())
        fv = np.ascontiguousarray(np.asarray(fixed_vals, dtype=np.float64).ravel())
        if fv.size != fd.size:
            raise SfemError(L.SFEM_BAD_ARG, "fixed_dofs and fixed_vals differ in length")
        nN = np.shape(NodeList)[1]
        nEl = np.shape(IEN)[0] if IEN is not None else self._nel_of_key.get(topology_key)
        if nEl is None:
            raise SfemError(L.SFEM_BAD_ARG, "IEN is needed for a topology key not submitted before")
        Ib, Db = _Buf(IEN, np.int64), _Buf(ID if nDof > 1 else None, np.int64)
        if X.space != L.MEM_HOST or Ib.space != L.MEM_HOST:
            raise SfemError(L.SFEM_BAD_ARG, "server requests are host arrays")
        fc = {"Q1": L.Q1, "Q2": L.Q2}[FunctionClass]
        rid = C.c_int64()
        code = lib().sfem_server_submit(self.h, ndim, fc, nDof, _plane(plane), int(topology_key), X.ptr,
                                        nN, Ib.ptr, nEl, Db.ptr, E.ctypes.data, E.size, V.ctypes.data,
                                        V.size, fd.ctypes.data if fd.size else None, fd.size,
                                        fv.ctypes.data if fv.size else None, C.byref(rid))
        if code:
            raise SfemError(code, "sfem_server_submit")
        if topology_key and IEN is not None:
            self._nel_of_key[topology_key] = nEl
        self._ndof[rid.value] = nDof * nN
        return rid.value

    def wait(self, request_id, timeout_ms=-1.0):
        """``(u, result dict)``; raises SfemError(SFEM_TIMEOUT) if not done in time."""
        n = self._ndof[request_id]
        u = np.empty(n)
        res = L.ServerResult()
        code = lib().sfem_server_wait(self.h, int(request_id), float(timeout_ms), u.ctypes.data, n,
                                      C.byref(res))
        if code:
            raise SfemError(code, f"sfem_server_wait({request_id})")
        del self._ndof[request_id]
        return u, {k: getattr(res, k) for k, _ in res._fields_}

    def info(self):
        t = L.ServerTotals()
        check(lib().sfem_server_info(self.h, C.byref(t)))
        return {k: getattr(t, k) for k, _ in t._fields_}

    def close(self):
        if getattr(self, "h", None):
            lib().sfem_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# reference-shaped entry points
# ---------------------------------------------------------------------------

def assemble_system(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1, ID=None, Young=1,
                    nu=0.3, plane="stress", ctx=None, as_handle=False):
    """``assemble_system`` of src/fem.jl:135-256 on the GPU.

    Processes elements ``1:ne^ndim`` of ``IEN`` (src/fem.jl:179).  Returns the
    stiffness matrix as ``scipy.sparse.csc_matrix`` -- same size, pattern and
    values (to rounding) as ``sparse(E,J,V)`` at src/fem.jl:253 -- or the GPU
    :class:`Matrix` handle when ``as_handle`` is true.  ``Young``/``nu`` may
    be scalars (the reference) or per-element arrays; ``plane`` picks the 2D
    law (the reference's is plane stress).
    """
    ctx = ctx or get_context()
    fc = {"Q1": L.Q1, "Q2": L.Q2}.get(FunctionClass)
    if fc is None:
        raise SfemError(L.SFEM_BAD_ARG, "FunctionClass must be 'Q1' or 'Q2'")
    X = _Buf(NodeList, np.float64)
    E = _Buf(IEN, np.int64)
    I = _Buf(ID, np.int64) if int(nDof) > 1 else _Buf(None, np.int64)
    # material values follow the mesh into device memory when the mesh lives there
    on_dev = X.space == L.MEM_DEVICE
    Young = _to_dev(Young, NodeList) if on_dev else Young
    nu = _to_dev(nu, NodeList) if on_dev else nu
    Y = _Buf(np.atleast_1d(Young) if not _is_dev(Young) else Young, np.float64)
    V = _Buf(np.atleast_1d(nu) if not _is_dev(nu) else nu, np.float64)
    space = _space(X, E, I, Y, V)
    rows, cols = np.shape(IEN)[0], np.shape(IEN)[1]
    h = C.c_void_p()
    n, nnz = C.c_int64(), C.c_int64()
    code = lib().sfem_assemble_system(ctx.h, int(ne), X.ptr, int(np.shape(NodeList)[1]), E.ptr,
                                      int(rows), int(cols), int(ndim), fc, int(nDof), I.ptr, Y.ptr,
                                      Y.size, V.ptr, V.size, _plane(plane), space, C.byref(h),
                                      C.byref(n), C.byref(nnz))
    check(code, ctx.h)
    K = Matrix(ctx, h)
    if as_handle:
        return K
    try:
        return K.to_scipy()
    finally:
        K.close()


def multigrid_info(nNodes, IEN, ndim, nDof=None, FunctionClass="Q1"):
    """Whether ``precond="multigrid"`` gives this mesh a hierarchy (host only,
    no GPU): ``{"ne": elements per direction of the meshgrid grid or 0,
    "levels": hierarchy levels or 0, "bytes": its device memory}``.
    ``IEN`` is the reference's nEl x nen array (1-based)."""
    nDof = int(nDof if nDof is not None else ndim)
    E = _Buf(IEN, np.int64)
    nEl = int(np.shape(IEN)[0])
    ne, lv, nb = C.c_int(), C.c_int(), C.c_int64()
    check(lib().sfem_multigrid_info(int(ndim), {"Q1": L.Q1, "Q2": L.Q2}[FunctionClass], nDof, int(nNodes),
                                    C.cast(E.ptr, L.I64P), nEl, C.byref(ne), C.byref(lv), C.byref(nb)))
    return {"ne": ne.value, "levels": lv.value, "bytes": nb.value}


def meshgrid(x0, x1, y0, y1, z0, z1, ne, ndim, device=False, ctx=None):
    """The reference's ``meshgrid`` (examples/vector3D.jl:10-130) generated on
    the GPU.  Returns ``(NodeList, IEN, ID, IEN_top, IEN_btm)`` in the
    reference's shapes, 1-based: numpy arrays, or with ``device=True`` CUDA
    tensors that stay on the GPU (the other entry points take them as they
    are, so no host copy of the mesh is made)."""
    ctx = ctx or get_context()
    ne, ndim = int(ne), int(ndim)
    n1 = ne + 1
    nN, nEl, nF, nenF = n1 ** ndim, ne ** ndim, ne ** (ndim - 1), 2 ** (ndim - 1)
    # (rows, cols) of each output in the reference's Julia shapes; stored column-major
    shapes = [(ndim, nN, np.float64), (nEl, 2 ** ndim, np.int64), (nN, ndim, np.int64), (nF, nenF, np.int64),
              (nF, nenF, np.int64)]
    tdt = {np.float64: _torch.float64, np.int64: _torch.int64}
    if device:
        dev = _torch.device("cuda", ctx.device)
        bufs = [_torch.empty(r * c, dtype=tdt[t], device=dev) for r, c, t in shapes]
        ptrs = [C.c_void_p(b.data_ptr()) for b in bufs]
        space = L.MEM_DEVICE
    else:
        bufs = [np.empty(r * c, dtype=t) for r, c, t in shapes]
        ptrs = [C.c_void_p(b.ctypes.data) for b in bufs]
        space = L.MEM_HOST
    check(lib().sfem_meshgrid(ctx.h, float(x0), float(x1), float(y0), float(y1), float(z0), float(z1), ne,
                              ndim, *ptrs, space), ctx.h)
    return tuple(b.view(c, r).t() if device else b.reshape(c, r).T for b, (r, c, _t) in zip(bufs, shapes))


def inflate_sphere(NodeList, x0, x1, y0, y1, ctx=None):
    """``inflate_sphere`` (src/PostProcess.jl:30-44) on the GPU.  A CUDA
    tensor is changed in place (as the reference changes its argument);
    a numpy array is returned as a new array."""
    ctx = ctx or get_context()
    if _is_dev(NodeList):
        X = NodeList
        flat = X.t().contiguous() if not X.t().is_contiguous() else X.t()
        check(lib().sfem_inflate_sphere(ctx.h, C.c_void_p(flat.data_ptr()), int(X.shape[0]), int(X.shape[1]),
                                        float(x0), float(x1), float(y0), float(y1), L.MEM_DEVICE), ctx.h)
        if flat.data_ptr() != X.t().data_ptr():
            X.copy_(flat.t())
        return X
    out = np.array(NodeList, dtype=np.float64, order="F", copy=True)
    check(lib().sfem_inflate_sphere(ctx.h, C.c_void_p(out.ctypes.data), int(out.shape[0]), int(out.shape[1]),
                                    float(x0), float(x1), float(y0), float(y1), L.MEM_HOST), ctx.h)
    return out


def _field_ncomp(q, nN):
    shape = tuple(q.shape)
    if len(shape) == 1:
        if shape[0] != nN:
            raise SfemError(L.SFEM_BAD_ARG, "a vector field has one value per node")
        return 1
    if shape[1] != nN:
        raise SfemError(L.SFEM_BAD_ARG, "a matrix field is (components, nNodes)")
    return shape[0]


def write_vtk(fileName, fieldName, NodeList, IEN, ne, ndim, q, ctx=None):
    """``write_vtk`` of src/PostProcess.jl:258-279: ``fileName`` + ".vtu" with
    cells ``IEN[1:ne^ndim, :]`` and the point field ``q`` (nNodes values, or
    a (components, nNodes) matrix like the driver's ``motion``).  Host
    arrays are written without a GPU; CUDA tensors are copied from it."""
    nEl = int(ne) ** int(ndim)
    X, E, Q = _Buf(NodeList, np.float64), _Buf(np.asarray(IEN)[:nEl] if not _is_dev(IEN) else IEN[:nEl],
                                               np.int64), _Buf(q, np.float64)
    space = _space(X, E, Q)
    nN = int(np.shape(NodeList)[1])
    ncomp = _field_ncomp(q, nN)
    h = get_context().h if space == L.MEM_DEVICE else (ctx.h if ctx else None)
    check(lib().sfem_vtk_write(h, (str(fileName) + ".vtu").encode(), X.ptr, int(np.shape(NodeList)[0]), nN, E.ptr,
                               nEl, int(np.shape(IEN)[1]), str(fieldName).encode(), Q.ptr, ncomp, space), h)


def write_scene(fileName, NodeList, IEN, ne, ndim, fields, ctx=None):
    """``write_scene`` of src/PostProcess.jl:281-304: one ``<fileName>timestep_i.vtu``
    per field (point data "u") and ``<fileName>displacement.pvd`` with the
    steps at times 0, 1, ...  ``fields``: a list of equally shaped arrays, or
    one (nsteps, components, nNodes) array or CUDA tensor."""
    nEl = int(ne) ** int(ndim)
    nN = int(np.shape(NodeList)[1])
    if _is_dev(fields):
        F = fields.contiguous()
        nsteps = int(F.shape[0])
        ncomp = _field_ncomp(F[0], nN) if nsteps else 1
        # each step (components, nNodes) must be column-major: (nNodes, components) rows
        F = F.transpose(1, 2).contiguous() if F.dim() == 3 else F
        Fp, space = C.c_void_p(F.data_ptr()), L.MEM_DEVICE
        keep = F
    else:
        arr = [np.asarray(f, dtype=np.float64) for f in fields]
        nsteps = len(arr)
        ncomp = _field_ncomp(arr[0], nN) if nsteps else 1
        keep = np.concatenate([f.ravel(order="F") for f in arr]) if nsteps else np.zeros(1)
        Fp, space = C.c_void_p(keep.ctypes.data), L.MEM_HOST
    X, E = _Buf(NodeList, np.float64), _Buf(np.asarray(IEN)[:nEl] if not _is_dev(IEN) else IEN[:nEl], np.int64)
    if _space(X, E) != space:
        raise SfemError(L.SFEM_BAD_ARG, "mesh and fields must be in the same memory space")
    h = get_context().h if space == L.MEM_DEVICE else (ctx.h if ctx else None)
    check(lib().sfem_vtk_write_scene(h, str(fileName).encode(), X.ptr, int(np.shape(NodeList)[0]), nN, E.ptr, nEl,
                                     int(np.shape(IEN)[1]), Fp, ncomp, nsteps, space), h)
    del keep


def apply_boundary_conditions(ne, NodeList, IEN, IEN_top, IEN_btm, ndim, FunctionClass="Q1", ID=None,
                              nDof=3, ctx=None):
    """``apply_boundary_conditions`` of examples/vector3D.jl:175-264 on the GPU.

    Returns the surface penalty matrix ``b`` as ``scipy.sparse.csc_matrix``
    with the reference's pattern: every DOF pair of every top/bottom face
    node pair, the off-diagonal DOF pairs as explicit zeros.  It is computed
    by adding the penalty (beta = 1) to an all-zero matrix with K's pattern;
    for the driver's ``K_bar = K + beta*b`` keep K on the GPU and call
    :meth:`Matrix.add_penalty` instead.  3D Q1 only, as the reference.
    """
    if ndim != 3 or FunctionClass != "Q1" or nDof != 3:
        raise SfemError(L.SFEM_UNSUPPORTED, "the reference's surface penalty exists for 3D Q1 "
                                            "elasticity only")
    ctx = ctx or get_context()
    nface = int(ne) ** (ndim - 1)
    faces = np.concatenate([np.asarray(IEN_btm, np.int64)[:nface], np.asarray(IEN_top, np.int64)[:nface]])
    Z = assemble_system(ne, NodeList, IEN, ndim, FunctionClass, nDof, ID, 0.0, 0.3, ctx=ctx, as_handle=True)
    try:
        Z.add_penalty(NodeList, faces, 1.0)
        b = Z.to_scipy()
    finally:
        Z.close()
    # keep the entries of node pairs that share a face (the reference's COO triplets)
    ID = np.asarray(ID, np.int64)
    dof_node = np.empty(ID.size, np.int64)
    dof_node[ID.ravel(order="C") - 1] = np.repeat(np.arange(ID.shape[0]), ID.shape[1])
    pairs = set()
    for f in faces - 1:
        for a in f:
            for c in f:
                pairs.add((int(a), int(c)))
    coo = b.tocoo()
    keep = np.array([(int(dof_node[r]), int(dof_node[c])) in pairs for r, c in zip(coo.row, coo.col)],
                    dtype=bool)
    import scipy.sparse as sp
    n = int(max(ID[faces - 1].max(), 1))
    out = sp.csc_matrix((coo.data[keep], (coo.row[keep], coo.col[keep])), shape=(n, n))
    out.sort_indices()
    return out


def solve_dirichlet(K, fixed_dofs, fixed_vals, f=None, **opts):
    """``q = q_d + C * (K_free \\ C'(f - K q_d))`` (examples/vector3D.jl:314-322).

    ``K`` is a :class:`Matrix` handle from ``assemble_system(...,
    as_handle=True)``.  Returns ``(q, stats)``.
    """
    if not isinstance(K, Matrix):
        raise SfemError(L.SFEM_BAD_ARG, "solve_dirichlet needs the GPU matrix handle "
                                        "(assemble_system(..., as_handle=True))")
    return K.solve(fixed_dofs, fixed_vals, f, **opts)
