"""ctypes wrapper around the C oracle (sfem_oracle.c) -- TEST INFRASTRUCTURE ONLY.

Build with :func:`build` (gcc, OpenMP, ``-ffp-contract=off`` so x86 and Arm
round the same way).  Used by the tests as the checker and by bench.py's
CPU-baseline leg; never by the GPU product.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "sfem_oracle.c")
LIB = os.path.join(HERE, "_build", "libsfem_oracle.so")

_lib = None


def build(force=False):
    """Compile the C oracle into oracle/_build/libsfem_oracle.so."""
    os.makedirs(os.path.dirname(LIB), exist_ok=True)
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(SRC):
        return LIB
    tmp = LIB + f".{os.getpid()}.tmp"
    subprocess.check_call(["gcc", "-O3", "-fopenmp", "-ffp-contract=off", "-fPIC", "-shared",
                           "-o", tmp, SRC, "-lm"])
    os.replace(tmp, LIB)
    return LIB


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB):
            build()
        L = C.CDLL(LIB)
        P = C.c_void_p
        i64p = np.ctypeslib.ndpointer(np.int64, flags="C_CONTIGUOUS")
        f64p = np.ctypeslib.ndpointer(np.float64, flags="C_CONTIGUOUS")
        L.oc_assemble.restype = P
        L.oc_assemble.argtypes = [C.c_int, C.c_int, C.c_int64, C.c_int, C.c_int, C.c_int,
                                  f64p, C.c_int64, i64p, C.c_int64, P, f64p, C.c_int64,
                                  f64p, C.c_int64, C.c_int, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
        L.oc_csc_info.argtypes = [P, C.POINTER(C.c_int64), C.POINTER(C.c_int64),
                                  C.POINTER(C.c_int64)]
        L.oc_csc_copy.argtypes = [P, i64p, i64p, f64p]
        L.oc_csc_wrap.restype = P
        L.oc_csc_wrap.argtypes = [C.c_int64, C.c_int64, i64p, i64p, f64p]
        L.oc_free.argtypes = [P]
        L.oc_solve_pcg.restype = C.c_int
        L.oc_solve_pcg.argtypes = [P, i64p, C.c_int64, f64p, P, C.c_double, C.c_int, C.c_int,
                                   f64p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                   C.POINTER(C.c_double)]
        L.oc_solve_pcg_mark.restype = C.c_int
        L.oc_solve_pcg_mark.argtypes = [P, i64p, C.c_int64, f64p, P, C.c_double, C.c_int, C.c_int,
                                        f64p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                        C.POINTER(C.c_double), C.c_double, C.POINTER(C.c_int),
                                        C.POINTER(C.c_double)]
        L.oc_pcg_begin.restype = P
        L.oc_pcg_begin.argtypes = [P, i64p, C.c_int64, f64p, P, C.c_int]
        L.oc_pcg_run.restype = C.c_int
        L.oc_pcg_run.argtypes = [P, C.c_int, C.c_double, C.c_double, C.POINTER(C.c_int),
                                 C.POINTER(C.c_double)]
        L.oc_pcg_end.restype = C.c_int
        L.oc_pcg_end.argtypes = [P, f64p, C.POINTER(C.c_int), C.POINTER(C.c_double),
                                 C.POINTER(C.c_double)]
        L.oc_max_threads.restype = C.c_int
        _lib = L
    return _lib


class OracleCSC:
    """Owns a CSC assembled (or wrapped) by the C oracle."""

    def __init__(self, handle, t_elem=0.0, t_sparse=0.0):
        self.h = handle
        self.t_elem = t_elem
        self.t_sparse = t_sparse

    def __del__(self):
        if getattr(self, "h", None):
            lib().oc_free(self.h)
            self.h = None

    def arrays(self):
        m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        lib().oc_csc_info(self.h, C.byref(m), C.byref(n), C.byref(nnz))
        colptr = np.empty(n.value + 1, np.int64)
        rowval = np.empty(nnz.value, np.int64)
        nzval = np.empty(nnz.value, np.float64)
        lib().oc_csc_copy(self.h, colptr, rowval, nzval)
        return colptr, rowval, nzval, m.value, n.value

    def solve(self, fixed_dofs, fixed_vals, f=None, rtol=1e-13, maxit=200000, nthreads=0,
              max_iters=None, mark_rtol=None):
        """Jacobi-PCG on the eliminated system.  With ``mark_rtol`` the stats
        also hold ``mark_iters`` / ``mark_s``: the iteration and the seconds
        since the solve started at which the relative residual first reached
        ``mark_rtol`` (a looser solve's cost, measured inside this one)."""
        m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        lib().oc_csc_info(self.h, C.byref(m), C.byref(n), C.byref(nnz))
        u = np.empty(n.value)
        it = C.c_int()
        rr = C.c_double()
        ts = C.c_double()
        fx = np.ascontiguousarray(fixed_dofs, dtype=np.int64)
        fv = np.ascontiguousarray(fixed_vals, dtype=np.float64)
        fp = None
        if f is not None:
            f = np.ascontiguousarray(f, dtype=np.float64)
            fp = f.ctypes.data
        mi, ms = C.c_int(-1), C.c_double(0.0)
        st = lib().oc_solve_pcg_mark(self.h, fx, fx.size, fv, fp, rtol,
                                     max_iters if max_iters else maxit, nthreads, u,
                                     C.byref(it), C.byref(rr), C.byref(ts),
                                     float(mark_rtol or 0.0), C.byref(mi), C.byref(ms))
        out = dict(status=st, iters=it.value, relres=rr.value, seconds=ts.value)
        if mark_rtol:
            out.update(mark_iters=mi.value, mark_s=ms.value)
        return u, out


class PcgSolve:
    """The oracle's Jacobi-PCG split into resumable pieces: ``run`` performs up
    to ``max_iters`` more iterations (the iterations of one uninterrupted
    solve), ``finish`` returns ``(u, stats)`` and frees the state."""

    def __init__(self, K, fixed_dofs, fixed_vals, f=None, nthreads=0):
        self.K = K  # keeps the matrix alive while the solve runs
        m, n, nnz = C.c_int64(), C.c_int64(), C.c_int64()
        lib().oc_csc_info(K.h, C.byref(m), C.byref(n), C.byref(nnz))
        self.n = n.value
        fx = np.ascontiguousarray(fixed_dofs, dtype=np.int64)
        fv = np.ascontiguousarray(fixed_vals, dtype=np.float64)
        fp = None
        if f is not None:
            self._f = np.ascontiguousarray(f, dtype=np.float64)
            fp = self._f.ctypes.data
        self.s = lib().oc_pcg_begin(K.h, fx, fx.size, fv, fp, int(nthreads))
        self.mark_iters, self.mark_s = C.c_int(-1), C.c_double(0.0)

    def run(self, max_iters, rtol, mark_rtol=0.0):
        """Returns 0 once converged, 1 while iterations remain, 2 on a zero diagonal."""
        return int(lib().oc_pcg_run(self.s, int(max_iters), float(rtol), float(mark_rtol),
                                    C.byref(self.mark_iters), C.byref(self.mark_s)))

    def finish(self):
        u = np.empty(self.n)
        it, rr, ts = C.c_int(), C.c_double(), C.c_double()
        st = lib().oc_pcg_end(self.s, u, C.byref(it), C.byref(rr), C.byref(ts))
        self.s = None
        return u, dict(status=st, iters=it.value, relres=rr.value, seconds=ts.value,
                       mark_iters=self.mark_iters.value, mark_s=self.mark_s.value)


def assemble(ne, NodeList, IEN, ndim, FunctionClass="Q1", nDof=1, ID=None, Young=1.0,
             nu=0.3, plane="stress", nthreads=0, n_elem=None):
    """C restatement of assemble_system (src/fem.jl:135-256); returns OracleCSC.

    ``n_elem`` overrides ``ne^ndim`` (used to time a bounded sample of the
    element loop).
    """
    NodeList = np.ascontiguousarray(np.asarray(NodeList, dtype=np.float64).T)  # (nN, ndim)
    IENf = np.asfortranarray(np.asarray(IEN, dtype=np.int64))
    nEl = int(ne) ** int(ndim) if n_elem is None else int(n_elem)
    if IENf.shape[0] < nEl:
        raise IndexError("IEN has fewer rows than ne^ndim")
    ien_flat = IENf.ravel(order="F")
    E = np.ascontiguousarray(np.atleast_1d(np.asarray(Young, dtype=np.float64)))
    NU = np.ascontiguousarray(np.atleast_1d(np.asarray(nu, dtype=np.float64)))
    IDp = None
    if nDof > 1:
        IDf = np.asfortranarray(np.asarray(ID, dtype=np.int64)).ravel(order="F")
        IDp = IDf.ctypes.data
    fclass = 1 if FunctionClass == "Q1" else 2
    te, tsp = C.c_double(), C.c_double()
    h = lib().oc_assemble(ndim, IENf.shape[1], nEl, nDof, fclass, 1 if plane == "strain" else 0,
                          NodeList.ravel(), NodeList.shape[0], ien_flat, IENf.shape[0], IDp,
                          E, E.size, NU, NU.size, nthreads, C.byref(te), C.byref(tsp))
    if not h:
        raise ValueError("oracle: unsupported element class")
    return OracleCSC(h, te.value, tsp.value)


def wrap_csc(colptr, rowval, nzval, n):
    colptr = np.ascontiguousarray(colptr, dtype=np.int64)
    rowval = np.ascontiguousarray(rowval, dtype=np.int64)
    nzval = np.ascontiguousarray(nzval, dtype=np.float64)
    return OracleCSC(lib().oc_csc_wrap(n, rowval.size, colptr, rowval, nzval))


def max_threads():
    return int(lib().oc_max_threads())


def time_call(fn, *a, **k):
    t = time.perf_counter()
    out = fn(*a, **k)
    return out, time.perf_counter() - t
