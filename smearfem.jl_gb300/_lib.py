"""ctypes binding of libsmearfem_gpu.so (include/smearfem_gpu.h).

The library is the product: there is no CPU fallback.  If the shared object
is missing, :func:`lib` raises with the build command; if no GPU is usable,
``sfem_ctx_create`` fails and :class:`SfemError` is raised.
"""
from __future__ import annotations

import ctypes as C
import os

PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG, "lib", "libsmearfem_gpu.so")

SFEM_OK, SFEM_BAD_ARG, SFEM_BAD_INDEX, SFEM_SINGULAR_JACOBIAN, SFEM_OOM = 0, 1, 2, 3, 4
SFEM_NOT_CONVERGED, SFEM_CUDA_ERROR, SFEM_SINGULAR, SFEM_UNSUPPORTED = 5, 6, 7, 8
SFEM_TIMEOUT = 9
STATUS_NAMES = {0: "SFEM_OK", 1: "SFEM_BAD_ARG", 2: "SFEM_BAD_INDEX", 3: "SFEM_SINGULAR_JACOBIAN",
                4: "SFEM_OOM", 5: "SFEM_NOT_CONVERGED", 6: "SFEM_CUDA_ERROR", 7: "SFEM_SINGULAR",
                8: "SFEM_UNSUPPORTED", 9: "SFEM_TIMEOUT"}
MEM_HOST, MEM_DEVICE = 0, 1
Q1, Q2 = 1, 2
PLANE_STRESS, PLANE_STRAIN = 0, 1
FP64, MIXED = 0, 1
PC_JACOBI, PC_BLOCK_JACOBI, PC_MULTIGRID = 0, 1, 2
FP32_UPPER, FP32_FULL = 0, 1


class SfemError(RuntimeError):
    """A non-OK sfem_status; ``code`` holds the status value."""

    def __init__(self, code, msg):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class SolveOpts(C.Structure):
    _fields_ = [("precision", C.c_int), ("precond", C.c_int), ("rtol", C.c_double),
                ("maxit", C.c_int), ("check_every", C.c_int), ("reliable_delta", C.c_double),
                ("profile", C.c_int), ("fp32_storage", C.c_int)]


class SolveStats(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("reliable_updates", C.c_int),
                ("relres", C.c_double), ("ms_total", C.c_double), ("ms_spmv", C.c_double),
                ("spmv_launches", C.c_int), ("kernel_launches", C.c_int), ("n_free", C.c_int64)]

    def as_dict(self):
        return {k: getattr(self, k) for k, _ in self._fields_}


class BatchStats(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("refreshes", C.c_int),
                ("group_ctas", C.c_int), ("relres", C.c_double), ("ms", C.c_double)]


class ServerConfig(C.Structure):
    _fields_ = [("cluster", C.c_int), ("threads", C.c_int), ("sm_fraction", C.c_double),
                ("hbm_budget_fraction", C.c_double), ("hbm_budget_bytes", C.c_int64),
                ("max_inflight", C.c_int), ("idle_exit_ms", C.c_double), ("solve", SolveOpts),
                ("warm_start", C.c_int)]


class ServerResult(C.Structure):
    _fields_ = [("status", C.c_int), ("iterations", C.c_int), ("refreshes", C.c_int),
                ("relres", C.c_double), ("queue_ms", C.c_double), ("gpu_ms", C.c_double),
                ("total_ms", C.c_double), ("ndof", C.c_int64), ("t_claim_ms", C.c_double),
                ("t_end_ms", C.c_double), ("smid", C.c_int)]


class ServerTotals(C.Structure):
    _fields_ = [("completed", C.c_int64), ("pending", C.c_int64), ("inflight", C.c_int64),
                ("peak_inflight", C.c_int64), ("kernel_launches", C.c_int64),
                ("bytes_in_use", C.c_int64), ("peak_bytes", C.c_int64), ("budget_bytes", C.c_int64),
                ("topologies", C.c_int64), ("grid", C.c_int), ("cluster", C.c_int),
                ("last_error", C.c_int)]


_lib = None

P = C.c_void_p
PP = C.POINTER(C.c_void_p)
I64 = C.c_int64
I64P = C.POINTER(C.c_int64)

# name: (restype, argtypes) -- mirrors include/smearfem_gpu.h
SIGNATURES = {
    "sfem_ctx_create": (C.c_int, [C.c_int, PP]),
    "sfem_ctx_destroy": (C.c_int, [P]),
    "sfem_last_error": (C.c_char_p, [P]),
    "sfem_ctx_synchronize": (C.c_int, [P]),
    "sfem_version": (C.c_char_p, []),
    "sfem_ctx_stream": (C.c_void_p, [P]),
    "sfem_ctx_kernel_launches": (C.c_int64, [P]),
    "sfem_gaussian_quadrature": (C.c_int, [C.c_double, C.c_double, C.c_int, P, P]),
    "sfem_basis_function": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, C.c_double, P, P]),
    "sfem_mesh_create": (C.c_int, [P, C.c_int, C.c_int, C.c_int, I64, P, I64, P, I64, C.c_int, P,
                                   C.c_int, PP]),
    "sfem_mesh_destroy": (C.c_int, [P]),
    "sfem_pattern_build": (C.c_int, [P, P, I64P, I64P]),
    "sfem_assemble": (C.c_int, [P, P, C.c_int, P, I64, P, I64, C.c_int, PP]),
    "sfem_assemble_system": (C.c_int, [P, I64, P, I64, P, I64, C.c_int, C.c_int, C.c_int, C.c_int,
                                       P, P, I64, P, I64, C.c_int, C.c_int, PP, I64P, I64P]),
    "sfem_reassemble_noalloc": (C.c_int, [P, P, P, I64, P, I64, C.c_int]),
    "sfem_matrix_info": (C.c_int, [P, I64P, I64P]),
    "sfem_matrix_export_csc": (C.c_int, [P, P, P, P, P, C.c_int]),
    "sfem_matrix_destroy": (C.c_int, [P]),
    "sfem_solve_opts_default": (None, [C.POINTER(SolveOpts)]),
    "sfem_batch_create": (C.c_int, [P, C.c_int, C.c_int, C.c_int, I64, P, P, P, P, P, C.c_int, PP]),
    "sfem_batch_info": (C.c_int, [P, I64P, I64P, I64P]),
    "sfem_batch_set_launch": (C.c_int, [P, C.c_int, C.c_int, C.c_int, I64]),
    "sfem_batch_solve": (C.c_int, [P, P, C.c_int, P, I64, P, I64, P, P, P, P, C.c_int,
                                   C.POINTER(SolveOpts), P]),
    "sfem_batch_autotune": (C.c_int, [P, P, C.c_int, P, I64, P, I64, P, P, P, C.c_int,
                                      C.POINTER(SolveOpts), I64, C.POINTER(C.c_double)]),
    "sfem_batch_get_launch": (C.c_int, [P, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                        C.POINTER(C.c_int), I64P, C.POINTER(C.c_int)]),
    "sfem_batch_destroy": (C.c_int, [P]),
    "sfem_multigrid_info": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int64, I64P, C.c_int64,
                                      C.POINTER(C.c_int), C.POINTER(C.c_int), I64P]),
    "sfem_solve_dirichlet": (C.c_int, [P, P, P, I64, P, P, P, C.c_int, C.POINTER(SolveOpts),
                                       C.POINTER(SolveStats)]),
    "sfem_penalty_add": (C.c_int, [P, P, P, P, I64, C.c_int, C.c_double, C.c_int]),
    "sfem_vtk_write": (C.c_int, [P, C.c_char_p, P, C.c_int, I64, P, I64, C.c_int, C.c_char_p, P, C.c_int,
                                 C.c_int]),
    "sfem_vtk_write_scene": (C.c_int, [P, C.c_char_p, P, C.c_int, I64, P, I64, C.c_int, P, C.c_int, I64,
                                       C.c_int]),
    "sfem_meshgrid": (C.c_int, [P, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double, C.c_double,
                                I64, C.c_int, P, P, P, P, P, C.c_int]),
    "sfem_inflate_sphere": (C.c_int, [P, P, C.c_int, I64, C.c_double, C.c_double, C.c_double, C.c_double,
                                      C.c_int]),
    "sfem_solve_increments": (C.c_int, [P, P, P, I64, P, I64, P, P, C.c_int, C.POINTER(SolveOpts), C.c_int,
                                        P]),
    "sfem_server_config_default": (None, [C.POINTER(ServerConfig)]),
    "sfem_server_create": (C.c_int, [C.c_int, C.POINTER(ServerConfig), PP]),
    "sfem_server_submit": (C.c_int, [P, C.c_int, C.c_int, C.c_int, C.c_int, I64, P, I64, P, I64, P,
                                     P, I64, P, I64, P, I64, P, I64P]),
    "sfem_server_wait": (C.c_int, [P, I64, C.c_double, P, I64, C.POINTER(ServerResult)]),
    "sfem_server_info": (C.c_int, [P, C.POINTER(ServerTotals)]),
    "sfem_server_destroy": (C.c_int, [P]),
}


def lib():
    """Load the shared library (raises if it has not been built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing; build it with "
                               "`python smearfem.jl_gb300/build.py` (nvcc, sm_103a)")
        L = C.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _lib = L
    return _lib


def check(code, ctx=None):
    if code != SFEM_OK:
        msg = lib().sfem_last_error(ctx).decode() if ctx else ""
        raise SfemError(code, msg)
