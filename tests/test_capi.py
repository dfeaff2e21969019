"""CPU: the C-ABI library builds for sm_103a, loads, and exports exactly what
include/*.h declares; the host-side helpers reproduce the reference's known
answers.  No kernel runs here."""
import ctypes
import glob
import math
import os
import re
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        txt = open(h).read()
        names |= set(re.findall(r"SFEM_API[^;(]*?\b(sfem_\w+)\s*\(", txt, flags=re.S))
    return names


def test_header_declares_entry_points():
    names = declared_symbols()
    for required in ("sfem_ctx_create", "sfem_assemble_system", "sfem_matrix_export_csc",
                     "sfem_solve_dirichlet", "sfem_gaussian_quadrature", "sfem_basis_function"):
        assert required in names


def test_library_exports_every_declared_symbol(sfem):
    path = sfem._lib.LIB_PATH
    lib = ctypes.CDLL(path)
    for name in declared_symbols():
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", path], capture_output=True, text=True).stdout
    exported = set(re.findall(r"\bT (sfem_\w+)", out))
    assert exported == declared_symbols()
    assert set(sfem._lib.SIGNATURES) == declared_symbols()


def test_header_compiles_as_c(tmp_path):
    src = tmp_path / "t.c"
    src.write_text('#include "smearfem_gpu.h"\nint main(void){sfem_solve_opts o; '
                   'sfem_solve_opts_default(&o); return o.maxit > 0 ? 0 : 1;}\n')
    subprocess.check_call(["gcc", "-std=c99", "-Wall", "-Werror", "-fsyntax-only",
                           "-I", os.path.join(ROOT, "include"), str(src)])


def test_reference_kats_through_library(sfem):
    """test/runtests.jl:15-35 against the library's host helpers (exact ==)."""
    bf, gq = sfem.basis_function, sfem.gaussian_quadrature
    assert list(bf(-1)[0]) == [1.0, 0.0] and list(bf(1)[0]) == [0.0, 1.0]
    for i, c in enumerate([(-1, -1), (1, -1), (1, 1), (-1, 1)]):
        assert list(bf(*c)[0]) == list(np.eye(4)[i])
    for i, c in enumerate([(-1, -1, -1), (1, -1, -1), (1, 1, -1), (-1, 1, -1),
                           (-1, -1, 1), (1, -1, 1), (1, 1, 1), (-1, 1, 1)]):
        assert list(bf(*c)[0]) == list(np.eye(8)[i])
    xi, w = gq(-1, 1, 2)
    assert list(xi) == [-1 / math.sqrt(3), 1 / math.sqrt(3)] and list(w) == [1.0, 1.0]
    xi, w = gq(-1, 1, 3)
    assert list(xi) == [-math.sqrt(3 / 5), 0.0, math.sqrt(3 / 5)] and list(w) == [5 / 9, 8 / 9, 5 / 9]


def test_library_helpers_match_oracle_bitwise(sfem, oracle):
    rng = np.random.default_rng(1)
    for _ in range(50):
        x, y, z = rng.uniform(-1, 1, 3)
        for args, fc in (((x, y, z), "Q1"), ((x, y), "Q1"), ((x, y), "Q2"), ((x,), "Q1")):
            a = sfem.basis_function(*args, FunctionClass=fc)
            b = oracle.basis_function(*args, FunctionClass=fc)
            assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    for a, b in ((-1, 1), (0, 2), (-0.3, 0.7)):
        for n in (2, 3):
            assert all(np.array_equal(u, v) for u, v in zip(sfem.gaussian_quadrature(a, b, n),
                                                            oracle.gaussian_quadrature(a, b, n)))


def test_no_gpu_fails_loudly(sfem):
    """Without a usable GPU the product refuses to run (no CPU fallback)."""
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(sfem.SfemError):
        sfem.Context(0)
    with pytest.raises(sfem.SfemError):
        sfem.Server()
    with pytest.raises(KeyError):
        sfem.Server(precision="fp16")


def test_missing_library_is_an_error(sfem, monkeypatch, tmp_path):
    from smearfem_gb300 import _lib
    monkeypatch.setattr(_lib, "_lib", None)
    monkeypatch.setattr(_lib, "LIB_PATH", str(tmp_path / "nope.so"))
    with pytest.raises(RuntimeError, match="missing"):
        _lib.lib()


def test_argument_validation_without_gpu(sfem):
    with pytest.raises(sfem.SfemError):
        sfem.gaussian_quadrature(-1, 1, 4)
    with pytest.raises(sfem.SfemError):
        sfem.basis_function(0.1, FunctionClass="Q2")
