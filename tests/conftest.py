import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

import __graft_entry__ as GE  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs the GB300 kernels)")


@pytest.fixture(scope="session")
def sfem():
    """The package, with libsmearfem_gpu.so built (nvcc cross-compiles without a GPU)."""
    mod = GE._build_module()
    mod.build()
    return GE.load_package()


@pytest.fixture(scope="session")
def ctx(sfem):
    return sfem.get_context(0)


@pytest.fixture(scope="session")
def oracle():
    from oracle import coracle, fem_ref
    coracle.build()
    return fem_ref


@pytest.fixture(scope="session")
def coracle():
    from oracle import coracle as co
    co.build()
    return co


def rowscaled_err(K_ref_csc, nzval, rowval):
    """max |K_ij - K_ij^ref| / max_k |K_ik^ref| over stored entries (1-based rowval)."""
    import scipy.sparse as sp
    colptr, rv, nz, m, n = K_ref_csc
    A = sp.csc_matrix((nz, rv - 1, colptr - 1), shape=(m, n))
    rowmax = np.asarray(abs(A).max(axis=1).todense()).ravel()
    rowmax[rowmax == 0] = 1.0
    return float(np.max(np.abs(nzval - nz) / rowmax[rowval - 1])) if nz.size else 0.0
