"""Generate the committed golden fixtures under tests/golden/.

    python tests/golden/make_golden.py            # small meshes (seconds)
    python tests/golden/make_golden.py --cube20   # + 20^3 dense-inverse solve (minutes, ~16 GB RAM)

Every fixture comes from the NumPy restatement of the reference
(oracle/fem_ref.py): the loop form of ``assemble_system`` (src/fem.jl:135-256)
for the small meshes, and for the 20^3 unit cube the reference's own solve
algorithm, ``inv(Matrix(K_free))`` (examples/vector3D.jl:315-322).  The
reference's Julia code cannot run here, so these vectors are restatement
outputs, not reference outputs; they pin the oracle and the GPU path against
regressions and carry the dense-inverse displacement that the GPU solve must
match to 1e-8.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "smearfem.jl_gb300"))

from oracle import fem_ref as R  # noqa: E402
import meshgen as M  # noqa: E402

# name: (ndim, ne, FunctionClass, nDof, plane, jitter, per-element E)
SMALL = {
    "lap2d_1": (2, 1, "Q1", 1, "stress", 0.0, False),
    "lap2d_2": (2, 2, "Q1", 1, "stress", 0.2, False),
    "lap3d_1": (3, 1, "Q1", 1, "stress", 0.0, False),
    "lap3d_2": (3, 2, "Q1", 1, "stress", 0.2, False),
    "el2d_1": (2, 1, "Q1", 2, "stress", 0.0, False),
    "el2d_2": (2, 2, "Q1", 2, "stress", 0.2, True),
    "el2d_3_strain": (2, 3, "Q1", 2, "strain", 0.2, True),
    "el3d_1": (3, 1, "Q1", 3, "stress", 0.0, False),
    "el3d_2": (3, 2, "Q1", 3, "stress", 0.2, True),
    "el3d_3": (3, 3, "Q1", 3, "stress", 0.2, True),
}


def small_case(name):
    ndim, ne, fc, nDof, plane, jit, pere = SMALL[name]
    rng = np.random.default_rng(7 + ne * 10 + ndim)
    NL, IEN, ID, _, _ = M.meshgrid(0, 1, 0, 1, 0, 1, ne, ndim)
    if jit:
        NL = M.jitter_interior(NL, ne, jit, rng)
    Y = np.exp(rng.normal(0, 0.5, ne ** ndim)) if pere else np.array(1.0)
    nu = 0.3
    return dict(ndim=ndim, ne=ne, fclass=fc, nDof=nDof, plane=plane, NodeList=NL, IEN=IEN,
                ID=ID, Young=np.atleast_1d(Y), nu=np.atleast_1d(nu))


def make_small():
    for name in SMALL:
        c = small_case(name)
        Y = c["Young"] if c["Young"].size > 1 else float(c["Young"][0])
        colptr, rowval, nzval, m, n = R.assemble_system_loops(
            c["ne"], c["NodeList"], c["IEN"], c["ndim"], c["fclass"], c["nDof"], c["ID"],
            Y, float(c["nu"][0]), c["plane"])
        np.savez_compressed(os.path.join(HERE, f"{name}.npz"), colptr=colptr, rowval=rowval,
                            nzval=nzval, m=m, n=n, **{k: v for k, v in c.items()
                                                      if isinstance(v, np.ndarray)},
                            meta=np.array([c["ndim"], c["ne"], c["nDof"]]),
                            fclass=c["fclass"], plane=c["plane"])
        print(name, m, len(nzval))


def make_cube20():
    p = M.parity_cube20()
    K = R.assemble_system(p.ne, p.NodeList, p.IEN, 3, "Q1", 3, p.ID, 1.0, 0.3)
    u = R.solve_eliminated(K, p.fixed_dofs, p.fixed_vals, method="inv")
    colptr, rowval, nzval, m, n = K
    np.savez_compressed(os.path.join(HERE, "cube20_dense_inv.npz"), u=u,
                        nnz=len(nzval), n=n, nzsum=nzval.sum(), nzabs=np.abs(nzval).sum(),
                        rowsum=np.int64(rowval.sum()), colptr_sum=np.int64(colptr.sum()))
    print("cube20", n, len(nzval), np.linalg.norm(u))


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--cube20", action="store_true")
    a = ap.parse_args()
    make_small()
    if a.cube20:
        make_cube20()
