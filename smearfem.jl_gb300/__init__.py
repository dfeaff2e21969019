"""smearfem_gb300: the smearFEM.jl hot path (Q1/Q2 assembly, Dirichlet
elimination, PCG solve) on one NVIDIA GB300, behind the reference's API.

The compute lives in libsmearfem_gpu.so (csrc/, C ABI in
include/smearfem_gpu.h); this package is the host-side mirror of the
reference's Julia calling surface plus the seeded mesh generators.
"""
from ._lib import SfemError, lib  # noqa: F401
from .fem import (Batch, Context, Matrix, Mesh, Server, apply_boundary_conditions,  # noqa: F401
                  assemble_system, basis_function, gaussian_quadrature, get_context,
                  inflate_sphere, meshgrid, multigrid_info, solve_dirichlet, version, write_scene,
                  write_vtk)
from . import meshgen  # noqa: F401
