"""GPU: the reference's squeeze-flow driver end to end (examples/vector3D.jl:
266-343 with src/PostProcess.jl:30-44,281-304) through the library: mesh on
the device, inflate_sphere, assembly, surface penalty, load increments with
warm starts, VTK scene from device fields -- each step's displacement
against the oracle's dense-inverse solve of K + beta*b within 1e-8.
"""
import numpy as np
import pytest

from test_vtk import read_vtu

pytestmark = pytest.mark.gpu


def test_squeeze_driver(sfem, ctx, oracle, tmp_path):
    import torch
    ne, Young, nu, beta = 4, 40.0, 0.4, 100.0
    NL, IEN, ID, IT, IB = sfem.meshgrid(0, 1, 0, 1, 0, 1, ne, 3, device=True, ctx=ctx)
    cyl = NL.clone()
    sfem.inflate_sphere(cyl, 0, 1, 0, 1, ctx=ctx)
    K = sfem.assemble_system(ne, NL, IEN, 3, "Q1", 3, ID, Young, nu, ctx=ctx, as_handle=True)
    faces = torch.cat([IB, IT])
    K.add_penalty(cyl, faces, beta)
    NLh = NL.cpu().numpy()
    deltas = np.arange(0.001, 0.5, 0.01)[:6]
    fd, fv = sfem.meshgen.squeeze_increments(NLh, deltas)
    U, st = K.solve_increments(fd, fv, precision="fp64", precond="block_jacobi", rtol=1e-12)
    K.close()
    # oracle: the same driver on the host
    NLo, IENo, IDo, ITo, IBo = oracle.meshgrid_loops(0, 1, 0, 1, 0, 1, ne, 3)
    assert np.array_equal(NLh, NLo)
    Ko = oracle.assemble_system(ne, NLo, IENo, 3, "Q1", 3, IDo, Young, nu)
    bo = oracle.apply_boundary_conditions_loops(ne, oracle.inflate_sphere(NLo, 0, 1, 0, 1), IENo, ITo, IBo, 3,
                                                "Q1", IDo)
    Kb = oracle.add_scaled(Ko, beta, bo).tocsc()
    Kb.sort_indices()
    Kb = (Kb.indptr + 1, Kb.indices + 1, Kb.data, Kb.shape[0], Kb.shape[1])
    motions = []
    for k in range(len(deltas)):
        q_d, rcol = oracle.set_boundary_cond(NLo, ne, 3, deltas[k], 3)
        ref = oracle.solve_eliminated(Kb, rcol, q_d[rcol - 1], method="inv")
        assert np.linalg.norm(U[k] - ref) / np.linalg.norm(ref) <= 1e-8, (k, st[k])
        motions.append(np.stack([U[k][IDo[:, c] - 1] for c in range(3)]))   # motion = [q[ID[:,1]] ...]'
    # the scene: first field the cylinder coordinates, then the motions (device fields)
    fields = torch.tensor(np.stack([cyl.cpu().numpy()] + motions), device=NL.device)
    base = str(tmp_path / "squeeze_flow")
    sfem.write_scene(base, NL, IEN, ne, 3, fields)
    for k in range(len(deltas) + 1):
        _, _, a = read_vtu(f"{base}timestep_{k + 1}.vtu")
        expect = cyl.cpu().numpy() if k == 0 else motions[k - 1]
        assert np.array_equal(a["u"], expect.T) and np.array_equal(a["Points"], NLh.T)
    assert open(base + "displacement.pvd").read().count("<DataSet") == len(deltas) + 1
