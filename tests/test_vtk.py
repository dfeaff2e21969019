"""VTK output (src/PostProcess.jl:258-304) written from host arrays, without
a GPU, and read back: points, cells, types and the point field must be the
inputs exactly; the collection file lists the steps at times 0, 1, ...
"""
import re
import xml.etree.ElementTree as ET

import numpy as np
import pytest


def read_vtu(path):
    data = open(path, "rb").read()
    head, _, app = data.partition(b'<AppendedData encoding="raw">\n_')
    root = ET.fromstring(head.decode() + "</VTKFile>" if b"</VTKFile>" not in head else head.decode())
    arrays = {}
    types = {"Float64": np.float64, "Int64": np.int64, "UInt8": np.uint8}
    for da in root.iter("DataArray"):
        off = int(da.get("offset"))
        nbytes = int(np.frombuffer(app[off:off + 8], np.uint64)[0])
        a = np.frombuffer(app[off + 8:off + 8 + nbytes], types[da.get("type")])
        nc = int(da.get("NumberOfComponents", "1"))
        arrays[da.get("Name")] = a.reshape(-1, nc) if nc > 1 else a
    piece = next(root.iter("Piece"))
    return int(piece.get("NumberOfPoints")), int(piece.get("NumberOfCells")), arrays


def test_write_vtk_hex_vector_field(sfem, tmp_path):
    NL, IEN, ID, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 2, 0, 1, 3, 3)
    motion = np.random.default_rng(0).normal(size=(3, NL.shape[1]))
    sfem.write_vtk(tmp_path / "cube", "u", NL, IEN, 3, 3, motion)
    nP, nC, a = read_vtu(tmp_path / "cube.vtu")
    assert (nP, nC) == (NL.shape[1], 27)
    assert np.array_equal(a["Points"], NL.T)
    assert np.array_equal(a["connectivity"].reshape(27, 8), IEN - 1)
    assert np.array_equal(a["offsets"], 8 * np.arange(1, 28)) and np.all(a["types"] == 12)
    assert np.array_equal(a["u"], motion.T)


def test_write_vtk_quad_scalar_field_2d(sfem, tmp_path):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 0, 4, 2)
    q = np.linspace(0, 1, NL.shape[1])
    sfem.write_vtk(tmp_path / "sq", "temperature", NL, IEN, 4, 2, q)
    nP, nC, a = read_vtu(tmp_path / "sq.vtu")
    assert nC == 16 and np.all(a["types"] == 9)
    assert np.array_equal(a["Points"][:, :2], NL.T) and np.all(a["Points"][:, 2] == 0)
    assert np.array_equal(a["temperature"], q)


def test_write_scene_collection(sfem, tmp_path):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, 2, 3)
    fields = [np.full((3, NL.shape[1]), float(k)) for k in range(4)]
    base = str(tmp_path / "squeeze_flow")
    sfem.write_scene(base, NL, IEN, 2, 3, fields)
    pvd = open(base + "displacement.pvd").read()
    steps = re.findall(r'timestep="(\d+)" part="0" file="([^"]+)"', pvd)
    assert steps == [(str(k), f"squeeze_flowtimestep_{k + 1}.vtu") for k in range(4)]
    for k in range(4):
        _, _, a = read_vtu(f"{base}timestep_{k + 1}.vtu")
        assert np.all(a["u"] == float(k)) and np.array_equal(a["Points"], NL.T)


def test_vtk_argument_errors(sfem, tmp_path):
    NL, IEN, _, _, _ = sfem.meshgen.meshgrid(0, 1, 0, 1, 0, 1, 2, 3)
    with pytest.raises(sfem.SfemError):
        sfem.write_vtk(tmp_path / "x", "u", NL, IEN, 2, 3, np.zeros(5))          # wrong field length
    with pytest.raises(sfem.SfemError):
        sfem.write_vtk(tmp_path / "no_such_dir" / "x", "u", NL, IEN, 2, 3, np.zeros(NL.shape[1]))
