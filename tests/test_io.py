"""On-disk formats (host only): PETSc binary vectors byte for byte as VecDump writes them on one process
(big-endian class id 1211214, size, doubles), forest files and the save/load folder layout of
my_p4est_save_forest_and_data round-trip exactly, and the VTK files describe the grid (points = node
coordinates, pixel/voxel cells = leaf corner nodes) and carry the fields exactly in ascii and binary."""
import base64
import os
import xml.etree.ElementTree as ET

import numpy as np
import pytest

import casl_p4est_gb300 as G
from grids import brick_2d, brick_3d, circle_2d, flower_3d


@pytest.mark.parametrize("int64", [False, True])
def test_vecdump_bytes(tmp_path, int64):
    a = np.linspace(-1.5, 2.25, 37)
    b = np.sin(np.arange(37.0))
    fn = str(tmp_path / "phi.petscbin")
    G.VecDump(fn, [a, b], petsc_int64=int64)
    raw = open(fn, "rb").read()
    hdr = 12 if int64 else 8
    rec = hdr + 37 * 8
    assert len(raw) == 2 * rec
    for k, v in enumerate((a, b)):
        r = raw[k * rec:(k + 1) * rec]
        assert np.frombuffer(r[:4], ">i4")[0] == 1211214
        assert np.frombuffer(r[4:hdr], ">i8" if int64 else ">i4")[0] == 37
        assert np.array_equal(np.frombuffer(r[hdr:], ">f8"), v)
    got = G.VecLoad(fn, 37, 2, petsc_int64=int64)
    assert np.array_equal(got[0], a) and np.array_equal(got[1], b)
    with pytest.raises(G.LsgInvalidArgument):
        G.VecLoad(fn, 36, 1, petsc_int64=int64)


@pytest.mark.parametrize("make", [lambda: circle_2d(2, 6), lambda: brick_3d(1, 4)])
def test_forest_and_data_round_trip(tmp_path, make):
    f = make()
    phi = np.cos(f.node_xyz()[:, 0])
    G.my_p4est_save_forest_and_data(str(tmp_path), f, "grid.forest", [("phi", [phi]), ("two", [phi, 2 * phi])])
    assert sorted(os.listdir(tmp_path)) == ["grid.forest", "phi.petscbin", "two.petscbin"]
    g, data = G.my_p4est_load_forest_and_data(str(tmp_path), "grid.forest", [("phi", 1), ("two", 2)])
    for x, y in zip(f.leaves(), g.leaves()):
        assert np.array_equal(x, y)
    assert np.array_equal(g.node_xyz(), f.node_xyz()) and g.n_xyz == f.n_xyz and g.xyz_min == f.xyz_min
    assert np.array_equal(data["phi"][0], phi) and np.array_equal(data["two"][1], 2 * phi)
    with pytest.raises(ValueError):
        G.my_p4est_save_forest_and_data(str(tmp_path / "missing"), f, "g", [])


def read_array(el):
    fmt, typ = el.get("format"), el.get("type")
    dt = {"Float64": "<f8", "Int32": "<i4", "UInt8": "u1"}[typ]
    if fmt == "ascii":
        return np.array(el.text.split(), dtype=np.float64 if typ == "Float64" else np.int64).astype(dt)
    raw = base64.b64decode(el.text.strip())
    n = np.frombuffer(raw[:4], "<u4")[0]
    return np.frombuffer(raw[4:4 + n], dt)


@pytest.mark.parametrize("binary", [False, True])
@pytest.mark.parametrize("make", [lambda: brick_2d(1, 5), lambda: flower_3d(2, 4)])
def test_vtk_files(tmp_path, make, binary):
    f = make()
    x = f.node_xyz()
    phi = np.sqrt(np.sum(x ** 2, axis=1)) - 0.5
    lvl = f.leaves()[1].astype(np.float64)
    name = str(tmp_path / "out")
    G.my_p4est_vtk_write_all(f, name, {"phi": phi, "x": x[:, 0]}, {"level": lvl}, binary=binary)
    piece = ET.parse(name + ".vtu/0000.vtu").getroot().find("UnstructuredGrid/Piece")
    assert int(piece.get("NumberOfPoints")) == f.num_nodes and int(piece.get("NumberOfCells")) == f.num_leaves
    arr = {e.get("Name"): read_array(e) for e in piece.iter("DataArray")}
    pos = arr["Position"].reshape(-1, 3)
    assert np.array_equal(pos[:, :f.dim], x) and (f.dim == 3 or np.all(pos[:, 2] == 0))
    ch = 1 << f.dim
    assert np.array_equal(arr["connectivity"].reshape(-1, ch), f.local_nodes())
    assert np.array_equal(arr["offsets"], ch * np.arange(1, f.num_leaves + 1))
    assert np.all(arr["types"] == (11 if f.dim == 3 else 8))
    assert np.array_equal(arr["phi"], phi) and np.array_equal(arr["x"], x[:, 0])
    assert np.array_equal(arr["level"], lvl) and np.array_equal(arr["tree_idx"], f.leaves()[0])
    master = ET.parse(name + ".pvtu").getroot()
    assert master.find("PUnstructuredGrid/Piece").get("Source") == "out.vtu/0000.vtu"
    names = [e.get("Name") for e in master.iter("PDataArray")]
    assert names == ["Position", "phi", "x", "proc_rank", "tree_idx", "level"]
