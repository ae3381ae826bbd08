"""Mesh files: Gmsh MSH 2.2 / 4.1 and legacy VTK read into meshio's layout (``points``,
``cells_dict``, ``cell_data_dict``), the way AutoPDEx's examples use meshio's result
(examples/cooks_membrane/quadrilaterals_autopdex_and_acegen.py:62-65).  The files are small
ones written here by hand (non-contiguous node tags, several blocks, physical groups)."""
import numpy as np
import pytest

from autopdex_gb300 import mesh_io, mesher

MSH22 = """$MeshFormat
2.2 0 8
$EndMeshFormat
$PhysicalNames
2
1 7 "left"
2 9 "domain"
$EndPhysicalNames
$Nodes
6
10 0 0 0
11 1 0 0
12 2 0 0
20 0 1 0
21 1 1 0
22 2 1 0
$EndNodes
$Elements
4
1 1 2 7 3 10 20
2 3 2 9 1 10 11 21 20
3 3 2 9 1 11 12 22 21
4 1 0 12 22
$EndElements
"""

MSH41 = """$MeshFormat
4.1 0 8
$EndMeshFormat
$Entities
2 1 1 0
1 0 0 0 0
2 0 1 0 1 5
1 0 0 0 0 1 0 1 7 2 1 -2
1 0 0 0 2 1 0 1 9 1 1
$EndEntities
$Nodes
2 6 1 6
1 1 0 2
1
4
0 0 0
0 1 0
2 1 0 4
2
3
5
6
1 0 0
2 0 0
1 1 0
2 1 0
$EndNodes
$Elements
2 3 1 3
1 1 1 1
1 1 4
2 1 3 2
2 1 2 5 4
3 2 3 6 5
$EndElements
"""

VTK51 = """# vtk DataFile Version 5.1
two cells
ASCII
DATASET UNSTRUCTURED_GRID
POINTS 4 float
0 0 0 1 0 0 1 1 0 0 1 0
CELLS 3 6
OFFSETS vtktypeint64
0 4 6
CONNECTIVITY vtktypeint64
0 1 2 3 0 3
CELL_TYPES 2
9
3
POINT_DATA 4
SCALARS T double 1
LOOKUP_TABLE default
0 1 2 3
"""


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_gmsh_22(tmp_path):
    m = mesh_io.read(_write(tmp_path, "a.msh", MSH22))
    assert np.array_equal(m.points[:, :2], [[0, 0], [1, 0], [2, 0], [0, 1], [1, 1], [2, 1]])
    cd = m.cells_dict
    assert np.array_equal(cd["quad"], [[0, 1, 4, 3], [1, 2, 5, 4]])
    assert np.array_equal(cd["line"], [[0, 3], [2, 5]])
    phys = m.cell_data_dict["gmsh:physical"]
    assert np.array_equal(phys["line"], [7, 0]) and np.array_equal(phys["quad"], [9, 9])
    assert np.array_equal(m.cell_data_dict["gmsh:geometrical"]["line"], [3, 0])
    assert np.array_equal(m.field_data["left"], [7, 1]) and np.array_equal(m.field_data["domain"], [9, 2])


def test_gmsh_41(tmp_path):
    m = mesh_io.read(_write(tmp_path, "b.msh", MSH41))
    assert np.array_equal(m.points[:, :2], [[0, 0], [0, 1], [1, 0], [2, 0], [1, 1], [2, 1]])
    cd = m.cells_dict
    assert np.array_equal(cd["line"], [[0, 1]])
    assert np.array_equal(cd["quad"], [[0, 2, 4, 1], [2, 3, 5, 4]])
    phys = m.cell_data_dict["gmsh:physical"]
    assert np.array_equal(phys["line"], [7]) and np.array_equal(phys["quad"], [9, 9])


def test_gmsh_binary_rejected(tmp_path):
    p = _write(tmp_path, "c.msh", "$MeshFormat\n4.1 1 8\n$EndMeshFormat\n")
    with pytest.raises(NotImplementedError):
        mesh_io.read(p)


def test_vtk_51(tmp_path):
    m = mesh_io.read(_write(tmp_path, "d.vtk", VTK51))
    assert np.array_equal(m.cells_dict["quad"], [[0, 1, 2, 3]])
    assert np.array_equal(m.cells_dict["line"], [[0, 3]])
    assert np.array_equal(m.point_data["T"], [0, 1, 2, 3])


def test_vtk_round_trip(tmp_path):
    """A structured quad mesh with its boundary lines, a scalar and a 2-vector field."""
    coords, elems = mesher.structured_mesh((5, 4), [[0., 0.], [48., 44.], [48., 60.], [0., 44.]], "quad")
    lines = np.array([[i, i + 1] for i in range(4)])
    T = np.linspace(0.0, 1.0, coords.shape[0])
    u = np.stack([T, -T], axis=1)
    p = str(tmp_path / "e.vtk")
    mesh_io.write_vtk(p, coords, {"quad": elems, "line": lines}, point_data={"T": T, "u": u},
                      cell_data={"k": np.arange(elems.shape[0] + lines.shape[0], dtype=float)})
    m = mesh_io.read(p)
    assert np.array_equal(m.points[:, :2], coords) and np.all(m.points[:, 2] == 0)
    assert np.array_equal(m.cells_dict["quad"], elems) and np.array_equal(m.cells_dict["line"], lines)
    assert np.array_equal(m.point_data["T"], T)
    assert np.array_equal(m.point_data["u"][:, :2], u)
    assert np.array_equal(m.cell_data_dict["k"]["quad"], np.arange(elems.shape[0]))


def test_gmsh_write_read(tmp_path):
    coords, elems = mesher.structured_mesh((3, 2), [[0., 0.], [1., 0.], [1., 1.], [0., 1.]], "quad")
    lines = np.array([[0, 1], [1, 2]])
    p = str(tmp_path / "f.msh")
    mesh_io.write_gmsh(p, coords, [("quad", elems[::-1]), ("line", lines)])
    m = mesh_io.read(p)
    assert np.array_equal(m.points[:, :2], coords)
    assert np.array_equal(m.cells_dict["quad"], elems[::-1]) and np.array_equal(m.cells_dict["line"], lines)
