"""VTK / VTU mesh and cell-data I/O (no GPU)."""
import numpy as np
import pytest

from mhfem import meshgen, vtkio

MESHES = {
    "triangles": lambda: meshgen.square_triangles(5),
    "tetrahedra": lambda: meshgen.cube_tetrahedra(3),
    "rectangles": lambda: meshgen.square_rectangles(5),
    "cuboids": lambda: meshgen.cube_cuboids(3),
}


@pytest.mark.parametrize("compress", [True, False])
@pytest.mark.parametrize("kind", sorted(MESHES))
def test_vtu_roundtrip(tmp_path, kind, compress):
    coords, cells = MESHES[kind]()
    z = np.random.default_rng(0).standard_normal(cells.shape[0])
    f = tmp_path / "m.vtu"
    vtkio.write_vtu(f, coords, cells, {"InitialCondition[Z0]": z, "Z": 2 * z}, time=0.5, cycle=3,
                    compress=compress)
    c2, k2 = vtkio.read_mesh(f)
    assert np.array_equal(c2, coords) and np.array_equal(k2, cells)
    assert np.array_equal(vtkio.read_cell_data(f, "InitialCondition[Z0]"), z)
    assert np.array_equal(vtkio.read_cell_data(f, "Z"), 2 * z)
    with pytest.raises(KeyError):
        vtkio.read_cell_data(f, "missing")


@pytest.mark.parametrize("kind", sorted(MESHES))
def test_legacy_vtk_roundtrip(tmp_path, kind):
    coords, cells = MESHES[kind]()
    f = tmp_path / "m.vtk"
    vtkio.write_legacy_vtk(f, coords, cells)
    c2, k2 = vtkio.read_mesh(f)
    assert np.allclose(c2, coords, rtol=0, atol=1e-15) and np.array_equal(k2, cells)


def _legacy_with_types(path, coords, cells, ctype):
    pts = np.zeros((coords.shape[0], 3))
    pts[:, :coords.shape[1]] = coords
    C, nv = cells.shape
    with open(path, "w") as fh:
        fh.write("# vtk DataFile Version 2.0\nt\nASCII\nDATASET UNSTRUCTURED_GRID\n")
        fh.write(f"POINTS {pts.shape[0]} double\n")
        np.savetxt(fh, pts, fmt="%.17g")
        fh.write(f"CELLS {C} {C * (nv + 1)}\n")
        np.savetxt(fh, np.hstack([np.full((C, 1), nv), cells]), fmt="%d")
        fh.write(f"CELL_TYPES {C}\n")
        np.savetxt(fh, np.full((C, 1), ctype), fmt="%d")


@pytest.mark.parametrize("kind", ["rectangles", "cuboids"])
def test_pixels_and_voxels_take_the_box_vertex_order(tmp_path, kind):
    """VTK pixels / voxels number their corners lexicographically; the reader
    returns them in the quadrilateral / hexahedron order the box cells use."""
    coords, cells = MESHES[kind]()
    lex = [0, 1, 3, 2] if kind == "rectangles" else [0, 1, 3, 2, 4, 5, 7, 6]
    f = tmp_path / "p.vtk"
    _legacy_with_types(f, coords, cells[:, lex], vtkio.VTK_PIXEL if kind == "rectangles" else vtkio.VTK_VOXEL)
    c2, k2 = vtkio.read_mesh(f)
    assert np.array_equal(k2, cells)


def test_mixed_cell_kinds_are_refused(tmp_path):
    coords, cells = meshgen.square_triangles(2)
    f = tmp_path / "x.vtk"
    _legacy_with_types(f, coords, cells, vtkio.VTK_QUAD)  # 3 vertices declared as quadrilaterals
    with pytest.raises(ValueError):
        vtkio.read_mesh(f)


@pytest.mark.parametrize("kind", ["triangles", "tetrahedra"])
def test_netgen_roundtrip(tmp_path, kind):
    coords, cells = MESHES[kind]()
    f = tmp_path / "m.ng"
    vtkio.write_netgen(f, coords, cells)
    c2, k2 = vtkio.read_mesh(f)
    assert np.allclose(c2, coords, rtol=0, atol=1e-15) and np.array_equal(k2, cells)


def test_netgen_reads_boundary_elements_and_rejects_bad_indices(tmp_path):
    f = tmp_path / "t.ng"
    # two triangles of the unit square, one boundary edge listed after the elements
    f.write_text("4\n0 0\n1 0\n1 1\n0 1\n2\n1 1 2 3\n1 1 3 4\n1\n1 1 2\n")
    c, k = vtkio.read_mesh(f)
    assert c.shape == (4, 2) and np.array_equal(k, [[0, 1, 2], [0, 2, 3]])
    f.write_text("3\n0 0\n1 0\n1 1\n1\n1 1 2 4\n")
    with pytest.raises(ValueError):
        vtkio.read_mesh(f)
