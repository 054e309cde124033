"""VTK / VTU mesh and cell-data I/O (no GPU)."""
import numpy as np
import pytest

from mhfem import meshgen, vtkio


@pytest.mark.parametrize("compress", [True, False])
@pytest.mark.parametrize("dim", [2, 3])
def test_vtu_roundtrip(tmp_path, dim, compress):
    coords, cells = meshgen.square_triangles(5) if dim == 2 else meshgen.cube_tetrahedra(3)
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


@pytest.mark.parametrize("dim", [2, 3])
def test_legacy_vtk_roundtrip(tmp_path, dim):
    coords, cells = meshgen.square_triangles(4) if dim == 2 else meshgen.cube_tetrahedra(2)
    f = tmp_path / "m.vtk"
    vtkio.write_legacy_vtk(f, coords, cells)
    c2, k2 = vtkio.read_mesh(f)
    assert np.allclose(c2, coords, rtol=0, atol=1e-15) and np.array_equal(k2, cells)
