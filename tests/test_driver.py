"""config.ini driver, boundary-condition storage and the init step."""
import struct

import numpy as np
import pytest

from helpers import rel_err
from mhfem import bcstorage, config, init, meshgen, vtkio

CONFIG = """output-directory = out
mesh = mesh.vtu
boundary-conditions-file = boundary.bcs
initial-condition = initial.vtu
initial-time = 0
final-time = 0.003
snapshot-period = 0.001
time-step = 0.0005
linear-solver = gmres
gmres-variant = CGS
gmres-restarting-max = 30
preconditioner = diagonal
convergence-residue = 1e-12
diffusivity = 1e-3
"""


def _write_case(tmp_path, N=6, box=False):
    coords, cells = meshgen.square_rectangles(N) if box else meshgen.square_triangles(N)
    vtkio.write_vtu(tmp_path / "mesh.vtu", coords, cells, {})
    assert init.main(["--mesh", str(tmp_path / "mesh.vtu"), "--output", str(tmp_path / "initial.vtu"),
                      "--output-boundary", str(tmp_path / "boundary.bcs")]) == 0
    (tmp_path / "config.ini").write_text(CONFIG)
    return coords, cells


def test_config_schema(tmp_path):
    _write_case(tmp_path)
    cfg = config.parse(tmp_path / "config.ini")
    assert cfg["diffusivity"] == 1e-3 and cfg["convergence-residue"] == 1e-12
    assert cfg["initial-time"] == 0.0 and cfg["mesh-format"] == "auto"
    # the example's solver keys: GMRES with classical Gram-Schmidt, restart 30
    assert cfg["_solver"] == "gmres" and cfg["_gmres_variant"] == "cgs" and cfg["_gmres_restart"] == 30
    (tmp_path / "mgs.ini").write_text(CONFIG.replace("gmres-variant = CGS", "gmres-variant = MGS")
                                      .replace("gmres-restarting-max = 30", "gmres-restarting-max = 50"))
    c2 = config.parse(tmp_path / "mgs.ini")
    assert c2["_gmres_variant"] == "cgsr" and c2["_gmres_restart"] == 32
    assert any("CGSR" in n for n in c2.notices) and any("32" in n for n in c2.notices)
    (tmp_path / "tfqmr.ini").write_text(CONFIG.replace("linear-solver = gmres", "linear-solver = tfqmr"))
    c3 = config.parse(tmp_path / "tfqmr.ini")
    assert c3["_solver"] == "bicgstab" and any("BiCGStab" in n for n in c3.notices)
    # fixed restart length unless gmres-restarting-min and a step are given
    assert cfg["_gmres_restart_min"] == 0 and cfg["_gmres_restart_steps"] == (0, 0)
    # the reference example's adaptive keys (examples/HeatEquation/config.ini:15-22)
    (tmp_path / "adaptive.ini").write_text(CONFIG.replace(
        "gmres-restarting-max = 30",
        "gmres-restarting-max = 30\ngmres-restarting-min = 3\ngmres-restarting-step-max = 4\n"
        "gmres-restarting-step-min = 2"))
    c4 = config.parse(tmp_path / "adaptive.ini")
    assert c4["_gmres_restart"] == 30 and c4["_gmres_restart_min"] == 3 and c4["_gmres_restart_steps"] == (2, 4)
    (tmp_path / "bad.ini").write_text(CONFIG + "no-such-key = 1\n")
    with pytest.raises(config.ConfigError, match="unknown"):
        config.parse(tmp_path / "bad.ini")
    (tmp_path / "missing.ini").write_text(CONFIG.replace("final-time = 0.003\n", ""))
    with pytest.raises(config.ConfigError, match="final-time"):
        config.parse(tmp_path / "missing.ini")
    (tmp_path / "time.ini").write_text(CONFIG.replace("final-time = 0.003", "final-time = -1"))
    with pytest.raises(config.ConfigError, match="Final time"):
        config.parse(tmp_path / "time.ini")


def test_bc_storage_roundtrip(tmp_path):
    b = bcstorage.BoundaryConditionsStorage(7)
    b.tags[:] = [0, 1, 2, 3, 0, 1, 2]
    b.values[:] = np.arange(7) * 0.5
    b.dirichletValues[:] = -np.arange(7)
    b.save(tmp_path / "b.bcs")
    c = bcstorage.BoundaryConditionsStorage.load(tmp_path / "b.bcs")
    assert c.dofSize == 7
    assert np.array_equal(c.tags, b.tags) and np.array_equal(c.values, b.values)
    assert np.array_equal(c.dirichletValues, b.dirichletValues)
    raw = bytearray((tmp_path / "b.bcs").read_bytes())
    raw[len(bcstorage.MAGIC) + 4 + len(bcstorage.SERIALIZATION_TYPE) + 8 + 8] = 9  # corrupt tag
    (tmp_path / "bad.bcs").write_bytes(bytes(raw))
    with pytest.raises(ValueError, match="tag"):
        bcstorage.BoundaryConditionsStorage.load(tmp_path / "bad.bcs")


def test_init_matches_reference_formula(tmp_path):
    coords, cells = _write_case(tmp_path)
    z = vtkio.read_cell_data(tmp_path / "initial.vtu", "InitialCondition[Z0]")
    c = meshgen.cell_centroids(coords, cells)
    x, y = c[:, 0] - 0.5, c[:, 1] - 0.5
    assert np.allclose(z, np.maximum(0, (x * x / -0.05 + y * y / -0.05 + 5) * 0.2))
    b = bcstorage.BoundaryConditionsStorage.load(tmp_path / "boundary.bcs")
    assert b.dofSize == 3 * 36 + 2 * 6 and np.all(b.tags == 0)


def test_init_counts_box_faces(tmp_path):
    _write_case(tmp_path, N=6, box=True)
    b = bcstorage.BoundaryConditionsStorage.load(tmp_path / "boundary.bcs")
    assert b.dofSize == 2 * 6 * 7


@pytest.mark.gpu
@pytest.mark.parametrize("box", [False, True])
def test_driver_end_to_end(tmp_path, box):
    from mhfem import problems, run
    from oracle.oracle import OracleModel

    coords, cells = _write_case(tmp_path, box=box)
    rc = run.main(["--config", str(tmp_path / "config.ini"), "--log-file", str(tmp_path / "log.txt"),
                   "--verbose", "0"])
    assert rc == 0
    out = tmp_path / "out"
    files = sorted(out.glob("data_*.vtu"))
    assert [f.name for f in files] == [f"data_{k:05d}.vtu" for k in range(4)]
    log = (tmp_path / "log.txt").read_text()
    assert ("rectangles" if box else "triangles") in log
    assert "Total number of time steps:" in log and "Total number of linear solver iterations:" in log
    z_gpu = vtkio.read_cell_data(files[-1], "Z")
    # the same model through the oracle: heat equation, D = 1e-3, dt = 5e-4, 6 steps
    z0 = vtkio.read_cell_data(tmp_path / "initial.vtu", "InitialCondition[Z0]")
    p = problems.heat2d_rect(N=6) if box else problems.heat2d(N=6)
    p.coords, p.cells, p.Z0 = coords, cells, z0
    p.coeffs["D"] = 1e-3
    m = OracleModel.from_problem(p)
    t = 0.0
    for _ in range(6):
        m.step(t, 5e-4, 1e-14)
        t += 5e-4
    assert rel_err(z_gpu, m.Z_iK) < 1e-9


def test_example_refuses_host_exec_and_mpi_ranks(tmp_path):
    from mhfem import example

    (tmp_path / "config.ini").write_text(CONFIG)
    assert example.main(["--config", str(tmp_path / "config.ini"), "--exec", "host"]) == 1
    assert example.main(["--config", str(tmp_path / "config.ini"), "--mpi-ranks", "2"]) == 1


@pytest.mark.gpu
def test_example_workflow(tmp_path):
    """The reference's examples/HeatEquation/run.py flow: init (IC + BC file at
    the configured paths) and then the solver, from one config.ini."""
    from mhfem import example

    coords, cells = meshgen.square_triangles(6)
    vtkio.write_vtu(tmp_path / "mesh.vtu", coords, cells, {})
    cfg = CONFIG.replace("boundary-conditions-file = boundary.bcs", "boundary-conditions-file = out/boundary.bcs")
    cfg = cfg.replace("initial-condition = initial.vtu", "initial-condition = out/initial.vtu")
    (tmp_path / "config.ini").write_text(cfg)
    assert example.main(["--config", str(tmp_path / "config.ini")]) == 0
    out = tmp_path / "out"
    assert (out / "initial.vtu").exists() and (out / "boundary.bcs").exists() and (out / "log.txt").exists()
    assert sorted(f.name for f in out.glob("data_*.vtu")) == [f"data_{k:05d}.vtu" for k in range(4)]


def _tnl_object(magic: bytes, typ: str) -> bytes:
    t = typ.encode()
    return magic + struct.pack("<i", len(t)) + t


@pytest.mark.parametrize("real", ["double", "float"])
def test_bc_storage_reads_the_tnl_file_layout(tmp_path, real):
    """The layout BoundaryConditionsStorage::save writes with TNL's File:
    object header, dofSize, then three arrays with their own headers."""
    n = 7
    rng = np.random.default_rng(2)
    tags = rng.integers(0, 4, n).astype(np.uint8)
    vals = rng.standard_normal(n)
    dvals = rng.standard_normal(n)
    fdt = "<f8" if real == "double" else "<f4"
    m = b"TNLMN"
    raw = _tnl_object(m, f"TNL::MHFEM::BoundaryConditionsStorage< {real} >") + struct.pack("<q", n)
    raw += _tnl_object(m, "TNL::Containers::Array< std::uint8_t, [any_device], std::int64_t >")
    raw += struct.pack("<q", n) + tags.tobytes()
    for arr in (vals, dvals):
        raw += _tnl_object(m, f"TNL::Containers::Array< {real}, [any_device], std::int64_t >")
        raw += struct.pack("<q", n) + arr.astype(fdt).tobytes()
    (tmp_path / "b.tnl").write_bytes(raw)
    b = bcstorage.BoundaryConditionsStorage.load(tmp_path / "b.tnl")
    assert b.dofSize == n and np.array_equal(b.tags, tags)
    assert np.array_equal(b.values, vals.astype(fdt).astype(np.float64))
    assert np.array_equal(b.dirichletValues, dvals.astype(fdt).astype(np.float64))
    (tmp_path / "short.tnl").write_bytes(raw[:-3])
    with pytest.raises(ValueError):
        bcstorage.BoundaryConditionsStorage.load(tmp_path / "short.tnl")
