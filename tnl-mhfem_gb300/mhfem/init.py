"""Initial and boundary conditions of the heat-equation example (the role of
examples/HeatEquation/init.py:11-42): the initial condition
max(0, (x^2/alpha + y^2/beta + gamma) * 0.2) at cell centres (relative to the
domain centre), written as cell data ``InitialCondition[Z0]`` in a VTU file,
and all-FixedValue zero boundary conditions.

    python -m mhfem.init --mesh mesh.vtk --output initial.vtu --output-boundary boundary.bcs
"""
from __future__ import annotations

import argparse

import numpy as np

from . import meshgen, vtkio
from .bcstorage import BoundaryConditionsStorage, BoundaryConditionsType
from .run import load_mesh


def initial_condition(coords, cells, alpha=-0.05, beta=-0.05, gamma=5.0):
    c = meshgen.cell_centroids(coords, cells)
    x = c[:, 0] - 0.5
    y = c[:, 1] - 0.5
    return np.maximum(0.0, (x * x / alpha + y * y / beta + gamma) * 0.2)


def boundary_condition(num_faces: int) -> BoundaryConditionsStorage:
    bcs = BoundaryConditionsStorage(num_faces)
    bcs.tags[:] = BoundaryConditionsType.FixedValue
    return bcs


def count_faces(cells: np.ndarray, box: bool = False) -> int:
    return meshgen.count_faces(cells, box)


def main(argv=None) -> int:
    from pathlib import Path

    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--mesh", required=True)
    ap.add_argument("--alpha", type=float, default=-0.05)
    ap.add_argument("--beta", type=float, default=-0.05)
    ap.add_argument("--gamma", type=float, default=5.0)
    ap.add_argument("--output", required=True)
    ap.add_argument("--output-boundary", required=True)
    a = ap.parse_args(argv)
    coords, cells = load_mesh(a.mesh, "auto", Path("."))
    ic = initial_condition(coords, cells, a.alpha, a.beta, a.gamma)
    vtkio.write_vtu(a.output, coords, cells, {"InitialCondition[Z0]": ic}, cycle=0)
    boundary_condition(count_faces(cells, meshgen.is_box_mesh(coords, cells))).save(a.output_boundary)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
