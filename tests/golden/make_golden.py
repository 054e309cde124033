"""Writes the golden fixtures of this directory: small MHFEM problems with the
oracle's outputs, so that parity tests have fixed expected vectors that do
not depend on regenerating meshes or fields, and a change of the oracle
itself shows up as a failing comparison.

The reference ships no golden vectors or tests of its own, so these come
from the CPU restatement (oracle/mhfem_oracle.c), run here at a relative
residual of 1e-13.  Each file holds:
  inputs   config (dim, n_eq, mass_lumping, advection, cell), coords, cells,
           every coefficient array (size 1 = uniform), boundary tags /
           values / Dirichlet values, Z0, dt, steps;
  outputs  face_verts, face_cells, cell_faces; the first step's b, Q^-1 R,
           CSR system (rowptr, cols, vals) and right-hand side; Z_iF and
           Z_iK after every step.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
REPO = HERE.parent.parent
for p in (str(REPO / "tnl-mhfem_gb300"), str(REPO), str(REPO / "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)

COEFS = ["N", "u", "m", "D", "w", "a", "r", "f", "m_upw", "m_bnd"]
SOLVE_TOL = 1e-13


def build(p) -> dict:
    from oracle.oracle import OracleModel

    c = p.config
    m = OracleModel.from_problem(p, threads=1)
    out = {
        "config": np.array([c.dim, c.n_eq, int(c.mass_lumping), c.advection, c.cell], np.int32),
        "coords": np.asarray(p.coords, np.float64), "cells": np.asarray(p.cells, np.int32),
        "bc_tags": m.tags, "bc_values": m.bvalues, "bc_dirichlet": m.bdirichlet,
        "Z0": np.asarray(p.Z0, np.float64).ravel(), "dt": np.float64(p.dt), "steps": np.int32(p.steps),
        "face_verts": m.face_verts, "face_cells": m.face_cells, "cell_faces": m.cell_faces,
    }
    # the coefficient arrays exactly as the oracle read them (size 1: uniform)
    for k in COEFS:
        out["coef_" + k] = (m.m_upw if k == "m_upw" else m.coeff_arrays[k]).copy()
    zf, zk = [], []
    t = 0.0
    for step in range(p.steps):
        m.pre_iterate(t, p.dt)
        m.assemble(t, p.dt)
        if step == 0:
            out.update(b0=m.b.copy(), R_ijKe0=m.R_ijKe.copy(), R_iK0=m.R_iK.copy(), rowptr=m.rowptr.copy(),
                       cols=m.cols.copy(), vals0=m.vals.copy(), rhs0=m.rhs.copy())
        m.solve(SOLVE_TOL)
        m.post_iterate(t, p.dt)
        zf.append(m.Z_iF.copy())
        zk.append(m.Z_iK.copy())
        t += p.dt
    out["Z_iF"] = np.array(zf)
    out["Z_iK"] = np.array(zk)
    return out


def golden_problems() -> dict:
    """Small cases over the cell types, component counts, mass lumping,
    advection variants and boundary tags.  None uses mobility upwinding,
    whose step parity needs the GPU's velocities where the upwind choice is
    at rounding level."""
    from helpers import box_cases, dummy_row_cases, three_component_cases, variant
    from mhfem import _lib as L
    from mhfem import problems

    cases = {}
    cases["heat2d"] = problems.heat2d(N=4, steps=3)
    cases["heat2d_lumped"] = variant(problems.heat2d(N=4, steps=2), mass_lumping=True)
    cases["diffusion3d"] = problems.diffusion3d(N=2, steps=3)
    cases["diffusion3d_lumped"] = variant(problems.diffusion3d(N=2, steps=2), mass_lumping=True)
    p = problems.adr2d(N=4, steps=3)
    cases["adr2d"] = p
    cases["adr2d_implicit_upwind"] = variant(p, advection=L.IMPLICIT_UPWIND)
    cases["adr2d_implicit_trace"] = variant(p, advection=L.IMPLICIT_TRACE,
                                            coeffs={"a": np.asarray(p.coeffs["a"]) * 0.02})
    cases["heat2d_rect"] = problems.heat2d_rect(N=4, steps=3)
    cases["diffusion3d_box"] = problems.diffusion3d_box(N=2, steps=3)
    p = problems.adr2d(N=4, steps=3, box=True)
    cases["adr2d_rect_implicit_upwind"] = variant(p, advection=L.IMPLICIT_UPWIND, mass_lumping=False)
    cases["adr2d_n3_implicit_upwind"] = three_component_cases()["adr2d_n3_implicit_upwind"]
    cases["diffusion3d_box_n2"] = box_cases()["diffusion3d_box_n2"]
    # an all-zero row of Q on isolated cells: the dummy equation of Solver.hpp:829-847
    cases["diffusion3d_dummy_row"] = dummy_row_cases(N=3)["diffusion3d_dummy_row"]
    return cases


def main() -> None:
    for old in HERE.glob("*.npz"):
        old.unlink()
    for name, p in golden_problems().items():
        assert not p.config.mobility_upwind and p.source is None
        np.savez_compressed(HERE / f"{name}.npz", **build(p))
        print(name, (HERE / f"{name}.npz").stat().st_size, "bytes")


if __name__ == "__main__":
    main()
