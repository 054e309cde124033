"""The config.ini driver: ``python -m mhfem.run --config config.ini``.

It mirrors the reference's command line and control flow:
- the CLI keys come from examples/main.h:32-50: --config, --output-directory,
  --log-file, --verbose, --print-static-configuration, --catch-exceptions;
- the flow is that of MHFEM::execute / init / solve (control.h:15-312):
  1. load the mesh, the boundary-conditions file and the initial condition;
  2. write the prolog to the log;
  3. run the snapshot loop, writing ``data_%05d.vtu`` with cell field ``Z``
     at the initial time and after every snapshot period;
  4. write the epilog: total linear-solver iterations and time steps, plus
     the phase timers.

The model is the heat equation of examples/HeatEquation (N = 1, D =
`diffusivity`, all other coefficients 0, constant mobility).  The mesh key
also accepts ``synthetic:square:N`` and ``synthetic:cube:N`` for the jittered
simplex meshes of mhfem.meshgen, and ``synthetic:rect:N`` / ``synthetic:cuboid:N``
for its graded box meshes; meshes of quadrilaterals / hexahedra (2^dim
vertices per cell) run with box cells.  `--exec cuda` is the only execution mode.  The
library has no CPU implementation, so `--exec host` is refused.
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

import numpy as np

from . import _lib as L
from . import bcstorage, config, meshgen, vtkio
from .solver import Solver, StaticConfig

FORMS = {"fp64": L.FORM_FP64, "mixed": L.FORM_MIXED, "learned": L.FORM_LEARNED}


def load_mesh(spec: str, fmt: str, base: Path):
    if spec.startswith("synthetic:"):
        _, kind, n = spec.split(":")
        if kind == "square":
            return meshgen.square_triangles(int(n))
        if kind == "cube":
            return meshgen.cube_tetrahedra(int(n))
        if kind == "rect":
            return meshgen.square_rectangles(int(n))
        if kind == "cuboid":
            return meshgen.cube_cuboids(int(n))
        raise ValueError(f"unknown synthetic mesh {kind!r} (square, cube, rect, cuboid)")
    return vtkio.read_mesh(base / spec, fmt)


class Logger:
    def __init__(self, path: Path | None, verbose: int):
        self.fh = open(path, "w") if path else None
        self.verbose = verbose

    def param(self, key, value):
        line = f"{key:<44s} {value}"
        if self.fh:
            self.fh.write(line + "\n")
        if self.verbose:
            print(line)

    def sep(self):
        self.param("-" * 40, "")

    def close(self):
        if self.fh:
            self.fh.close()


def run(cfg: config.Config, log: Logger, device: int = 0) -> dict:
    base = cfg.path.parent
    out_dir = Path(cfg["output-directory"] or "output")
    if not out_dir.is_absolute():
        out_dir = base / out_dir
    out_dir.mkdir(parents=True, exist_ok=True)
    coords, cells = load_mesh(cfg["mesh"], cfg["mesh-format"], base)
    dim = coords.shape[1]
    box = meshgen.is_box_mesh(coords, cells)
    static = StaticConfig(dim=dim, n_eq=1, mass_lumping=cfg["mass-lumping"] == "enabled",
                          advection=L.EXPLICIT_UPWIND, mobility_upwind=False, form=FORMS[cfg["solver-form"]],
                          device=device, cell=L.CELL_BOX if box else L.CELL_SIMPLEX)
    s = Solver(static)
    s.setMesh(coords, cells)
    # heat-equation model coefficients (HeatEquationModel.h:114-133)
    for k, v in {"N": 1.0, "u": 0.0, "m": 1.0, "D": cfg["diffusivity"], "w": 0.0, "a": 0.0, "r": 0.0,
                 "f": 0.0, "m_upw": 1.0, "m_bnd": 1.0}.items():
        s.set_coeff(k, v)
    if cfg.get("boundary-conditions-file"):
        bcs = bcstorage.BoundaryConditionsStorage.load(base / cfg["boundary-conditions-file"])
        if bcs.dofSize != s.F:  # Solver.hpp:274-278
            raise ValueError(f"Wrong dofSize in BoundaryConditionsStorage: expected {s.F}, got {bcs.dofSize}")
        s.set_bc(bcs.tags, bcs.values, bcs.dirichletValues)
    if cfg.get("initial-condition"):
        z0 = vtkio.read_cell_data(base / cfg["initial-condition"], "InitialCondition[Z0]")
        if z0.size != s.C:
            raise ValueError(f"wrong vector length for the initial condition: expected {s.C}, got {z0.size}")
    else:
        z0 = np.zeros(s.C)
    s.setup(tol=cfg["convergence-residue"], max_iter=min(cfg["max-iterations"], 2 ** 31 - 1),
            inner_tol=cfg["inner-tolerance"], linear_solver=cfg["_solver"], gmres_restart=cfg["_gmres_restart"],
            gmres_variant=cfg["_gmres_variant"], gmres_restart_min=cfg["_gmres_restart_min"],
            gmres_restart_step_min=cfg["_gmres_restart_steps"][0],
            gmres_restart_step_max=cfg["_gmres_restart_steps"][1])
    if cfg["solver-form"] == "learned":
        s.learned_options(train_steps=cfg["learned-train-steps"])
    s.setInitialCondition(z0)
    s.setupLinearSystem()

    # prolog (control.h:151-203)
    log.param("MHFEM solver", "GB300 native (libmhfem_gb300)")
    log.param("Device type:", "CUDA (sm_103a)")
    log.param("Real type:", "double")
    log.param("Index type:", "int")
    log.param("Mesh type:", ("rectangles" if dim == 2 else "cuboids") if box else
              ("triangles" if dim == 2 else "tetrahedra"))
    log.param("Sparse matrix:", "ELL (off-diagonal part, unit diagonal)")
    restart = (f"{cfg['_gmres_restart_min']}..{cfg['_gmres_restart']}" if cfg["_gmres_restart_min"]
               else f"{cfg['_gmres_restart']}")
    log.param("Linear solver:", f"GMRES({restart}, {cfg['_gmres_variant'].upper()})"
              if cfg["_solver"] == "gmres" else "BiCGStab")
    log.param("Mass lumping:", cfg["mass-lumping"])
    log.param("Advection discretization:", "explicit upwind")
    log.param("Solver form:", cfg["solver-form"])
    log.param("Cells / faces:", f"{s.C} / {s.F}")
    for n in cfg.notices:
        log.param("Notice:", n)
    log.sep()

    compute = io = 0.0
    t0 = cfg["initial-time"]
    final, period, dt = cfg["final-time"], cfg["snapshot-period"], cfg["time-step"]

    def snapshot(t, step):
        zf, zk = s.state()
        vtkio.write_vtu(out_dir / f"data_{step:05d}.vtu", coords, cells, {"Z": zk}, time=t, cycle=step)

    a = time.perf_counter()
    snapshot(t0, 0)
    io += time.perf_counter() - a
    steps = int(np.ceil((final - t0) / period))
    t = t0
    stats = []
    for step in range(1, steps + 1):
        tau = min(period, final - t)
        a = time.perf_counter()
        stats += s.solve(t, t + tau, dt)  # control.h:64-102
        compute += time.perf_counter() - a
        t += tau
        a = time.perf_counter()
        snapshot(t, step)
        io += time.perf_counter() - a
    iters, tsteps, _ = s.totals()
    log.sep()
    log.param("Total number of linear solver iterations:", iters)
    log.param("Total number of time steps:", tsteps)
    for key, name in [("ms_pre", "Pre-iterate time:"), ("ms_assemble", "Linear system assembler time:"),
                      ("ms_solve", "Linear system solver time:"), ("ms_post", "Post-iterate time:")]:
        log.param(name, f"{sum(x[key] for x in stats) / 1e3:.6e} s")
    log.param("Compute time:", f"{compute:.6e} s")
    log.param("I/O time:", f"{io:.6e} s")
    s.close()
    return {"iterations": iters, "time_steps": tsteps, "snapshots": steps + 1, "output": str(out_dir)}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="MHFEM heat-equation solver (GB300)")
    ap.add_argument("--config", required=True)
    ap.add_argument("--output-directory")
    ap.add_argument("--log-file", default="log.txt")
    ap.add_argument("--verbose", type=int, default=2)
    ap.add_argument("--catch-exceptions", default="true")
    ap.add_argument("--print-static-configuration", action="store_true")
    ap.add_argument("--exec", default="cuda", choices=["host", "cuda"])
    ap.add_argument("--device", type=int, default=0)
    args = ap.parse_args(argv)
    if args.exec != "cuda":
        print("this library runs on the GPU only (--exec cuda); it has no host implementation", file=sys.stderr)
        return 1
    if args.print_static_configuration:
        print("Real: double, Index: int, cells: triangles, tetrahedra, rectangles or cuboids (from the "
              "mesh), matrix: ELL, advection: explicit upwind, model: heat equation")
        return 0
    try:
        cfg = config.parse(args.config, {"output-directory": args.output_directory})
    except (config.ConfigError, OSError) as exc:
        print(f"Failed to parse the configuration file {args.config} due to the following error:\n{exc}",
              file=sys.stderr)
        return 1
    log = Logger(Path(args.log_file), args.verbose)
    catch = args.catch_exceptions.lower() in ("1", "true", "yes")
    try:
        res = run(cfg, log, args.device)
    except Exception as exc:  # control.h:289-311
        if not catch:
            raise
        print(f"MHFEM solver failed due to a C++ exception with description: {exc}", file=sys.stderr)
        return 1
    finally:
        log.close()
    print(res)
    return 0


if __name__ == "__main__":
    sys.exit(main())
