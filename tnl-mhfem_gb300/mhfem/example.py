"""The heat-equation example workflow: ``python -m mhfem.example --config config.ini``.

The counterpart of the reference's examples/HeatEquation/run.py:
1. read config.ini (an INI file without section headers, run.py:17-24);
2. create the output directory;
3. write the initial condition and the boundary-condition file for the
   configured mesh (the example's init.py, run.py:47-67), at the paths the
   config names;
4. run the solver on that configuration (run.py:70-99), here the GB300
   library through ``mhfem.run``.

Paths in the config are relative to the config file's directory.
``--exec cuda`` is the only execution mode (the library has no host
implementation) and ``--mpi-ranks`` must be 1: the reference decomposes the
mesh with METIS for MPI ranks (run.py:27-44, 133-155), while this library
solves the whole mesh on one GPU.
"""
from __future__ import annotations

import argparse
import sys
from pathlib import Path

from . import config, init, run


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="Heat equation example (GB300)")
    ap.add_argument("--config", default="config.ini", help="path to the config file")
    ap.add_argument("--exec", default="cuda", choices=["host", "cuda"], help="execution of the MHFEM solver")
    ap.add_argument("--mpi-ranks", default=1, type=int, help="number of MPI ranks (1: one GPU)")
    ap.add_argument("--log-file", default=None, help="log file (default: log.txt in the output directory)")
    args = ap.parse_args(argv)
    if args.exec != "cuda":
        print("this library runs on the GPU only (--exec cuda); it has no host implementation", file=sys.stderr)
        return 1
    if args.mpi_ranks != 1:
        print("distributed runs are not provided: the whole mesh is solved on one GPU (--mpi-ranks 1)",
              file=sys.stderr)
        return 1
    config_path = Path(args.config).resolve()
    try:
        cfg = config.parse(config_path)
    except (config.ConfigError, OSError) as exc:
        print(f"Failed to parse the configuration file {config_path}: {exc}", file=sys.stderr)
        return 1
    base = config_path.parent
    out_dir = base / (cfg["output-directory"] or "output")
    out_dir.mkdir(parents=True, exist_ok=True)
    if not cfg.get("initial-condition") or not cfg.get("boundary-conditions-file"):
        print("config.ini must name initial-condition and boundary-conditions-file", file=sys.stderr)
        return 1
    mesh = cfg["mesh"] if cfg["mesh"].startswith("synthetic:") else str(base / cfg["mesh"])
    rc = init.main(["--mesh", mesh, "--output", str(base / cfg["initial-condition"]),
                    "--output-boundary", str(base / cfg["boundary-conditions-file"])])
    if rc != 0:
        return rc
    log = args.log_file or str(out_dir / "log.txt")
    return run.main(["--config", str(config_path), "--log-file", log])


if __name__ == "__main__":
    raise SystemExit(main())
