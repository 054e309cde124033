"""config.ini parsing with the reference's schema.

Keys follow MHFEM::configSetup (configSetup.h:9-63), the iterative-solver keys
it registers, and the heat-equation model's `diffusivity`
(HeatEquationModel.h:107-112).  Keys this library adds (`solver-form`,
`inner-tolerance`, `learned-train-steps`, `mass-lumping`) are optional.
As in TNL's parser, an unknown key is an error and a missing required key is
an error.  The file has no section header (run.py:17-24).
"""
from __future__ import annotations

import configparser
from dataclasses import dataclass, field
from pathlib import Path

# key -> (type, default, required)
SCHEMA = {
    "output-directory": (str, None, False),
    "mesh": (str, None, True),
    "mesh-format": (str, "auto", False),
    "boundary-conditions-file": (str, None, False),
    "initial-condition": (str, None, False),
    "final-time": (float, None, True),
    "initial-time": (float, 0.0, False),
    "snapshot-period": (float, None, True),
    "time-step": (float, 1.0, False),
    "linear-solver": (str, None, True),
    "preconditioner": (str, "none", False),
    # TNL IterativeSolver / Krylov keys (configSetup.h:55-62)
    "convergence-residue": (float, 1e-6, False),
    "divergence-residue": (float, 1e300, False),
    "max-iterations": (int, 1000000000, False),
    "min-iterations": (int, 0, False),
    "refresh-rate": (int, 1, False),
    "residual-history-file": (str, None, False),
    "gmres-variant": (str, None, False),
    "gmres-restarting-min": (int, None, False),
    "gmres-restarting-max": (int, None, False),
    "gmres-restarting-step-min": (int, None, False),
    "gmres-restarting-step-max": (int, None, False),
    "bicgstab-exact-residue": (str, None, False),
    "bicgstab-ell": (int, None, False),
    "idr-s": (int, None, False),
    "sor-omega": (float, None, False),
    "ilut-max-fill": (int, None, False),
    "ilut-threshold": (float, None, False),
    # heat-equation model
    "diffusivity": (float, 1.0, False),
    # this library
    "solver-form": (str, "fp64", False),
    "inner-tolerance": (float, 1e-4, False),
    "learned-train-steps": (int, 200, False),
    "mass-lumping": (str, "disabled", False),
}

LINEAR_SOLVERS = {"bicgstab", "bicgstabl", "gmres", "cg", "tfqmr", "idrs", "sor", "jacobi"}
GMRES_VARIANTS = {"CGS", "CGSR", "MGS", "MGSR", "CWY"}
PRECONDITIONERS = {"none", "diagonal", "ilu0", "ilut"}
MESH_FORMATS = {"auto", "vtk", "vtu", "ng"}


class ConfigError(ValueError):
    pass


@dataclass
class Config:
    values: dict
    path: Path
    notices: list = field(default_factory=list)

    def __getitem__(self, key):
        return self.values[key]

    def get(self, key, default=None):
        v = self.values.get(key)
        return default if v is None else v


def parse(path, overrides: dict | None = None) -> Config:
    path = Path(path)
    parser = configparser.ConfigParser(interpolation=None)
    parser.optionxform = str
    parser.read_string("[top]\n" + path.read_text())
    raw = dict(parser["top"])
    raw.update({k: str(v) for k, v in (overrides or {}).items() if v is not None})
    values, notices = {}, []
    for key in raw:
        if key not in SCHEMA:
            raise ConfigError(f"{path}: unknown configuration key {key!r}")
    for key, (typ, default, required) in SCHEMA.items():
        if key in raw:
            try:
                values[key] = typ(raw[key])
            except ValueError as exc:
                raise ConfigError(f"{path}: key {key!r}: {exc}") from None
        elif required:
            raise ConfigError(f"{path}: missing required key {key!r}")
        else:
            values[key] = default
    if values["mesh-format"] not in MESH_FORMATS:
        raise ConfigError(f"mesh-format must be one of {sorted(MESH_FORMATS)}")
    solver = values["linear-solver"].lower()
    if solver not in LINEAR_SOLVERS:
        raise ConfigError(f"linear-solver {solver!r} is not a TNL solver name")
    # the solver this library runs: BiCGStab or restarted GMRES (the others map to BiCGStab)
    values["_solver"], values["_gmres_restart"], values["_gmres_variant"] = "bicgstab", 30, "cgs"
    values["_gmres_restart_min"], values["_gmres_restart_steps"] = 0, (0, 0)
    if solver == "gmres":
        values["_solver"] = "gmres"
        variant = (values["gmres-variant"] or "CGS").upper()
        if variant not in GMRES_VARIANTS:
            raise ConfigError(f"gmres-variant {variant!r} is not one of {sorted(GMRES_VARIANTS)}")
        if variant in ("MGS", "MGSR", "CWY"):
            notices.append(f"gmres-variant = {variant}: runs as CGSR (classical Gram-Schmidt with one "
                           "reorthogonalization pass, which keeps the basis as orthogonal as MGS does)")
            variant = "CGSR"
        values["_gmres_variant"] = variant.lower()
        restart = values["gmres-restarting-max"] or 30
        if restart > 32:
            notices.append(f"gmres-restarting-max = {restart}: restarts after 32 iterations (the longest cycle)")
            restart = 32
        values["_gmres_restart"] = int(restart)
        rmin = values["gmres-restarting-min"]
        if rmin is not None and 0 < rmin < restart:
            smin = values["gmres-restarting-step-min"]
            smax = values["gmres-restarting-step-max"]
            smin = 3 if smin is None else smin  # the published rule's decrement when no step is given
            smax = smin if smax is None else max(smax, smin)
            if smin > 0:
                values["_gmres_restart_min"], values["_gmres_restart_steps"] = int(rmin), (int(smin), int(smax))
    elif solver != "bicgstab":
        notices.append(f"linear-solver = {solver}: this library's Krylov solvers are BiCGStab and GMRES; it "
                       "runs BiCGStab with the same convergence-residue and max-iterations")
    prec = values["preconditioner"].lower()
    if prec not in PRECONDITIONERS:
        raise ConfigError(f"preconditioner {prec!r} is not a TNL preconditioner name")
    if prec in ("ilu0", "ilut"):
        notices.append(f"preconditioner = {prec}: not provided; every row has a unit diagonal, so the "
                       "diagonal (Jacobi) preconditioner used here is the identity")
    if values["solver-form"] not in ("fp64", "mixed", "learned"):
        raise ConfigError("solver-form must be fp64, mixed or learned")
    if values["mass-lumping"] not in ("enabled", "disabled"):
        raise ConfigError("mass-lumping must be enabled or disabled")
    if values["final-time"] <= values["initial-time"]:
        raise ConfigError("Final time must larger than the initial time.")  # control.h:116-117
    if values["snapshot-period"] <= 0:
        raise ConfigError("Snapshot period must be positive value.")
    if values["time-step"] <= 0:
        raise ConfigError("Time step must be positive value.")
    return Config(values, path, notices)
