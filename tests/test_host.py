"""Host-side checks that need no GPU: the C-ABI library loads, exports every
symbol include/mhfem.h declares, refuses to run without a device, and the
model builders reproduce the workload sizes."""
import ctypes as ct
import math
import re
from pathlib import Path

import numpy as np
import pytest

from mhfem import _lib as L
from mhfem import meshgen, problems
from oracle.oracle import build_faces

REPO = Path(__file__).resolve().parent.parent


def _declared_symbols():
    text = (REPO / "include" / "mhfem.h").read_text()
    return sorted(set(re.findall(r"^\s*(?:mhfem_status|const char\*|void)\s+(mhfem_\w+)\s*\(", text, re.M)))


def test_library_exports_every_declared_symbol():
    lib = ct.CDLL(str(L.LIB_PATH))
    declared = _declared_symbols()
    assert len(declared) >= 20
    for name in declared:
        assert hasattr(lib, name), f"{name} declared in include/mhfem.h but not exported"
    bound = {s[0] for s in L.SIGNATURES}
    assert set(declared) == bound, "ctypes signatures out of sync with the header"


def test_integration_table_names_every_entry_point():
    """INTEGRATION.md's entry-point table (the reference interface each call
    replaces) lists every function the header declares."""
    text = (REPO / "INTEGRATION.md").read_text()
    missing = [name for name in _declared_symbols() if f"`{name}" not in text]
    assert not missing, f"entry points missing from INTEGRATION.md: {missing}"


def test_create_without_device_fails_loudly():
    import torch

    if torch.cuda.is_available():
        pytest.skip("a GPU is visible")
    lib = L.load()
    desc = L.Desc(3, 1, 0, 0, 0, 0, 0)
    h = ct.c_void_p()
    assert lib.mhfem_create(ct.byref(desc), ct.byref(h)) == L.ERR_NO_DEVICE


def test_create_validates_the_cell_type():
    """An unknown cell type is an invalid argument; box cells with the learned
    form (whose face features are defined for simplices) are unsupported.
    Both are refused before any device is touched."""
    lib = L.load()
    h = ct.c_void_p()
    bad = L.Desc(3, 1, 0, 0, 0, L.FORM_FP64, 0, 7)
    assert lib.mhfem_create(ct.byref(bad), ct.byref(h)) == L.ERR_INVALID_ARGUMENT
    learned_box = L.Desc(3, 1, 0, 0, 0, L.FORM_LEARNED, 0, L.CELL_BOX)
    assert lib.mhfem_create(ct.byref(learned_box), ct.byref(h)) == L.ERR_UNSUPPORTED


def test_box_mesh_counts():
    for dim, N in ((2, 5), (3, 4)):
        coords, cells = meshgen.square_rectangles(N) if dim == 2 else meshgen.cube_cuboids(N)
        assert cells.shape == (N ** dim, 2 ** dim)
        fv, fc, cf = build_faces(dim, cells, L.CELL_BOX)
        assert fc.shape[0] == dim * N ** (dim - 1) * (N + 1)
        assert fv.shape[1] == 2 ** (dim - 1)
        h = coords[cells[:, 2 if dim == 2 else 6]] - coords[cells[:, 0]]
        assert np.all(h > 0)  # v0 is the lowest corner, the opposite corner the highest
        assert abs(np.prod(h, axis=1).sum() - 1.0) < 1e-12


@pytest.mark.parametrize("N", [1, 3, 8])
def test_triangle_mesh_counts(N):
    coords, cells = meshgen.square_triangles(N)
    fv, fc, cf = build_faces(2, cells)
    assert cells.shape[0] == 2 * N * N
    assert fv.shape[0] == 3 * N * N + 2 * N
    assert int((fc[:, 1] < 0).sum()) == 4 * N


@pytest.mark.parametrize("N", [1, 2, 5])
def test_tetrahedron_mesh_counts(N):
    coords, cells = meshgen.cube_tetrahedra(N)
    fv, fc, cf = build_faces(3, cells)
    assert cells.shape[0] == 6 * N ** 3
    assert fv.shape[0] == 12 * N ** 3 + 6 * N ** 2
    assert int((fc[:, 1] < 0).sum()) == 12 * N * N


def test_mesh_cells_positive_measure():
    for coords, cells in [meshgen.square_triangles(16), meshgen.cube_tetrahedra(6)]:
        X = coords[cells]
        E = X[:, 1:] - X[:, :1]
        vol = np.abs(np.linalg.det(E))
        assert vol.min() > 0.1 * vol.mean()


def test_diffusion3d_workload_sizes():
    """64^3 tetrahedra: C, F, boundary split as the workload states."""
    p = problems.diffusion3d(N=64, steps=1)
    assert p.C == 1572864
    fv, fc, _ = build_faces(3, p.cells)
    assert fv.shape[0] == 3170304
    tags, _, _ = p.bc_fn(fv, fc)
    bnd = fc[:, 1] < 0
    assert int(bnd.sum()) == 49152
    assert int((tags[bnd] == problems.BC_FIXED_VALUE).sum()) == 16384
    assert int((tags[bnd] == problems.BC_FIXED_FLUX).sum()) == 32768


def test_solver_checks_array_sizes_before_the_library_call():
    """The Python mirror refuses arrays of the wrong size itself: the C ABI
    takes plain pointers and would read past a short buffer."""
    from mhfem.solver import Solver, StaticConfig

    class NoLibrary:
        def __getattr__(self, name):
            raise AssertionError(f"the library was called: {name}")

    s = object.__new__(Solver)  # no handle: every check must fire before a library call
    s.config = StaticConfig(dim=3, n_eq=2)
    s.lib = NoLibrary()
    s.V, s.C, s.F = 8, 10, 25
    with pytest.raises(ValueError, match="Z_iK"):
        s.setInitialCondition(np.zeros(10))
    with pytest.raises(ValueError, match="Z_iF"):
        s.setInitialCondition(np.zeros(20), np.zeros(25))
    with pytest.raises(ValueError, match="boundary"):
        s.set_bc(np.zeros(25, np.uint8), np.zeros(50), np.zeros(50))
    with pytest.raises(ValueError, match="coords"):
        s.setMesh(np.zeros((8, 2)), np.zeros((10, 4), np.int32))
    with pytest.raises(ValueError, match="cells"):
        s.setMesh(np.zeros((8, 3)), np.zeros((10, 3), np.int32))
    with pytest.raises(ValueError, match="features"):
        s.learned_forward(np.zeros((25, 3), np.float32))
    with pytest.raises(ValueError, match="target"):
        s.learned_gradients(np.zeros((25, L.LEARNED_FEATURES), np.float32), np.zeros(24))


@pytest.mark.parametrize("lang,std", [("c", "-std=c99"), ("c++", "-std=c++17")])
def test_header_compiles_as_strict_c_and_cpp(tmp_path, lang, std):
    """include/mhfem.h is a plain C header (what an FFI binds), warning-free
    as strict C99 and as C++17, and links against the library's symbols."""
    import shutil
    import subprocess

    cc = shutil.which("gcc" if lang == "c" else "g++")
    if cc is None:
        pytest.skip("no host compiler")
    src = tmp_path / "use_header.c"
    src.write_text('#include "mhfem.h"\n'
                   "int main(void) { mhfem_solver_opts o; mhfem_default_solver_opts(&o);\n"
                   "  return o.max_iter > 0 && o.tol > 0 ? 0 : 1; }\n")
    flags = ["-Wall", "-Wextra", "-Werror"] + (["-pedantic"] if lang == "c" else [])
    out = tmp_path / "use_header"
    r = subprocess.run([cc, std, *flags, "-I", str(REPO / "include"), "-x", lang, str(src), "-x", "none",
                        str(L.LIB_PATH), f"-Wl,-rpath,{L.LIB_PATH.parent}", "-o", str(out)],
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stderr
    assert subprocess.run([str(out)], timeout=60).returncode == 0


def test_integer_pipe_conversions_match_ieee_casts(tmp_path):
    """csrc/fp_convert.h (the FP64 -> FP32 round-to-nearest-even and exact
    FP32 -> FP64 conversions the mixed form runs on the integer pipes) gives
    bit for bit what the compiler's IEEE casts give, over millions of inputs
    including every tie at every binary32 exponent and the range edges."""
    import shutil
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    out = tmp_path / "fp_convert_check"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(REPO / "tnl-mhfem_gb300" / "csrc"),
                        str(REPO / "tests" / "fp_convert_check.cpp"), "-o", str(out)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(out)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout[-2000:]


def _next_restart(m_min, m_max, step_min, step_max, m, cr):
    """Baker, Jessup and Kolev's restart-length rule with the step as the
    library applies it (restated independently of gmres_restart.h)."""
    if not (0 < m_min < m_max and step_min > 0):
        return m_max
    max_cr, min_cr = math.cos(math.radians(8.0)), math.cos(math.radians(80.0))
    if not cr <= max_cr:
        return m_max
    if cr < min_cr:
        return m
    d = max(step_max, step_min) if cr < 0.5 * (min_cr + max_cr) else step_min
    return m - d if m - d >= m_min else m_max


def test_gmres_restart_rule(tmp_path):
    """The host rule of the adaptive GMRES restart length (gmres_restart.h,
    compiled here as plain C++) against its restatement, over restart
    ratios across all three bands, the band edges, a non-finite ratio, the
    wrap below the minimum and the fixed-length settings."""
    import shutil
    import subprocess

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("g++ not available")
    out = tmp_path / "gmres_restart_check"
    r = subprocess.run([cxx, "-std=c++17", "-O2", "-I", str(REPO / "tnl-mhfem_gb300" / "csrc"),
                        str(REPO / "tests" / "gmres_restart_check.cpp"), "-o", str(out)], capture_output=True,
                       text=True)
    assert r.returncode == 0, r.stderr
    rng = np.random.default_rng(5)
    edges = [math.cos(math.radians(8.0)), math.cos(math.radians(80.0)),
             0.5 * (math.cos(math.radians(8.0)) + math.cos(math.radians(80.0)))]
    cases = []
    for rule in [(3, 30, 2, 4), (3, 30, 3, 3), (1, 8, 1, 2), (0, 30, 2, 4), (30, 30, 2, 4), (3, 30, 0, 0)]:
        for m in (30, 29, 12, 5, 4, 3, 1):
            for cr in list(rng.uniform(0.0, 1.2, 12)) + edges + [0.0, 1.0, float("nan"), float("inf")]:
                cases.append((*rule, m, cr))
    text = "\n".join(f"{a} {b} {c} {d} {m} {float(cr)!r}" for a, b, c, d, m, cr in cases) + "\n"
    r = subprocess.run([str(out)], input=text, capture_output=True, text=True, timeout=60)
    assert r.returncode == 0
    got = [int(v) for v in r.stdout.split()]
    want = [_next_restart(*c) for c in cases]
    assert got == want
