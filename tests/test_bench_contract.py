"""The benchmark's JSON line, on the CPU: the reference arm (the oracle port,
OpenMP on the host's cores) on a small grid prints the keys the contract
asks for; the roofline's DRAM traffic comes from the committed ncu summary
with the commit it was captured on; the per-iteration byte model is the
documented one."""
import json
import os
import subprocess
import sys
from pathlib import Path

REPO = Path(__file__).resolve().parent.parent

KEYS = ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
        "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e")


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--grid", "8", "--steps", "2",
                          "--warmup", "1"], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    d = json.loads(out.stdout.strip().splitlines()[-1])
    for k in KEYS:
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["steps"] == 2 and d["warmup"] == 1
    assert d["higher_is_better"] is True and d["dtype"] == "f64"
    assert d["config"]["workload"] == "diffusion3d_8"
    # the same config keys as the GPU arm's line (bench.workload_config), the threads this process may use
    assert set(d["config"]) == {"workload", "cells", "faces", "rows", "tol", "dt", "l2"}
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["cores"] == len(os.sched_getaffinity(0))
    assert "8^3" in d["cpu_baseline"]["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}


def _bench():
    sys.path.insert(0, str(REPO))
    import bench
    return bench


def test_roofline_traffic_names_its_capture():
    bench = _bench()
    summary = (REPO / "profiles" / "iteration_kernels_fp64_diffusion3d64.txt").read_text()
    for name in ("spmv_dot", "spmv_dots2"):
        value, source = bench.ncu_traffic(name, 64)
        line = [l.split() for l in summary.splitlines() if l.startswith(f"traffic {name} ")][0]
        assert value == float(line[2]) and source.endswith(f"ncu capture of commit {line[3]}")
        assert f"captured on commit {line[3]}" in summary
    assert bench.ncu_traffic("spmv_dots2", 32) == (None, None)  # captured at 64^3 only


def test_iteration_bytes_model():
    """One FP64 BiCGStab iteration moves R (24 W + 160) bytes: the two SpMVs
    (12 W + 24 and 12 W + 16 per row) and the s, x / r and p updates (24, 56
    and 32 per row); 296 bytes per row at width 6."""
    bench = _bench()
    n, nf, S, C, F, V, W = 1, 4, 14, 1572864, 3170304, 274625, 6
    per_iter = bench.step_bytes(n, nf, S, C, F, V, W, 1) - bench.step_bytes(n, nf, S, C, F, V, W, 0)
    assert per_iter == F * ((12 * W + 24) + (12 * W + 16) + 24 + 56 + 32) == F * 296
