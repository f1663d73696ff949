"""The reference arm of bench.py on the CPU: one JSON line with the keys the
bench contract asks for, on a 16^3 version of the cfg3 workload (the oracle
port runs the reference's algorithm; no GPU is involved)."""
from __future__ import annotations

import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_prints_one_contract_line(sg, oracle):
    out = subprocess.run(
        [sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--grid", "16",
         "--steps", "1", "--warmup", "3"],
        cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
                "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
                "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference"
    assert d["unit"] == "s" and d["higher_is_better"] is False
    assert d["warmup"] >= 3 and d["steps"] == 1
    assert d["value"] > 0 and d["config"]["n"] == 16 ** 3
    assert "16^3" in d["config"]["workload"]
    # the same workload description as the GPU arm's (bench.cfg3_config)
    for key in ("nnz", "nparts", "overlap", "restart", "rtol", "partition", "rhs",
                "parallelism"):
        assert key in d["config"], key
    assert d["config"]["restart"] == 30 and d["config"]["rtol"] == 1e-8
    # the oracle reaches the target residual within the cycles it ran
    assert d["cycles_to_rtol"] is not None and d["cycles_to_rtol"] >= 1
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_loads_nothing_of_the_package(oracle):
    """The reference arm builds its inputs with the oracle alone: the package
    (and its CUDA library) is never imported."""
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--grid', '12', "
            "'--steps', '1', '--warmup', '3']; runpy.run_path('bench.py', run_name='__main__'); "
            "print('PACKAGE_LOADED', any(m.startswith('schwarz_gmres_dashboard_gb300') "
            "for m in sys.modules))")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True,
                         timeout=600, check=True)
    assert "PACKAGE_LOADED False" in out.stdout, out.stdout


def test_reference_arm_under_torchrun_prints_once(sg, oracle):
    """Launched as the multi-GPU bench is (torchrun, two ranks), rank 0 alone
    runs the reference arm and prints; the other rank exits 0 without work."""
    with socket.socket() as so:  # a port free right now (no fixed port to collide on)
        so.bind(("127.0.0.1", 0))
        port = so.getsockname()[1]
    out = subprocess.run(
        [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
         "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
         "--impl", "reference", "--grid", "16", "--steps", "1", "--warmup", "3", "--gpus", "2"],
        cwd=ROOT, capture_output=True, text=True, timeout=600, check=True)
    lines = [ln for ln in out.stdout.splitlines() if ln.strip().startswith("{")]
    assert len(lines) == 1, out.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2
