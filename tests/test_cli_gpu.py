"""The schwarz_solve CLI: the reference's flags, stdout lines, JSONL record and
exit code (src/main.cpp:37-61, :245-249, :274; src/io/metrics_logger.h:28-51),
plus the GPU extensions (mixed precision, learned stage, batched solves)."""
from __future__ import annotations

import json
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "schwarz_gmres_dashboard_gb300", "_build", "schwarz_solve")


def _run(*args, timeout=300):
    return subprocess.run([CLI, *args], capture_output=True, text=True, timeout=timeout)


def _field(out, key):
    for line in out.splitlines():
        if line.strip().startswith(key):
            return line.split(":", 1)[1].strip()
    raise KeyError(key)


def test_cli_usage_and_rejected_flags(sg):
    r = _run()
    assert r.returncode == 1 and "Usage" in r.stderr
    r = _run("--poisson", "8", "--drop-tol", "1e-3")
    assert r.returncode == 1 and "outside the GPU solve path" in r.stderr


@pytest.mark.gpu
def test_cli_reference_run_and_jsonl(sg, tmp_path):
    out = tmp_path / "m.jsonl"
    r = _run("--poisson", "64", "--precond", "ilu0", "--tol", "1e-10", "--output", str(out))
    assert r.returncode == 0, r.stderr
    assert _field(r.stdout, "Converged") == "yes"
    assert int(_field(r.stdout, "Iterations")) > 0
    rec = json.loads(out.read_text().splitlines()[-1])
    for k in ("matrix", "method", "n", "nnz", "ranks", "threads", "overlap", "restart",
              "iterations", "tol", "residual_norm", "time_setup_s", "time_solve_s", "speedup",
              "efficiency"):
        assert k in rec
    assert rec["n"] == 64 * 64 and rec["method"] == "GPU_GMRES+ilu0"


@pytest.mark.gpu
def test_cli_mixed_two_level(sg):
    r = _run("--varcoef", "32", "--precond", "twolevel_ras", "--nparts", "8", "--partition",
             "boxes", "--precision", "mixed", "--factor", "bf16", "--stop", "true_rel", "--tol",
             "1e-8")
    assert r.returncode == 0, r.stderr
    assert float(_field(r.stdout, "True relative residual")) <= 1e-8


@pytest.mark.gpu
def test_cli_multi_rhs(sg):
    r = _run("--poisson3d", "24", "--precond", "ras", "--nparts", "8", "--nrhs", "3", "--stop",
             "true_rel", "--tol", "1e-8", "--precision", "mixed")
    assert r.returncode == 0, r.stderr
    assert _field(r.stdout, "Converged") == "yes (3/3)"
    assert float(_field(r.stdout, "Max true relative residual")) <= 1e-8


@pytest.mark.gpu
def test_cli_aniso_batch(sg, tmp_path):
    out = tmp_path / "b.jsonl"
    r = _run("--aniso-batch", "6", "--nrhs", "2", "--output", str(out))
    assert r.returncode == 0, r.stderr
    assert _field(r.stdout, "Converged") == "yes (12/12)"
    rec = json.loads(out.read_text().splitlines()[-1])
    assert rec["solves"] == 12 and rec["true_rel_residual"] <= 1e-8


@pytest.mark.gpu
def test_cli_learned_stage(sg, tmp_path):
    st = sg.LearnedCorrection(32)
    st.init_weights(7)
    w = st.weights
    w[-1] = 1.0
    st.weights = w
    path = tmp_path / "w.bin"
    st.save(str(path))
    st.close()
    r = _run("--varcoef", "32", "--precond", "twolevel_ras", "--nparts", "8", "--learned",
             str(path), "--stop", "true_rel", "--tol", "1e-8")
    assert r.returncode == 0, r.stderr
    assert "Learned stage:" in r.stdout and "FGMRES" in r.stdout
    assert float(_field(r.stdout, "True relative residual")) <= 1e-8
    # a short weights file is refused
    (tmp_path / "short.bin").write_bytes(b"\0" * 16)
    r = _run("--varcoef", "32", "--precond", "twolevel_ras", "--learned",
             str(tmp_path / "short.bin"))
    assert r.returncode == 2 and "float32 weights" in r.stderr


@pytest.mark.gpu
def test_cli_matrix_market_input(sg, tmp_path):
    """--matrix with a symmetric file (lower triangle stored): the reader
    mirrors it, b = A * ones, and the solve converges to x = ones."""
    A = sg.make_poisson_2d(20, 20)
    p = tmp_path / "p.mtx"
    rows = []
    for i in range(A.nrows):
        for e in range(A.row_ptr[i], A.row_ptr[i + 1]):
            if A.col_idx[e] <= i:
                rows.append(f"{i + 1} {A.col_idx[e] + 1} {float(A.vals[e])!r}")
    p.write_text("%%MatrixMarket matrix coordinate real symmetric\n% Poisson 20x20\n"
                 f"{A.nrows} {A.ncols} {len(rows)}\n" + "\n".join(rows) + "\n")
    out = tmp_path / "m.jsonl"
    r = _run("--matrix", str(p), "--precond", "ras", "--nparts", "4", "--output", str(out))
    assert r.returncode == 0, r.stderr
    assert f"n={A.nrows}  nnz={A.nnz()}" in r.stdout
    assert _field(r.stdout, "Converged") == "yes"
    rec = json.loads(out.read_text().splitlines()[-1])
    assert rec["matrix"] == str(p) and rec["nnz"] == A.nnz()


@pytest.mark.gpu
def test_cli_bicgstab_and_analysis(sg, tmp_path):
    """--bicgstab and --analyze: the pre-solve condition / spectral estimates
    are printed, the solve converges, and <output>.conv.jsonl receives the
    reference's convergence record."""
    out = tmp_path / "b.jsonl"
    r = _run("--poisson", "32", "--precond", "ilu0", "--bicgstab", "--analyze", "--tol", "1e-10",
             "--output", str(out))
    assert r.returncode == 0, r.stderr
    assert "Solving with BiCGSTAB + ilu0" in r.stdout
    assert "Condition estimate (A (unpreconditioned)) [Lanczos 80 steps]" in r.stdout
    assert "rho(I - M^{-1}A)" in r.stdout and "Convergence analysis" in r.stdout
    assert _field(r.stdout, "Converged") == "yes"
    rec = json.loads(out.read_text().splitlines()[-1])
    assert rec["method"] == "GPU_BiCGSTAB+ilu0"
    conv = json.loads((tmp_path / "b.jsonl.conv.jsonl").read_text().splitlines()[-1])
    assert conv["type"] == "convergence" and conv["converged"] is True
    assert conv["iterations"] == len(conv["residual_history"]) > 0
