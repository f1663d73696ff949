"""Pin the oracle's BiCGSTAB (src/core/bicgstab.h:57-204), Lanczos condition
estimate (src/analysis/condition_estimator.h:94-191) and power-iteration
spectral radius (src/analysis/spectral_analysis.h:30-97) against golden
outputs of the reference's own sources (tests/golden/make_golden.py).  The
oracle keeps the reference's operation order, so on the generating host the
results are identical; FP_RTOL allows a few ulps for another libm."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_matrix

SOLVER_KINDS = ["none", "jacobi", "ilu0", "ras", "twolevel_ras"]
CASES = ["p2d_blocks", "p3d_slabs"]
FP_RTOL = 1e-12


def close(a, b, rtol=FP_RTOL):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    scale = max(np.abs(b).max(initial=0.0), 1e-300)
    return np.abs(a - b).max(initial=0.0) <= rtol * scale


def _pc(oracle, golden, case, kind):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    return A, oracle.precond(kind, A, nparts, 1, part)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", SOLVER_KINDS)
def test_bicgstab(oracle, golden, case, kind):
    A, pc = _pc(oracle, golden, case, kind)
    key = f"{case}/bicgstab/{kind}"
    r = oracle.bicgstab(A, golden[f"{case}/b"], np.zeros(A.nrows), pc, max_iter=500, tol=1e-10,
                        hist_cap=600)
    assert r["iterations"] == int(golden[key + "/iterations"])
    assert r["converged"] == bool(golden[key + "/converged"])
    assert close(r["x"], golden[key + "/x"], 1e-10)
    assert close(r["history"], golden[key + "/history"], 1e-10)
    assert close(r["residual_norm"], golden[key + "/residual_norm"], 1e-9)


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", SOLVER_KINDS)
def test_condition_and_spectral(oracle, golden, case, kind):
    A, pc = _pc(oracle, golden, case, kind)
    c = oracle.condition(A, pc, 80, 42)
    g = golden[f"{case}/condition/{kind}"]
    assert c["lanczos_steps"] == int(g[3]) and c["valid"] == bool(g[4])
    assert close([c["lambda_min"], c["lambda_max"]], g[:2], 1e-9)
    s = oracle.spectral(A, pc, 200, 1e-6, 123)
    g = golden[f"{case}/spectral/{kind}"]
    assert s["power_iters"] == int(g[1]) and s["convergence_ok"] == bool(g[2])
    assert close(s["spectral_radius"], g[0], 1e-9)


def test_bicgstab_known_answers(oracle):
    """The reference's BiCGSTAB known answers restated: identity system and a
    3x3 SPD system (tests/test_gmres.cpp style), converged to tol."""
    from conftest import HostCSR
    I = HostCSR(np.arange(6, dtype=np.int32), np.arange(5, dtype=np.int32), np.ones(5))
    b = np.arange(1.0, 6.0)
    r = oracle.bicgstab(I, b, np.zeros(5), None, max_iter=10, tol=1e-12)
    assert r["converged"] and np.allclose(r["x"], b)
    A = HostCSR([0, 2, 5, 7], [0, 1, 0, 1, 2, 1, 2], [4.0, 1, 1, 3, 1, 1, 2])
    xs = np.array([1.0, 2.0, 3.0])
    bb = np.array([4 + 2, 1 + 6 + 3, 2 + 6], dtype=np.float64)
    r = oracle.bicgstab(A, bb, np.zeros(3), None, max_iter=50, tol=1e-12)
    assert r["converged"] and np.allclose(r["x"], xs, atol=1e-10)
