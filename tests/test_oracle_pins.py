"""Pin the oracle (oracle/oracle.c) before trusting it.

1. Against golden vectors produced by the reference's own sources
   (tests/golden/make_golden.py drives oracle/_ref): SpMV, ILU(0) factors,
   decompositions, coarse operator, every preconditioner apply, and full
   GMRES/FGMRES solves.  Integer data must match exactly; floating-point data
   too, because the oracle keeps the reference's operation order and is built
   without multiply-add contraction (a tolerance of a few ulps is allowed for
   hosts whose libm differs).
2. Against the reference's own known-answer tests (tests/test_gmres.cpp,
   tests/test_schwarz.cpp, tests/test_two_level.cpp), restated.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import HostCSR, golden_matrix

KINDS = ["jacobi", "ilu0", "asm", "ras", "twolevel_asm", "twolevel_ras"]
CASES = ["p2d_blocks", "p2d_scatter", "p3d_slabs"]
SOLVE_CASES = ["p2d_blocks", "p3d_slabs"]

FP_RTOL = 1e-13  # ulp-level; the expected difference on the generating host is 0


def close(a, b, rtol=FP_RTOL):
    a, b = np.asarray(a), np.asarray(b)
    scale = max(np.abs(b).max(initial=0.0), 1e-300)
    return np.abs(a - b).max(initial=0.0) <= rtol * scale


@pytest.mark.parametrize("case", CASES)
def test_spmv_and_ilu0(oracle, golden, case):
    A = golden_matrix(golden, case)
    x = golden[f"{case}/x"]
    assert close(oracle.spmv(A, x), golden[f"{case}/spmv"])
    lu, dg = oracle.ilu0_factor(A)
    assert np.array_equal(dg, golden[f"{case}/ilu0_diag"])
    assert close(lu, golden[f"{case}/ilu0_lu"])


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("overlap", [0, 1, 2])
def test_decomposition_bit_exact(oracle, golden, case, overlap):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    d = oracle.decompose(A, part, nparts, overlap)
    for k in ("owned_ptr", "owned", "sub_ptr", "sub", "ownloc_ptr", "ownloc"):
        assert np.array_equal(d[k], golden[f"{case}/dd{overlap}/{k}"]), k


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_precond_apply(oracle, golden, case, kind):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pc = oracle.precond(kind, A, nparts, 1, part)
    assert close(pc.apply(golden[f"{case}/x"]), golden[f"{case}/apply/{kind}"])
    if kind.startswith("twolevel"):
        # sparse restatement of the dense R0 coarse space: same bits
        assert close(pc.coarse_a0(), golden[f"{case}/a0"])


@pytest.mark.parametrize("case", SOLVE_CASES)
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("solver", ["gmres", "fgmres"])
def test_solves(oracle, golden, case, kind, solver):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pc = oracle.precond(kind, A, nparts, 1, part)
    b = golden[f"{case}/b"]
    fn = oracle.gmres if solver == "gmres" else oracle.fgmres
    r = fn(A, b, np.zeros(A.nrows), pc, restart=30, max_iter=500, tol=1e-10, hist_cap=600)
    key = f"{case}/{solver}/{kind}"
    assert r["iterations"] == int(golden[key + "/iterations"])
    assert r["converged"] == bool(golden[key + "/converged"])
    assert close(r["x"], golden[key + "/x"], 1e-11)
    assert close(r["history"], golden[key + "/history"], 1e-9)


# ------------------------------------------------------------ reference tests
def test_identity_kat(oracle):
    """tests/test_gmres.cpp:27-44"""
    n = 10
    A = HostCSR(np.arange(n + 1), np.arange(n), np.ones(n))
    b = np.arange(1, 11, dtype=np.float64)
    r = oracle.gmres(A, b, np.zeros(n), None, restart=10, max_iter=1000, tol=1e-12)
    assert r["converged"] and r["iterations"] <= 2
    assert np.abs(r["x"] - b).sum() < 1e-10


@pytest.mark.parametrize("kind", [None, "jacobi", "ilu0"])
def test_small_spd_kat(oracle, kind):
    """tests/test_gmres.cpp:46-92"""
    A = HostCSR([0, 2, 5, 7], [0, 1, 0, 1, 2, 1, 2], [4, 1, 1, 3, 1, 1, 2])
    xe = np.array([1.0, 2.0, 3.0])
    b = oracle.spmv(A, xe)
    pc = oracle.precond(kind, A) if kind else None
    r = oracle.gmres(A, b, np.zeros(3), pc)
    assert r["converged"]
    assert np.abs(r["x"] - xe).sum() < 1e-8


def test_poisson5_kat(oracle, golden):
    """tests/test_gmres.cpp:94-142"""
    A = HostCSR(golden["kat/p2d5/row_ptr"], golden["kat/p2d5/col_idx"], golden["kat/p2d5/vals"])
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    pc = oracle.precond("ilu0", A)
    r = oracle.gmres(A, b, np.zeros(n), pc, restart=25, tol=1e-10)
    assert r["converged"] and r["residual_norm"] < 1e-10
    assert np.abs(r["x"] - 1.0).sum() < 1e-6


def _poisson(oracle, nx):
    rp, ci, v = oracle.poisson2d(nx, nx)
    return HostCSR(rp, ci, v)


def _blocks(n, p):
    return (np.arange(n) * p // n).astype(np.int32)


def test_schwarz_kats(oracle):
    """tests/test_schwarz.cpp:26-149 (with a contiguous-block partition in
    place of METIS)."""
    A = _poisson(oracle, 20)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    for kind in ("asm", "ras"):
        pc = oracle.precond(kind, A, 4, 1, _blocks(n, 4))
        r = oracle.gmres(A, b, np.zeros(n), pc, restart=30, max_iter=500, tol=1e-10)
        assert r["converged"] and r["residual_norm"] < 1e-9
    A = _poisson(oracle, 30)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    its = {}
    for kind in ("asm", "ras"):
        pc = oracle.precond(kind, A, 8, 2, _blocks(n, 8))
        r = oracle.gmres(A, b, np.zeros(n), pc, restart=50, max_iter=1000, tol=1e-10)
        assert r["converged"]
        its[kind] = r["iterations"]
    assert its["ras"] <= its["asm"] + 5
    A = _poisson(oracle, 20)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    it = []
    for ov in (0, 2):
        pc = oracle.precond("ras", A, 4, ov, _blocks(n, 4))
        it.append(oracle.gmres(A, b, np.zeros(n), pc, restart=30, max_iter=500, tol=1e-10)["iterations"])
    assert it[1] <= it[0]


def test_two_level_kats(oracle):
    """tests/test_two_level.cpp:27-143"""
    A = _poisson(oracle, 30)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    for kind in ("twolevel_asm", "twolevel_ras"):
        pc = oracle.precond(kind, A, 8, 1, _blocks(n, 8))
        r = oracle.gmres(A, b, np.zeros(n), pc, restart=50, max_iter=500, tol=1e-10)
        assert r["converged"] and r["residual_norm"] < 1e-9
    A = _poisson(oracle, 40)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    r1 = oracle.gmres(A, b, np.zeros(n), oracle.precond("ras", A, 16, 1, _blocks(n, 16)),
                      restart=50, max_iter=1000, tol=1e-10)
    r2 = oracle.gmres(A, b, np.zeros(n), oracle.precond("twolevel_ras", A, 16, 1, _blocks(n, 16)),
                      restart=50, max_iter=1000, tol=1e-10)
    assert r1["converged"] and r2["converged"]
    assert r2["iterations"] <= r1["iterations"] + 5
    A = _poisson(oracle, 30)
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    for p in (4, 8, 16):
        pc = oracle.precond("twolevel_ras", A, p, 1, _blocks(n, p))
        assert oracle.gmres(A, b, np.zeros(n), pc, restart=50, max_iter=500, tol=1e-10)["converged"]


def test_level_schedule_is_a_valid_order(oracle, golden):
    """Levels: every row depends only on rows of strictly lower level."""
    A = golden_matrix(golden, "p3d_slabs")
    lu, dg = oracle.ilu0_factor(A)
    lo, up = oracle.levels(A, dg)
    for i in range(A.nrows):
        for e in range(A.row_ptr[i], A.row_ptr[i + 1]):
            c = A.col_idx[e]
            if c < i:
                assert lo[c] < lo[i]
            if c > i:
                assert up[c] < up[i]
