"""The reference's own Schwarz and two-level known-answer tests, run on the
GPU path (the oracle runs the same assertions in test_oracle_pins.py).

Restated from tests/test_schwarz.cpp:26-149 and tests/test_two_level.cpp:27-143
of the reference, with a contiguous-block partition in place of METIS (the
partition both sides take).  The assertions are the reference's: convergence
below the tolerance, RAS within 5 iterations of ASM, more overlap never
slower, two-level within 5 iterations of one-level RAS, two-level converging
for 4, 8 and 16 parts.  Each iteration count is also checked against the
oracle's on the same system (within 3), since both follow the reference's
arithmetic.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _blocks(n, p):
    return (np.arange(n) * p // n).astype(np.int32)


def _pc(sg, kind, p, ov, part):
    if kind == "asm":
        return sg.ASMPrecond(p, ov, partition=part)
    if kind == "ras":
        return sg.RASPrecond(p, ov, partition=part)
    fine = sg.FineLevelType.ASM if kind == "twolevel_asm" else sg.FineLevelType.RAS
    return sg.TwoLevelSchwarzPrecond(p, ov, fine, part)


def _solve(sg, A, kind, p, ov, restart, max_iter):
    n = A.nrows
    b = A.spmv(np.ones(n))
    pc = _pc(sg, kind, p, ov, _blocks(n, p))
    pc.setup(A)
    x = np.zeros(n)
    return sg.gmres(A, b, x, pc, sg.GMRESParams(restart=restart, max_iter=max_iter, tol=1e-10))


def _oracle_its(oracle, A, kind, p, ov, restart, max_iter):
    n = A.nrows
    b = oracle.spmv(A, np.ones(n))
    pc = oracle.precond(kind, A, p, ov, _blocks(n, p))
    r = oracle.gmres(A, b, np.zeros(n), pc, restart=restart, max_iter=max_iter, tol=1e-10)
    return r["iterations"]


def test_schwarz_kats_on_gpu(sg, oracle):
    A = sg.make_poisson_2d(20, 20)
    for kind in ("asm", "ras"):
        r = _solve(sg, A, kind, 4, 1, 30, 500)
        assert r.converged and r.residual_norm < 1e-9, (kind, r)
        assert abs(r.iterations - _oracle_its(oracle, A, kind, 4, 1, 30, 500)) <= 3
    A = sg.make_poisson_2d(30, 30)
    its = {}
    for kind in ("asm", "ras"):
        r = _solve(sg, A, kind, 8, 2, 50, 1000)
        assert r.converged, (kind, r)
        its[kind] = r.iterations
    assert its["ras"] <= its["asm"] + 5, its
    A = sg.make_poisson_2d(20, 20)
    it = [_solve(sg, A, "ras", 4, ov, 30, 500).iterations for ov in (0, 2)]
    assert it[1] <= it[0], it


def test_two_level_kats_on_gpu(sg, oracle):
    A = sg.make_poisson_2d(30, 30)
    for kind in ("twolevel_asm", "twolevel_ras"):
        r = _solve(sg, A, kind, 8, 1, 50, 500)
        assert r.converged and r.residual_norm < 1e-9, (kind, r)
        assert abs(r.iterations - _oracle_its(oracle, A, kind, 8, 1, 50, 500)) <= 3
    A = sg.make_poisson_2d(40, 40)
    r1 = _solve(sg, A, "ras", 16, 1, 50, 1000)
    r2 = _solve(sg, A, "twolevel_ras", 16, 1, 50, 1000)
    assert r1.converged and r2.converged
    assert r2.iterations <= r1.iterations + 5, (r1.iterations, r2.iterations)
    A = sg.make_poisson_2d(30, 30)
    for p in (4, 8, 16):
        assert _solve(sg, A, "twolevel_ras", p, 1, 50, 500).converged, p
