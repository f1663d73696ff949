"""The lagged two-pass CGS2 of the GMRES cycle (restart < 32, FP32 or FP64
basis).

Each Arnoldi step defers the second projection of its new basis vector to the
next step and corrects that step's Hessenberg column through the Arnoldi
relation; in exact arithmetic it is CGS2.  The residual estimates of the
first cycle must therefore follow the classic three-pass CGS2 of the FP64
solver (ortho=1) to FP32 accuracy for the FP32 basis and to near FP64
accuracy for the FP64 basis, and the FP32 solve with a restart of 31 (lagged)
must behave like one of 32 (classic).
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _setup(sg, n, nparts, sd):
    A = sg.make_varcoef_3d(n, n, n, 1.0, 4.0, 3)
    b = A.spmv(sg.uniform(A.nrows, seed=4))
    part = sg.partition_boxes(n, n, n, nparts, 0.08, 2)
    pc = sg.TwoLevelSchwarzPrecond(nparts, 1, sg.FineLevelType.RAS, part, sd, sd)
    pc.setup(A)
    return A, b, pc


def test_first_cycle_residual_estimates_match_fp64(sg):
    hist = {}
    for prec in (sg.FP64, sg.FP32):
        sd = sg.FP64 if prec == sg.FP64 else sg.FP32
        A, b, pc = _setup(sg, 32, 8, sd)
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=30, tol=1e-30,
                                                  tol_kind=sg.TOL_REF_ABS, precision=prec,
                                                  ortho=1 if prec == sg.FP64 else 0))
        hist[prec] = np.asarray(r.residual_history)
    h64, h32 = hist[sg.FP64], hist[sg.FP32]
    assert len(h64) == len(h32) == 30
    # relative to the FP64 estimates, scaled by the starting norm (GMRES-IR's
    # inner cycle works on the preconditioned residual, like the FP64 one)
    rel = np.abs(h32 / h32[0] - h64 / h64[0]) / (h64 / h64[0])
    assert rel[:20].max() <= 2e-3, rel


def test_fp64_lagged_matches_classic(sg):
    A, b, pc = _setup(sg, 32, 8, sg.FP64)
    hist, xs = {}, {}
    for ortho in (0, 1):
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=30, tol=1e-30,
                                                  tol_kind=sg.TOL_REF_ABS, precision=sg.FP64,
                                                  ortho=ortho))
        hist[ortho] = np.asarray(r.residual_history)
        xs[ortho] = x
    h0, h1 = hist[0], hist[1]
    assert len(h0) == len(h1) == 30
    # the same Krylov space to FP64 rounding: estimates agree to 1e-12 of the
    # starting norm, and to 1e-6 relative even after they have fallen far
    assert (np.abs(h0 - h1) / h1[0]).max() <= 1e-12
    assert (np.abs(h0 - h1) / h1).max() <= 1e-6
    assert np.linalg.norm(xs[0] - xs[1]) <= 1e-8 * np.linalg.norm(xs[1])
    # and both solvers reach the target with the same iteration count (+-1)
    its = []
    for ortho in (0, 1):
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=3000, tol=1e-8,
                                                  tol_kind=sg.TOL_TRUE_REL, precision=sg.FP64,
                                                  ortho=ortho))
        assert r.converged and r.true_rel_residual <= 1e-8
        its.append(r.iterations)
    assert abs(its[0] - its[1]) <= 1, its


@pytest.mark.parametrize("restart", [31, 32])
def test_lagged_and_classic_restart_lengths(sg, restart):
    A, b, pc = _setup(sg, 40, 8, sg.FP32)
    Af, bf, pcf = _setup(sg, 40, 8, sg.FP64)
    x = np.zeros(A.nrows)
    r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=restart, max_iter=3000, tol=1e-8,
                                              tol_kind=sg.TOL_TRUE_REL, precision=sg.FP32))
    xf = np.zeros(Af.nrows)
    rf = sg.gmres(Af, bf, xf, pcf, sg.GMRESParams(restart=restart, max_iter=3000, tol=1e-8,
                                                  tol_kind=sg.TOL_TRUE_REL, precision=sg.FP64))
    assert r.converged and r.true_rel_residual <= 1e-8
    assert r.iterations <= 1.1 * rf.iterations + 3, (r.iterations, rf.iterations)


def test_lagged_cycle_odd_size_and_short_restart(sg):
    # n = 13^3 is not a multiple of the 4-element vectors: tail elements
    A = sg.make_poisson_3d(13, 13, 13)
    b = A.spmv(sg.uniform(A.nrows, seed=8))
    pc = sg.RASPrecond(4, 1, factor_dtype=sg.FP32, sweep_dtype=sg.FP32)
    pc.setup(A)
    for restart in (1, 2, 5, 17):
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=restart, max_iter=5000, tol=1e-9,
                                                  tol_kind=sg.TOL_TRUE_REL, precision=sg.FP32))
        assert r.converged and r.true_rel_residual <= 1e-9, (restart, r)
        res = np.linalg.norm(b - A.spmv(x)) / np.linalg.norm(b)
        assert res <= 1e-9
