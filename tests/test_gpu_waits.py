"""Bounded device waits of the TMA-fed subdomain sweep, made to run out on
purpose without any fault.

The sweep waits on mbarriers for its level records and, when it computes the
two-level coarse restriction itself, on a grid-wide arrival counter.  Every
such wait has a cycle budget; on expiry the CTA records an error word, drains
the bulk copies it issued and returns without writing y.  The test hook
`set_wait_test` makes one wait impossible to satisfy (mode 1: no record
group 0 is copied; mode 2: no CTA counts its restriction) with a ~1 ms
budget, so the give-up path runs: the call reports SG_ERR_DEVICE_TIMEOUT, y
keeps its previous contents, and the next call with the normal waits returns
the normal result (the error word and the restriction counters were
cleared)."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

TIMEOUT = 7  # SG_ERR_DEVICE_TIMEOUT


def _problem(sg, kind):
    A = sg.make_poisson_3d(24, 24, 24)
    part = sg.partition_boxes(24, 24, 24, 16, 0.1, seed=3)
    if kind == "twolevel":
        M = sg.TwoLevelSchwarzPrecond(16, 1, sg.FineLevelType.RAS, part, factor_dtype=sg.FP32,
                                      sweep_dtype=sg.FP32)
    else:
        M = sg.RASPrecond(16, 1, partition=part, factor_dtype=sg.FP32, sweep_dtype=sg.FP32)
    M.setup(A)
    assert M.sweep_choice()["sweep"] == "tma"
    return A, M


@pytest.mark.parametrize("kind,mode", [("ras", 1), ("twolevel", 1), ("twolevel", 2)])
def test_wait_runs_out_then_recovers(sg, kind, mode):
    torch = pytest.importorskip("torch")
    A, M = _problem(sg, kind)
    x = sg.uniform(A.nrows, seed=5)
    want = M.apply(x)
    xd = torch.from_numpy(x).cuda()
    yd = torch.full_like(xd, 123.0)
    M.set_wait_test(mode)
    with pytest.raises(sg.SgError) as ei:
        M.apply(xd, yd)
    assert ei.value.status == TIMEOUT
    torch.cuda.synchronize()
    assert bool(torch.all(yd == 123.0)), "a sweep that gave up wrote its output"
    # a second apply in the test mode fails the same way (the state was cleared)
    with pytest.raises(sg.SgError) as ei:
        M.apply(x)
    assert ei.value.status == TIMEOUT
    M.set_wait_test(0)
    got = M.apply(xd, yd)
    np.testing.assert_array_equal(got.cpu().numpy(), want)
    np.testing.assert_array_equal(M.apply(x), want)


def test_solve_reports_timeout_then_converges(sg):
    A, M = _problem(sg, "twolevel")
    b = A.spmv(sg.uniform(A.nrows, seed=6))
    prm = sg.GMRESParams(restart=20, max_iter=200, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                         precision=sg.FP32)
    M.set_wait_test(1)
    with pytest.raises(sg.SgError) as ei:
        sg.gmres(A, b, np.zeros(A.nrows), M, prm)
    assert ei.value.status == TIMEOUT
    M.set_wait_test(0)
    x = np.zeros(A.nrows)
    r = sg.gmres(A, b, x, M, prm)
    assert r.converged and r.true_rel_residual <= 1e-8


def test_wait_test_needs_the_wait(sg):
    A = sg.make_poisson_3d(12, 12, 12)
    part = sg.partition_boxes(12, 12, 12, 4, 0.0, seed=1)
    M = sg.RASPrecond(4, 1, partition=part, sweep="level")
    M.setup(A)
    with pytest.raises(sg.SgError) as ei:
        M.set_wait_test(1)
    assert ei.value.status == 8  # SG_ERR_UNSUPPORTED: this sweep has no record waits
    R = sg.RASPrecond(4, 1, partition=part)
    R.setup(A)
    with pytest.raises(sg.SgError) as ei:
        R.set_wait_test(2)  # one-level: no coarse restriction to wait for
    assert ei.value.status == 8


@pytest.mark.parametrize("mode", [1, 2])
def test_learned_convolution_wait_runs_out_then_recovers(sg, mode):
    """The tcgen05 convolution waits on one mbarrier for its TMA halo and
    weight copies and on another for its MMAs.  Mode 1 (2) makes the first
    (second) barrier expect 16 bytes (one arrival) that nothing supplies, with
    a ~1 ms budget: every CTA's wait runs out, the CTA supplies what was
    withheld, drains its real copies (MMAs), frees its tensor memory and
    leaves its tile unwritten; the call reports SG_ERR_DEVICE_TIMEOUT, and
    the next call with the normal waits returns the normal network output."""
    st = sg.LearnedCorrection(32)
    try:
        rng = np.random.default_rng(40 + mode)
        p = (rng.uniform(-1, 1, sg.learned.NUM_PARAMS) * 0.2).astype(np.float32)
        p[-1] = 1.0
        st.weights = p
        x2 = rng.standard_normal((2, st.nc, 2)).astype(np.float32)
        want = st.forward(x2)
        st.set_wait_test(mode)
        with pytest.raises(sg.SgError) as ei:
            st.forward(x2)
        assert ei.value.status == TIMEOUT
        st.set_wait_test(0)
        np.testing.assert_array_equal(st.forward(x2), want)
    finally:
        st.close()


def test_learned_wait_runs_out_inside_an_apply_and_a_solve(sg):
    """The same give-up path reached through the preconditioner the stage is
    attached to: an apply and an FGMRES solve report SG_ERR_DEVICE_TIMEOUT,
    and both succeed again once the normal waits are back."""
    N = 32
    A = sg.make_varcoef_3d(N, N, N, 1.0, 8.0 * N / 96, 3)
    part = sg.partition_boxes(N, N, N, 8, 0.08, 7)
    M = sg.TwoLevelSchwarzPrecond(8, 1, sg.FineLevelType.RAS, partition=part,
                                  factor_dtype=sg.FP32, sweep_dtype=sg.FP32)
    M.setup(A)
    st = sg.LearnedCorrection(N)
    try:
        st.set_matrix(A)
        rng = np.random.default_rng(43)
        p = (rng.uniform(-1, 1, sg.learned.NUM_PARAMS) * 0.1).astype(np.float32)
        p[-1] = 0.5
        st.weights = p
        st.attach(M, stagnation=0.0)
        v = rng.standard_normal(A.nrows)
        want = M.apply(v)
        b = rng.standard_normal(A.nrows)
        prm = sg.GMRESParams(restart=30, max_iter=300, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                             precision=sg.FP32)
        st.set_wait_test(1)
        with pytest.raises(sg.SgError) as ei:
            M.apply(v)
        assert ei.value.status == TIMEOUT
        short = sg.GMRESParams(restart=30, max_iter=5, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                               precision=sg.FP32)  # every wait that runs out costs ~1 ms
        with pytest.raises(sg.SgError) as ei:
            sg.fgmres(A, b, np.zeros(A.nrows), M, short)
        assert ei.value.status == TIMEOUT
        st.set_wait_test(0)
        np.testing.assert_array_equal(M.apply(v), want)
        res = sg.fgmres(A, b, np.zeros(A.nrows), M, prm)
        assert res.converged
        st.detach()
    finally:
        st.close()
