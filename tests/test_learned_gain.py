"""What the trained learned stage gains inside FGMRES, and its fallback.

The stage is trained on the GPU (libsgmres's own forward/backward kernels and
Adam) from (residual, error) pairs of plain two-level RAS FGMRES solves over
seeded coefficient fields, then FGMRES(40) with and without the stage solves
held-out fields to an FP64 true relative residual of 1e-8.  The grid is 32^3
(a 16^3 network grid) with 8 box subdomains so that data generation and
training take seconds; the bench's learned workload runs the 96^3 case.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, NP = 32, 8
TRAIN_SEEDS = range(100, 124)
HELD_OUT = (900, 901, 902)


def _field(sg, seed):
    A = sg.make_varcoef_3d(N, N, N, 1.0, 8.0 * N / 96, seed)
    part = sg.partition_boxes(N, N, N, NP, 0.08, 7)
    M = sg.TwoLevelSchwarzPrecond(NP, 1, sg.FineLevelType.RAS, partition=part,
                                  factor_dtype=sg.FP32, sweep_dtype=sg.FP32)
    M.setup(A)
    return A, M


@pytest.fixture(scope="module")
def trained(sg):
    st = sg.LearnedCorrection(N)
    st.init_weights(0)
    for seed in TRAIN_SEEDS:
        A, M = _field(sg, seed)
        sg.collect_pairs(st, A, M, sg.uniform(A.nrows, seed + 5000))
    ntrain = st.num_samples
    for seed in (800, 801):  # validation fields
        A, M = _field(sg, seed)
        sg.collect_pairs(st, A, M, sg.uniform(A.nrows, seed + 5000))
    nval = st.num_samples - ntrain
    losses = st.train(0, ntrain, epochs=40, batch=8, lr=1e-3, seed=1)
    yield st, ntrain, nval, losses
    st.close()


def _solve(sg, A, M, b, precision, use_graph=True):
    x = np.zeros(A.nrows)
    res = sg.fgmres(A, b, x, M, sg.GMRESParams(restart=40, max_iter=400, tol=1e-8,
                                               tol_kind=sg.TOL_TRUE_REL, precision=precision,
                                               use_graph=use_graph))
    return res, x


def test_training_lowers_the_loss(trained):
    st, ntrain, nval, losses = trained
    assert ntrain == len(TRAIN_SEEDS) * 6 and nval == 12
    assert np.all(np.isfinite(losses))
    assert losses[-1] < 0.6 * losses[0], losses
    # held-out pairs: better than predicting zero (loss 1 after the output scaling)
    assert st.eval(ntrain, nval) < 0.8


@pytest.mark.parametrize("precision", ["fp32", "fp64"])
def test_learned_fgmres_beats_plain_on_held_out_fields(sg, trained, precision):
    st, _ntrain, _nval, _losses = trained
    prec = sg.FP32 if precision == "fp32" else sg.FP64
    plain, learned = [], []
    for seed in HELD_OUT:
        A, M = _field(sg, seed)
        xs = sg.uniform(A.nrows, seed + 5000)
        b = A.spmv(xs)
        r0, _ = _solve(sg, A, M, b, prec)
        st.set_matrix(A)
        st.attach(M, stagnation=0.5)
        r1, x1 = _solve(sg, A, M, b, prec)
        state = st.state()
        st.detach()
        assert r0.converged and r1.converged
        assert r0.true_rel_residual <= 1e-8 and r1.true_rel_residual <= 1e-8
        # the FP64 true residual of the returned x, recomputed here
        assert np.linalg.norm(b - A.spmv(x1)) / np.linalg.norm(b) <= 1e-8
        assert state["fallback_cycle"] == -1 and state["applies"] > 0
        plain.append(r0.iterations)
        learned.append(r1.iterations)
    print(f"\n{precision}: plain {plain} learned {learned}")
    assert np.mean(learned) <= 0.8 * np.mean(plain), (plain, learned)


def test_graph_and_eager_solves_agree(sg, trained):
    st = trained[0]
    A, M = _field(sg, HELD_OUT[0])
    b = A.spmv(sg.uniform(A.nrows, HELD_OUT[0] + 5000))
    st.set_matrix(A)
    st.attach(M, stagnation=0.5)
    rg, xg = _solve(sg, A, M, b, sg.FP32, use_graph=True)
    re, xe = _solve(sg, A, M, b, sg.FP32, use_graph=False)
    st.detach()
    assert rg.iterations == re.iterations
    assert np.array_equal(xg, xe)


def test_fallback_switches_off_a_harmful_stage(sg, trained):
    st = trained[0]
    good = st.weights
    try:
        bad = good.copy()
        bad[-1] = 1e4  # output scale: the correction swamps M v
        st.weights = bad
        A, M = _field(sg, HELD_OUT[1])
        b = A.spmv(sg.uniform(A.nrows, HELD_OUT[1] + 5000))
        r_plain, _ = _solve(sg, A, M, b, sg.FP32)
        st.set_matrix(A)
        st.attach(M, stagnation=0.5)
        r, _x = _solve(sg, A, M, b, sg.FP32)
        state = st.state()
        st.detach()
        assert state["fallback_cycle"] >= 1 and state["enabled"] == 0
        assert r.converged and r.true_rel_residual <= 1e-8
        # after the switch the plain method finishes the solve
        assert r.iterations <= r_plain.iterations + 40 * (state["fallback_cycle"] + 1)
    finally:
        st.weights = good
