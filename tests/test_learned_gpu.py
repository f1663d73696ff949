"""Learned coarse-correction stage on the GPU against the oracle
(oracle/learned_oracle.py), plus what the trained stage gains inside FGMRES.

Tolerances.  The GPU network stores weights, activations and activation
gradients in BF16 and accumulates in FP32; the oracle rounds the same
tensors to BF16 and accumulates in FP64.  The two differ by FP32 rounding of
the accumulations, which now and then moves a stored activation by one BF16
ulp (2^-8 relative): outputs agree to a relative L2 error of 5e-3, gradients
to 2e-2 per layer.  Training pairs are FP64 arithmetic stored in FP32
(relative 1e-6).
"""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

from oracle import learned_oracle as lo

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def _he_params(seed, c=1.7, bias=0.05):
    rng = np.random.default_rng(seed)
    p = np.zeros(lo.NUM_PARAMS)
    for l in range(lo.LAYERS):
        fan = 27 * (2 if l == 0 else 16)
        base = l * lo.LAYER_P
        p[base: base + lo.LAYER_W] = rng.uniform(-1, 1, lo.LAYER_W) * np.sqrt(6.0 / fan)
        p[base + lo.LAYER_W: base + lo.LAYER_P] = rng.uniform(-bias, bias, 16)
    p[: lo.NET_PARAMS] *= lo.param_mask()
    p[lo.NET_PARAMS] = c
    return p.astype(np.float32)


@pytest.fixture(scope="module")
def stage32(sg):
    st = sg.LearnedCorrection(32)
    yield st
    st.close()


def test_parameter_count(sg):
    assert sg.learned.NUM_PARAMS == lo.NUM_PARAMS


@pytest.mark.parametrize("batch", [1, 3])
def test_forward_matches_oracle(stage32, batch):
    p = _he_params(11)
    stage32.weights = p
    rng = np.random.default_rng(12 + batch)
    x2 = rng.standard_normal((batch, stage32.nc, 2)).astype(np.float32)
    y = stage32.forward(x2)
    yo, _ = lo.forward(p.astype(np.float64), x2, 16, emulate_bf16=True)
    assert _rel(y, yo) <= 5e-3, _rel(y, yo)
    assert np.max(np.abs(y - yo)) <= 3e-2 * np.max(np.abs(yo))


@pytest.mark.parametrize("nx", [16, 48])
def test_forward_matches_oracle_on_partial_tiles(sg, nx):
    """Network grids whose edge is not a multiple of the convolution tile's
    16 y rows (nx = 48: 24^3, nx = 16: 8^3): the TMA halo reads zeros past
    the volume and the rows past it are not stored."""
    st = sg.LearnedCorrection(nx)
    try:
        p = _he_params(31)
        st.weights = p
        rng = np.random.default_rng(32)
        x2 = rng.standard_normal((2, st.nc, 2)).astype(np.float32)
        y = st.forward(x2)
        yo, _ = lo.forward(p.astype(np.float64), x2, nx // 2, emulate_bf16=True)
        assert _rel(y, yo) <= 5e-3, _rel(y, yo)
    finally:
        st.close()


def test_weights_round_trip_and_padding(stage32):
    p = _he_params(13)
    q = p.copy()
    q[: lo.NET_PARAMS][lo.param_mask() == 0] = 1.0  # padded entries are forced to 0
    stage32.weights = q
    assert np.array_equal(stage32.weights, p)


@pytest.mark.parametrize("batch", [1, 2])
def test_gradient_matches_oracle(stage32, batch):
    p = _he_params(21)
    stage32.weights = p
    rng = np.random.default_rng(22 + batch)
    x2 = rng.standard_normal((batch, stage32.nc, 2)).astype(np.float32)
    t = rng.standard_normal((batch, stage32.nc)).astype(np.float32)
    loss, g = stage32.gradient(x2, t)
    lo_loss, go = lo.loss_and_grad(p.astype(np.float64), x2, t, 16, emulate_bf16=True)
    assert abs(loss - lo_loss) <= 1e-3 * lo_loss
    for l in range(lo.LAYERS):
        sl = slice(l * lo.LAYER_P, (l + 1) * lo.LAYER_P)
        assert _rel(g[sl], go[sl]) <= 2e-2, (l, _rel(g[sl], go[sl]))
    assert np.all(g[lo.param_mask() == 0] == 0)


def _problem(sg, oracle, N, NP, seed, fp64=True):
    A = sg.make_varcoef_3d(N, N, N, 1.0, 8.0 * N / 96, seed)
    part = sg.partition_boxes(N, N, N, NP, 0.08, 7)
    dt = sg.FP64 if fp64 else sg.FP32
    M = sg.TwoLevelSchwarzPrecond(NP, 1, sg.FineLevelType.RAS, partition=part,
                                  factor_dtype=dt, sweep_dtype=dt)
    M.setup(A)
    S = sp.csr_matrix((A.vals, A.col_idx, A.row_ptr), shape=(A.nrows, A.nrows))
    opc = oracle.precond("twolevel_ras", A, NP, 1, part) if oracle is not None else None
    return A, M, S, opc


def test_training_pair_matches_oracle(sg, oracle):
    N = 32
    A, M, S, opc = _problem(sg, oracle, N, 8, 5)
    st = sg.LearnedCorrection(N)
    st.set_matrix(A)
    rng = np.random.default_rng(31)
    r = rng.standard_normal(A.nrows)
    e = rng.standard_normal(A.nrows)
    st.add_pair(M, r, e)
    assert st.num_samples == 1
    a, f, t = st.sample(0)
    ao, fo, to, eo, en_o = lo.training_pair(lambda x: S @ x, opc.apply, S.diagonal(), r, e, N)
    assert _rel(a, ao) <= 1e-6 and _rel(t, to) <= 1e-6
    assert np.max(np.abs(f - fo)) <= 1e-5
    err, en, fld = st.sample_fine(0)
    assert _rel(err, eo) <= 1e-6 and abs(en - en_o) <= 1e-5 * en_o and fld == 0
    st.clear_samples()
    assert st.num_samples == 0
    st.close()


def test_energy_gradient_matches_oracle(sg, oracle):
    """Energy-norm loss gradient over stored pairs of two fields (the GPU keeps
    one FP32 copy of each field's values) against the oracle."""
    N = 32
    st = sg.LearnedCorrection(N)
    mats = []
    rng = np.random.default_rng(51)
    for seed in (8, 9):
        A, M, S, _ = _problem(sg, None, N, 8, seed, fp64=True)
        st.set_matrix(A)
        for _ in range(2):
            st.add_pair(M, rng.standard_normal(A.nrows), rng.standard_normal(A.nrows))
        mats.append((A, S))
    assert st.num_samples == 4
    p = _he_params(52, c=3.0)
    st.weights = p
    st.set_loss("energy")
    loss, g = st.sample_gradient(0, 4)
    x2 = np.stack([np.stack(st.sample(i)[:2], axis=-1) for i in range(4)])
    fines = [st.sample_fine(i) for i in range(4)]
    err = np.stack([fi[0] for fi in fines]).astype(np.float64)
    energy = [fi[1] for fi in fines]
    assert [fi[2] for fi in fines] == [0, 0, 1, 1]
    S32 = [S.astype(np.float32).astype(np.float64) for _A, S in mats]
    spmvs = [S32[fi[2]].__matmul__ for fi in fines]
    lo_loss, go = lo.energy_loss_and_grad(p.astype(np.float64), x2, err, energy, spmvs, N)
    assert abs(loss - lo_loss) <= 2e-3 * lo_loss, (loss, lo_loss)
    for l in range(lo.LAYERS):
        sl = slice(l * lo.LAYER_P, (l + 1) * lo.LAYER_P)
        assert _rel(g[sl], go[sl]) <= 2e-2, (l, _rel(g[sl], go[sl]))
    # eval of the same samples gives the same loss
    assert abs(st.eval(0, 4) - loss) <= 1e-3 * loss
    st.close()


def test_stage_apply_matches_oracle(sg, oracle):
    N = 32
    A, M, S, opc = _problem(sg, oracle, N, 8, 6)
    st = sg.LearnedCorrection(N)
    st.set_matrix(A)
    p = _he_params(41)
    st.weights = p
    st.attach(M, stagnation=0.0)
    v = np.random.default_rng(42).standard_normal(A.nrows)
    z = M.apply(v)
    zo, z1o = lo.stage_apply(p.astype(np.float64), lambda x: S @ x, opc.apply, S.diagonal(), v, N)
    corr, corr_o = z - z1o, zo - z1o
    assert np.linalg.norm(corr_o) > 1e-3 * np.linalg.norm(z1o)  # the stage does something
    assert _rel(corr, corr_o) <= 2e-2, _rel(corr, corr_o)
    assert st.state()["applies"] >= 1
    # switched off: the plain preconditioner exactly
    st.enabled = False
    assert np.array_equal(M.apply(v), opc.apply(v)) or _rel(M.apply(v), opc.apply(v)) <= 1e-14
    st.enabled = True
    st.detach()
    assert _rel(M.apply(v), z1o) <= 1e-14
    st.close()


def test_gmres_rejects_a_learned_stage(sg):
    N = 32
    A, M, _S, _ = _problem(sg, None, N, 8, 7)
    st = sg.LearnedCorrection(N)
    st.set_matrix(A)
    st.init_weights(1)
    st.attach(M)
    b = np.ones(A.nrows)
    x = np.zeros(A.nrows)
    with pytest.raises(sg.SgError) as ei:
        sg.gmres(A, b, x, M, sg.GMRESParams(restart=30, max_iter=30, tol=1e-8))
    assert ei.value.status == 1
    st.close()


def test_create_rejects_bad_grids(sg):
    for bad in (30, 0, 24):
        with pytest.raises(sg.SgError):
            sg.LearnedCorrection(bad)
