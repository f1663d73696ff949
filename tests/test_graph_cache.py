"""Reuse of the captured restart cycle across solves.

A solve captures its restart cycle as a CUDA graph once and later solves
replay it while nothing the capture baked in has changed.  These tests check
that a reused cycle gives bit-identical results to a fresh capture, and that
every change that alters the launches (preconditioner re-set-up, learned
stage attach/detach, SpMV format, new vectors, restart length, precision)
captures again instead of replaying stale pointers.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

N, NP = 24, 8


def _params(sg, **kw):
    base = dict(restart=20, max_iter=2000, tol=1e-9, tol_kind=sg.TOL_TRUE_REL,
                precision=sg.FP32)
    base.update(kw)
    return sg.GMRESParams(**base)


def _problem(sg, seed=11):
    A = sg.make_varcoef_3d(N, N, N, 1.0, 3.0, seed)
    part = sg.partition_boxes(N, N, N, NP, 0.08, 3)
    b = A.spmv(sg.uniform(A.nrows, 5))
    return A, part, b


def _pc(sg, part, ctx):
    return sg.TwoLevelSchwarzPrecond(NP, 1, sg.FineLevelType.RAS, partition=part,
                                     factor_dtype=sg.BF16, sweep_dtype=sg.FP32, ctx=ctx)


def test_repeated_solves_reuse_the_cycle_bit_identically(sg):
    ctx = sg.Context(0)
    A, part, b = _problem(sg)
    A.upload(ctx)
    M = _pc(sg, part, ctx)
    M.setup(A)
    p = _params(sg)
    xs = []
    c0 = ctx.capture_count
    for _ in range(3):
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, M, p)
        assert r.converged
        xs.append(x)
    assert ctx.capture_count == c0 + 1
    assert np.array_equal(xs[0], xs[1]) and np.array_equal(xs[0], xs[2])
    # a new right-hand side in the same (staging) buffer is picked up
    b2 = 2.0 * b
    x2 = np.zeros(A.nrows)
    assert sg.gmres(A, b2, x2, M, p).converged
    assert ctx.capture_count == c0 + 1
    assert np.allclose(x2, 2.0 * xs[0], rtol=1e-6, atol=1e-9 * np.abs(xs[0]).max())


def test_resetup_and_new_objects_capture_again(sg):
    ctx = sg.Context(0)
    A1, part, b = _problem(sg, 11)
    A2, _, _ = _problem(sg, 12)
    A1.upload(ctx)
    A2.upload(ctx)
    M = _pc(sg, part, ctx)
    M.setup(A1)
    p = _params(sg)
    x = np.zeros(A1.nrows)
    sg.gmres(A1, b, x, M, p)
    c1 = ctx.capture_count
    # same preconditioner object, new coefficients: must not replay the old cycle
    M.setup(A2)
    xr = np.zeros(A2.nrows)
    rr = sg.gmres(A2, b, xr, M, p)
    assert ctx.capture_count == c1 + 1
    fresh = _pc(sg, part, ctx)
    fresh.setup(A2)
    xf = np.zeros(A2.nrows)
    rf = sg.gmres(A2, b, xf, fresh, p)
    assert rr.iterations == rf.iterations
    assert np.array_equal(xr, xf)
    # restart length and precision are part of the capture
    c2 = ctx.capture_count
    sg.gmres(A2, b, np.zeros(A2.nrows), fresh, _params(sg, restart=15))
    sg.gmres(A2, b, np.zeros(A2.nrows), fresh, _params(sg, precision=sg.FP64))
    assert ctx.capture_count == c2 + 2


def test_device_vectors_and_format_change(sg):
    torch = pytest.importorskip("torch")
    ctx = sg.Context(0)
    A, part, b = _problem(sg)
    A.upload(ctx)
    M = _pc(sg, part, ctx)
    M.setup(A)
    p = _params(sg)
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros_like(bd)
    stream = torch.cuda.ExternalStream(ctx.stream)
    sg.gmres(A, bd, xd, M, p)
    ref = xd.cpu().numpy()
    c = ctx.capture_count
    with torch.cuda.stream(stream):
        xd.zero_()
    sg.gmres(A, bd, xd, M, p)
    assert ctx.capture_count == c
    assert np.array_equal(xd.cpu().numpy(), ref)
    # another solution buffer: a new capture, same result
    xd2 = torch.zeros_like(bd)
    sg.gmres(A, bd, xd2, M, p)
    assert ctx.capture_count == c + 1
    assert np.array_equal(xd2.cpu().numpy(), ref)
    # switching the SpMV format recaptures; SpMV results are format-independent
    A.format = 2 if A.format == 1 else 1
    with torch.cuda.stream(stream):
        xd2.zero_()
    sg.gmres(A, bd, xd2, M, p)
    assert ctx.capture_count == c + 2
    assert np.array_equal(xd2.cpu().numpy(), ref)


def test_learned_attach_detach_captures_again(sg):
    ctx = sg.Context(0)
    n = 32
    A = sg.make_varcoef_3d(n, n, n, 1.0, 3.0, 4)
    part = sg.partition_boxes(n, n, n, 8, 0.08, 3)
    b = A.spmv(sg.uniform(A.nrows, 6))
    A.upload(ctx)
    M = _pc(sg, part, ctx)
    M.setup(A)
    st = sg.LearnedCorrection(n, ctx=ctx)
    st.init_weights(7)
    w = st.weights
    w[-1] = 1.0
    st.weights = w
    st.set_matrix(A)
    p = _params(sg)
    x0 = np.zeros(A.nrows)
    r_plain = sg.fgmres(A, b, x0, M, p)
    c = ctx.capture_count
    st.attach(M)
    x1 = np.zeros(A.nrows)
    r_learned = sg.fgmres(A, b, x1, M, p)
    assert ctx.capture_count == c + 1
    st.detach()
    x2 = np.zeros(A.nrows)
    r_again = sg.fgmres(A, b, x2, M, p)
    assert ctx.capture_count == c + 2
    assert r_again.iterations == r_plain.iterations
    assert np.array_equal(x2, x0)
    assert r_learned.converged
    st.close()
