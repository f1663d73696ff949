"""Batched solver (sg_solve_batched): many independent systems and right-hand
sides in one call, checked against the single-system path.

The union of the systems is one block-diagonal matrix and the Schwarz
preconditioner is set up on it with a partition whose parts stay inside one
system, so its apply must equal the per-system preconditioners bit for bit.
Every (system, rhs) pair must then converge to an FP64 true relative residual
<= 1e-8 (recomputed here in FP64) in about as many iterations as the
single-system solver needs for the same pair: the FP64 batched Krylov loop
sums its dot products in a different order, so counts may differ by one or
two near the threshold.
"""
from __future__ import annotations

import numpy as np
import pytest
import scipy.sparse as sp

pytestmark = pytest.mark.gpu


def _small_batch(sg, seed=3, nsys=7):
    return sg.make_aniso_batch(nsys, seed=seed, nmin=20, nmax=44, rows_per_part=256,
                               min_parts=2, max_parts=6)


def _sub(prob, s):
    lo, hi = prob.sys_row_ptr[s], prob.sys_row_ptr[s + 1]
    S = sp.csr_matrix((prob.A.vals, prob.A.col_idx, prob.A.row_ptr), shape=(prob.n, prob.n))
    Ss = S[lo:hi, lo:hi].tocsr()
    Ss.sort_indices()
    return Ss, lo, hi


def _precond(sg, prob, fp64, part=None, nparts=None):
    dt = sg.FP64 if fp64 else sg.FP32
    return sg.RASPrecond(nparts or prob.nparts, 1,
                         partition=prob.partition if part is None else part,
                         factor_dtype=dt, sweep_dtype=dt)


@pytest.mark.parametrize("fp64", [True, False])
def test_block_diagonal_ras_equals_per_system_ras(sg, fp64):
    prob = _small_batch(sg)
    M = _precond(sg, prob, fp64)
    M.setup(prob.A)
    v = sg.uniform(prob.n, 11)
    y = M.apply(v)
    for s in range(prob.nsys):
        Ss, lo, hi = _sub(prob, s)
        As = sg.CSRMatrix(hi - lo, hi - lo, Ss.indptr.astype(np.int32),
                          Ss.indices.astype(np.int32), Ss.data)
        ps = prob.partition[lo:hi]
        ps = ps - ps.min()
        Ms = _precond(sg, prob, fp64, part=ps, nparts=int(ps.max()) + 1)
        Ms.setup(As)
        assert np.array_equal(Ms.apply(v[lo:hi]), y[lo:hi]), s


@pytest.mark.parametrize("ortho", [0, 1])
@pytest.mark.parametrize("precision", ["fp64", "fp32"])
def test_batched_solve_matches_single_solves(sg, precision, ortho):
    """ortho 0: the lagged two-pass CGS2 (restart < 32), ortho 1: three
    passes; the single-system solver runs the same form."""
    prob = _small_batch(sg)
    prec = sg.FP64 if precision == "fp64" else sg.FP32
    M = _precond(sg, prob, precision == "fp64")
    M.setup(prob.A)
    R = 3
    B = sg.uniform(R * prob.n, 21).reshape(R, prob.n)
    X = np.zeros_like(B)
    prm = sg.GMRESParams(restart=30, max_iter=2000, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                         precision=prec, ortho=ortho)
    res, t = sg.solve_batched(prob.A, M, prob.sys_row_ptr, R, B, X, prm)
    assert t > 0 and len(res) == R * prob.nsys
    assert np.all(res["converged"] == 1) and np.all(res["status"] == 0)
    S = sp.csr_matrix((prob.A.vals, prob.A.col_idx, prob.A.row_ptr), shape=(prob.n, prob.n))
    for r in range(R):
        for s in range(prob.nsys):
            i = r * prob.nsys + s
            Ss, lo, hi = _sub(prob, s)
            b = B[r, lo:hi]
            rel = np.linalg.norm(b - Ss @ X[r, lo:hi]) / np.linalg.norm(b)
            assert rel <= 1e-8 and abs(rel - res["true_rel_residual"][i]) <= 1e-9
            # the same pair through the single-system solver
            As = sg.CSRMatrix(hi - lo, hi - lo, Ss.indptr.astype(np.int32),
                              Ss.indices.astype(np.int32), Ss.data)
            ps = prob.partition[lo:hi] - prob.partition[lo:hi].min()
            Ms = _precond(sg, prob, precision == "fp64", part=ps, nparts=int(ps.max()) + 1)
            Ms.setup(As)
            xs = np.zeros(hi - lo)
            rs = sg.gmres(As, b, xs, Ms, prm)
            assert rs.converged
            slack = 2 if precision == "fp64" else 4
            assert abs(rs.iterations - int(res["iterations"][i])) <= slack, \
                (r, s, rs.iterations, res["iterations"][i])


def test_batched_graph_and_eager_agree_and_x0_is_used(sg):
    prob = _small_batch(sg, seed=5, nsys=5)
    M = _precond(sg, prob, False)
    M.setup(prob.A)
    B = sg.uniform(2 * prob.n, 31).reshape(2, prob.n)
    outs = []
    for graph in (True, False):
        X = np.zeros_like(B)
        prm = sg.GMRESParams(restart=20, max_iter=2000, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                             precision=sg.FP32, use_graph=graph)
        res, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 2, B, X, prm)
        outs.append((res, X))
    assert np.array_equal(outs[0][0]["iterations"], outs[1][0]["iterations"])
    assert np.array_equal(outs[0][1], outs[1][1])
    # warm start from the solution: every pair is done before the first cycle
    X = outs[0][1].copy()
    res, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 2, B, X,
                              sg.GMRESParams(restart=20, max_iter=2000, tol=1e-8,
                                             tol_kind=sg.TOL_TRUE_REL, precision=sg.FP32))
    assert np.all(res["iterations"] == 0) and np.all(res["converged"] == 1)


def test_batched_device_arrays(sg):
    torch = pytest.importorskip("torch")
    prob = _small_batch(sg, seed=6, nsys=4)
    M = _precond(sg, prob, False)
    M.setup(prob.A)
    B = sg.uniform(prob.n, 41).reshape(1, prob.n)
    Xh = np.zeros_like(B)
    res_h, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 1, B, Xh)
    Bd = torch.from_numpy(B).cuda()
    Xd = torch.zeros_like(Bd)
    res_d, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 1, Bd, Xd)
    assert np.array_equal(res_h["iterations"], res_d["iterations"])
    assert np.array_equal(Xh, Xd.cpu().numpy())


def test_batched_rejects_coupled_systems_and_crossing_parts(sg):
    prob = _small_batch(sg, seed=7, nsys=3)
    bad = prob.partition.copy()
    lo1 = prob.sys_row_ptr[1]
    bad[lo1] = bad[lo1 - 1]  # a row of system 1 in a part of system 0
    M = sg.RASPrecond(prob.nparts, 1, partition=bad, factor_dtype=sg.FP32,
                      sweep_dtype=sg.FP32)
    M.setup(prob.A)
    B = np.ones((1, prob.n))
    with pytest.raises(sg.SgError) as ei:
        sg.solve_batched(prob.A, M, prob.sys_row_ptr, 1, B, np.zeros_like(B))
    assert "spans systems" in str(ei.value)
    # a matrix whose rows couple two systems
    with pytest.raises(sg.SgError) as ei:
        srp = prob.sys_row_ptr.copy()
        srp[1] += 1
        M2 = _precond(sg, prob, False)
        M2.setup(prob.A)
        sg.solve_batched(prob.A, None, srp, 1, B, np.zeros_like(B))
    assert "couples" in str(ei.value)
    with pytest.raises(sg.SgError):
        sg.solve_batched(prob.A, None, prob.sys_row_ptr, 1, B, np.zeros_like(B),
                         sg.GMRESParams(restart=40))


@pytest.mark.parametrize("launch", ["per_subdomain", "persistent", 3])
@pytest.mark.parametrize("fdt", ["fp32", "bf16"])
def test_four_rhs_sweep_equals_single_rhs_solves(sg, launch, fdt):
    """Four right-hand sides go through one sweep that reads every level
    record once for all of them; per right-hand side it does the
    single-vector arithmetic, so a batched solve with four right-hand sides
    must give the bits of four one-right-hand-side solves.  Both launch
    shapes (a CTA per subdomain; resident CTAs looping over subdomains from
    a work counter, here also a grid of three CTAs that each take ~10
    subdomains) give the same bits."""
    prob = _small_batch(sg, seed=8, nsys=9)
    f = sg.BF16 if fdt == "bf16" else sg.FP32
    M = sg.RASPrecond(prob.nparts, 1, partition=prob.partition, factor_dtype=f,
                      sweep_dtype=sg.FP32, sweep_launch=launch)
    M.setup(prob.A)
    assert M.check() == 0
    prm = sg.GMRESParams(restart=30, max_iter=2000, tol=1e-8, tol_kind=sg.TOL_TRUE_REL,
                         precision=sg.FP32)
    B = sg.uniform(4 * prob.n, seed=21).reshape(4, prob.n)
    X4 = np.zeros_like(B)
    r4, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 4, B, X4, prm)
    assert M.check() == 0  # the four-vector ring schedule holds too
    for rr in range(4):
        X1 = np.zeros((1, prob.n))
        r1, _ = sg.solve_batched(prob.A, M, prob.sys_row_ptr, 1, B[rr:rr + 1].copy(), X1, prm)
        assert np.array_equal(X1[0], X4[rr]), rr
        assert np.array_equal(r1["iterations"], r4["iterations"][rr * prob.nsys:(rr + 1) * prob.nsys])
    assert np.all(r4["converged"] == 1) and r4["true_rel_residual"].max() <= 1e-8
