"""Host preconditioners (sg_precond_create_host): the flexible FGMRES apply
(FlexApply / fgmres_flex, src/core/fgmres.h:37, src/core/fgmres.cpp:164-172)
and Preconditioner plug-ins of the caller's own, applied in stream order on
a CUDA host-function thread inside the GPU solves.

A host Jacobi gives the GPU Jacobi's results (GMRES, FGMRES, BiCGSTAB,
graph and eager); FGMRES applies the function to the normalised basis
vector, as the reference does (checked against the oracle's FGMRES with the
same Jacobi); a nonlinear apply still converges in FGMRES; an exception in
the function surfaces as SG_ERR_CALLBACK with its message."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import HostCSR

pytestmark = pytest.mark.gpu


def _jacobi(A):
    d = np.array([A.vals[A.row_ptr[i] + np.where(A.col_idx[A.row_ptr[i]:A.row_ptr[i + 1]] == i)
                         [0][0]] for i in range(A.nrows)])
    inv = 1.0 / d

    def apply(x, y):
        np.multiply(inv, x, out=y)
    return apply


@pytest.mark.parametrize("solver", ["gmres", "fgmres", "bicgstab"])
@pytest.mark.parametrize("graph", [True, False])
def test_host_jacobi_matches_device_jacobi(sg, solver, graph):
    A = sg.make_varcoef_3d(16, 16, 16, 1.0, 4.0, seed=2)
    b = A.spmv(sg.uniform(A.nrows, seed=3))
    H = sg.HostPreconditioner(_jacobi(A), A.nrows)
    D = sg.JacobiPrecond()
    D.setup(A)
    fn = getattr(sg, solver)
    prm = sg.GMRESParams(restart=30, max_iter=2000, tol=1e-10, use_graph=graph)
    xh, xd = np.zeros(A.nrows), np.zeros(A.nrows)
    rh = fn(A, b, xh, H, prm)
    rd = fn(A, b, xd, D, prm)
    assert rh.converged and rd.converged
    assert abs(rh.iterations - rd.iterations) <= 1, (rh.iterations, rd.iterations)
    assert np.linalg.norm(xh - xd) <= 1e-8 * np.linalg.norm(xd)


def test_flexible_apply_matches_oracle_fgmres(sg, oracle):
    """FGMRES with the host Jacobi against the oracle's FGMRES with Jacobi
    (the reference's fgmres): same iterations within 2, x within 1e-8."""
    A = sg.make_poisson_2d(40, 40)
    b = A.spmv(sg.uniform(A.nrows, seed=5))
    H = sg.HostPreconditioner(_jacobi(A), A.nrows)
    x = np.zeros(A.nrows)
    r = sg.fgmres(A, b, x, H, sg.GMRESParams(restart=30, max_iter=2000, tol=1e-10))
    Ho = HostCSR(A.row_ptr, A.col_idx, A.vals)
    ro = oracle.fgmres(Ho, b, np.zeros(A.nrows), oracle.precond("jacobi", Ho), restart=30,
                       max_iter=2000, tol=1e-10)
    assert r.converged and ro["converged"]
    assert abs(r.iterations - ro["iterations"]) <= 2
    assert np.linalg.norm(x - ro["x"]) <= 1e-8 * np.linalg.norm(ro["x"])


def test_nonlinear_flexible_apply(sg):
    """An apply that changes from call to call (a varying number of damped
    Jacobi sweeps on A z = v): FGMRES converges to the FP64 target."""
    A = sg.make_poisson_2d(32, 32)
    S = __import__("scipy.sparse", fromlist=["csr_matrix"]).csr_matrix(
        (A.vals, A.col_idx, A.row_ptr), shape=(A.nrows, A.nrows))
    dinv = 1.0 / S.diagonal()
    calls = [0]

    def apply(v, z):
        calls[0] += 1
        t = np.zeros_like(v)
        for _ in range(1 + calls[0] % 4):
            t += 0.8 * dinv * (v - S @ t)
        z[:] = t

    H = sg.HostPreconditioner(apply, A.nrows)
    b = A.spmv(sg.uniform(A.nrows, seed=6))
    x = np.zeros(A.nrows)
    r = sg.fgmres(A, b, x, H, sg.GMRESParams(restart=30, max_iter=3000, tol=1e-8,
                                              tol_kind=sg.TOL_TRUE_REL))
    assert r.converged and r.true_rel_residual <= 1e-8
    assert calls[0] >= r.iterations


def test_callback_error_surfaces(sg):
    A = sg.make_poisson_2d(16, 16)

    def bad(x, y):
        raise ValueError("plug-in failure 7")

    H = sg.HostPreconditioner(bad, A.nrows)
    with pytest.raises(sg.SgError) as ei:
        sg.gmres(A, np.ones(A.nrows), np.zeros(A.nrows), H, sg.GMRESParams(max_iter=40))
    assert ei.value.status == 10 and "plug-in failure 7" in str(ei.value)
    # another host preconditioner works after the error
    G = sg.HostPreconditioner(_jacobi(A), A.nrows)
    x = np.zeros(A.nrows)
    assert sg.gmres(A, A.spmv(np.ones(A.nrows)), x, G, sg.GMRESParams(tol=1e-10)).converged
    # the batched solver takes no host preconditioner
    with pytest.raises(sg.SgError) as ei:
        sg.solve_batched(A, G, np.array([0, A.nrows], np.int32), 1, np.ones((1, A.nrows)),
                         np.zeros((1, A.nrows)))
    assert ei.value.status == 1
