"""BiCGSTAB (src/core/bicgstab.h:57-204) and the analysis tools
(src/analysis/condition_estimator.h:94-191, spectral_analysis.h:30-97) on
the GPU against the reference's golden outputs (tests/golden/make_golden.py)
and the oracle.

BiCGSTAB reduces its dot products in another order than the reference's
serial loops, so the iterates differ by rounding: the test asks for the same
converged flag, iterations within 2 and x within 1e-8 (relative) of the
reference, and residual histories within 1e-6 relative over the first steps.
The Lanczos and power iterations likewise: extreme Ritz values within 1e-6
relative for the symmetric operators (none, Jacobi, ILU(0) -- the latter's
M^{-1}A is not symmetric but its Ritz values are well separated), the same
step counts within a few, and the same verdicts."""
from __future__ import annotations

import numpy as np
import pytest

from conftest import golden_matrix

pytestmark = pytest.mark.gpu

KINDS = ["none", "jacobi", "ilu0", "ras", "twolevel_ras"]
CASES = ["p2d_blocks", "p3d_slabs"]


def _gpu(sg, golden, case, kind):
    H = golden_matrix(golden, case)
    A = sg.CSRMatrix(H.nrows, H.ncols, H.row_ptr, H.col_idx, H.vals)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    M = None
    if kind == "jacobi":
        M = sg.JacobiPrecond()
    elif kind == "ilu0":
        M = sg.ILU0Precond()
    elif kind == "ras":
        M = sg.RASPrecond(nparts, 1, partition=part)
    elif kind == "twolevel_ras":
        M = sg.TwoLevelSchwarzPrecond(nparts, 1, sg.FineLevelType.RAS, part)
    if M is not None:
        M.setup(A)
    return A, M


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_bicgstab_matches_reference(sg, golden, case, kind):
    A, M = _gpu(sg, golden, case, kind)
    key = f"{case}/bicgstab/{kind}"
    b = golden[f"{case}/b"]
    x = np.zeros(A.nrows)
    r = sg.bicgstab(A, b, x, M, sg.GMRESParams(max_iter=500, tol=1e-10))
    assert r.converged == bool(golden[key + "/converged"])
    assert abs(r.iterations - int(golden[key + "/iterations"])) <= 2, (r.iterations,)
    xr = golden[key + "/x"]
    assert np.linalg.norm(x - xr) <= 1e-8 * np.linalg.norm(xr)
    hr = golden[key + "/history"]
    h = np.asarray(r.residual_history)
    k = min(len(h), len(hr), 5)
    np.testing.assert_allclose(h[:k], hr[:k], rtol=1e-6)
    assert r.true_rel_residual <= 1e-9


def test_bicgstab_true_residual_restarts(sg):
    """With the FP64 true-residual rule the solve restarts until ||b-Ax||/||b||
    meets the target; a device-resident b and x take the same path."""
    torch = pytest.importorskip("torch")
    A = sg.make_poisson_3d(20, 20, 20)
    xs = sg.uniform(A.nrows, seed=3)
    b = A.spmv(xs)
    M = sg.RASPrecond(8, 1, partition=sg.partition_boxes(20, 20, 20, 8, 0.1, seed=2))
    M.setup(A)
    prm = sg.GMRESParams(max_iter=2000, tol=1e-10, tol_kind=sg.TOL_TRUE_REL)
    x = np.zeros(A.nrows)
    r = sg.bicgstab(A, b, x, M, prm)
    assert r.converged and r.true_rel_residual <= 1e-10
    assert np.linalg.norm(b - A.spmv(x)) / np.linalg.norm(b) <= 1e-10
    bd = torch.from_numpy(b).cuda()
    xd = torch.zeros_like(bd)
    r2 = sg.bicgstab(A, bd, xd, M, prm)
    assert r2.iterations == r.iterations
    np.testing.assert_array_equal(xd.cpu().numpy(), x)


def test_bicgstab_nonfinite_rhs(sg):
    A = sg.make_poisson_2d(16, 16)
    b = np.ones(A.nrows)
    b[7] = np.nan
    with pytest.raises(sg.SgError) as ei:
        sg.bicgstab(A, b, np.zeros(A.nrows), None, sg.GMRESParams(max_iter=50, tol=1e-10))
    assert ei.value.status == 6  # SG_ERR_NONFINITE


@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_condition_and_spectral_match_reference(sg, golden, case, kind):
    A, M = _gpu(sg, golden, case, kind)
    c = sg.estimate_condition(A, M, 80, 42)
    g = golden[f"{case}/condition/{kind}"]
    assert c["valid"] == bool(g[4])
    assert abs(c["lanczos_steps"] - int(g[3])) <= 2
    if kind in ("none", "jacobi", "ilu0"):
        np.testing.assert_allclose([c["lambda_min"], c["lambda_max"]], g[:2], rtol=1e-6)
    else:  # nonsymmetric M^{-1}A: Ritz values are sensitive; same sign pattern, 5%
        np.testing.assert_allclose([c["lambda_min"], c["lambda_max"]], g[:2], rtol=5e-2)
    s = sg.estimate_spectral_radius(A, M, 200, 1e-6, 123)
    g = golden[f"{case}/spectral/{kind}"]
    assert s["convergence_ok"] == bool(g[2])
    assert abs(s["power_iters"] - int(g[1])) <= 3
    np.testing.assert_allclose(s["spectral_radius"], g[0], rtol=1e-5)
