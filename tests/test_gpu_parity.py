"""GPU parity: the sm_103a kernels against the oracle and the reference's
golden vectors, through the C ABI.

Tolerances (FP64 unless stated):
  SpMV, ILU(0) factors, Jacobi / ILU(0) / RAS applies, A0: bit-exact -- the
      kernels round each product and difference in the reference's order.
  ASM apply: 1e-14 relative (overlap sums arrive in atomic order).
  two-level apply: 1e-12 relative (coarse solve by the explicit inverse built
      from the same LU factors).
  FP32 sweeps: 1e-5 relative; BF16 factors: 2e-2 relative.
  Solves (reference stopping rule): iterations within 3 of the reference
      (CGS2 in place of MGS), solutions within 1e-7 relative.
"""
from __future__ import annotations

import numpy as np
import pytest

from conftest import HostCSR, golden_matrix

pytestmark = pytest.mark.gpu

KINDS = ["jacobi", "ilu0", "asm", "ras", "twolevel_asm", "twolevel_ras"]
CASES = ["p2d_blocks", "p2d_scatter", "p3d_slabs"]


def to_sg(sg, A):
    return sg.CSRMatrix(A.nrows, A.ncols, A.row_ptr, A.col_idx, A.vals)


def make_pc(sg, kind, nparts, overlap, part, fdt=None, sdt=None, sweep="tma", sweep_threads=0):
    fdt = sg.FP64 if fdt is None else fdt
    sdt = sg.FP64 if sdt is None else sdt
    kw = {"sweep": sweep, "sweep_threads": sweep_threads}
    if kind == "jacobi":
        return sg.JacobiPrecond(sweep_dtype=sdt, **kw)
    if kind == "ilu0":
        return sg.ILU0Precond(factor_dtype=fdt, sweep_dtype=sdt, **kw)
    if kind == "asm":
        return sg.ASMPrecond(nparts, overlap, part, fdt, sdt, **kw)
    if kind == "ras":
        return sg.RASPrecond(nparts, overlap, part, fdt, sdt, **kw)
    ft = sg.FineLevelType.ASM if kind == "twolevel_asm" else sg.FineLevelType.RAS
    return sg.TwoLevelSchwarzPrecond(nparts, overlap, ft, part, fdt, sdt, **kw)


def rel(a, b):
    return np.abs(np.asarray(a) - np.asarray(b)).max() / max(np.abs(b).max(), 1e-300)


# ------------------------------------------------------------------ SpMV
@pytest.mark.parametrize("case", CASES)
def test_spmv_golden_bit_exact(sg, golden, case):
    A = to_sg(sg, golden_matrix(golden, case))
    y = A.spmv(golden[f"{case}/x"])
    assert np.array_equal(y, golden[f"{case}/spmv"])


def _irregular(n, seed):
    """Ragged rows: empty rows, a very long row (several windows), random columns."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, n)
    lens[n // 3] = 0
    lens[n // 2] = 3000
    rp = np.zeros(n + 1, np.int32)
    rp[1:] = np.cumsum(lens)
    ci = np.concatenate([np.sort(rng.choice(n, size=l, replace=l > n)) for l in lens]).astype(np.int32)
    v = rng.standard_normal(rp[-1])
    return HostCSR(rp, ci, v)


@pytest.mark.parametrize("fmt", [1, 2, 3])
@pytest.mark.parametrize("maker", ["p3d", "varcoef", "irregular", "tiny", "wide"])
def test_spmv_matches_oracle(sg, oracle, maker, fmt):
    if maker == "p3d":
        A = sg.make_poisson_3d(40, 37, 23)
    elif maker == "varcoef":
        A = sg.make_varcoef_3d(32, 32, 32, 1.0, 8.0, 5)
    elif maker == "irregular":
        H = _irregular(5000, 3)
        A = to_sg(sg, H)
    elif maker == "wide":
        # 3D Laplacian whose z-neighbours lie 40,000 rows away: no 16-bit offsets
        A = sg.make_poisson_3d(200, 200, 3)
    else:
        A = sg.make_poisson_2d(1, 3)
    x = sg.uniform(A.ncols, seed=11)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    try:
        A.format = fmt
    except sg.SgError as e:  # no SELL copy (padding too large) or no 16-bit offsets
        assert fmt >= 2 and e.status == 8
        # SELL is refused for padding > 25% (irregular, the 3-row matrix);
        # 16-bit offsets for columns more than 32767 rows away (wide)
        assert maker in ("irregular", "tiny") or (maker == "wide" and fmt == 3)
        return
    assert maker != "wide" or fmt != 3
    assert np.array_equal(A.spmv(x), oracle.spmv(H, x))


@pytest.mark.parametrize("variant", list(range(10)))
def test_every_sell_variant_matches_oracle(sg, oracle, variant):
    """Every launch variant the SpMV autotuner may pick (column width,
    residency, grid, pipelined kernel) gives the reference's bits."""
    A = sg.make_varcoef_3d(32, 32, 40, 1.0, 6.0, 9)
    x = sg.uniform(A.ncols, seed=12)
    A.set_spmv_variant(variant)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    assert np.array_equal(A.spmv(x), oracle.spmv(H, x))
    # and inside a mixed-precision solve (FP32 copy, same variant)
    b = A.spmv(sg.uniform(A.nrows, seed=13))
    pc = sg.RASPrecond(8, 1, factor_dtype=sg.FP32, sweep_dtype=sg.FP32)
    pc.setup(A)
    xs = np.zeros(A.nrows)
    r = sg.gmres(A, b, xs, pc, sg.GMRESParams(restart=30, max_iter=500, tol=1e-8,
                                             tol_kind=sg.TOL_TRUE_REL, precision=sg.FP32))
    assert r.converged and r.true_rel_residual <= 1e-8


@pytest.mark.parametrize("fmt", [1, 2, 3])
def test_solve_same_bits_in_both_formats(sg, fmt):
    """The SpMV storage is a pure performance choice: FP64 solves give the
    same bits whichever format runs."""
    A = sg.make_poisson_3d(30, 30, 30)
    b = A.spmv(sg.uniform(A.nrows, seed=3))
    pc = sg.RASPrecond(8, 1)
    pc.setup(A)
    out = []
    for f in (1, fmt):
        A.format = f
        x = np.zeros(A.nrows)
        sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=500, tol=1e-10))
        out.append(x)
    assert np.array_equal(out[0], out[1])


def test_spmv_device_pointers(sg):
    torch = pytest.importorskip("torch")
    A = sg.make_poisson_3d(20, 20, 20)
    x = sg.uniform(A.nrows, seed=2)
    xd = torch.from_numpy(x).cuda()
    yd = torch.empty_like(xd)
    A.spmv(xd, yd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), A.spmv(x))


# ------------------------------------------------------------------ BLAS-1
@pytest.mark.parametrize("n", [0, 1, 31, 1000, 262144 + 17])
def test_blas1_vs_reference_loops(sg, n):
    """dot/norm2 within 1e-14 relative (summation order); axpy/scale bit-exact
    (src/core/vector.h:11-44)."""
    x = sg.uniform(n, seed=5)
    y = sg.uniform(n, seed=6)
    ref_dot = 0.0
    for a, b in zip(x.tolist(), y.tolist()):
        ref_dot += a * b
    d = sg.dot(x, y)
    assert abs(d - ref_dot) <= 1e-14 * max(1.0, np.abs(x * y).sum())
    assert abs(sg.norm2(x) - np.sqrt(np.dot(x, x))) <= 1e-14 * max(1.0, np.sqrt(np.dot(x, x)))
    z = y.copy()
    sg.axpy(-0.37, x, z)
    assert np.array_equal(z, y + (-0.37) * x)
    w = x.copy()
    sg.scale(1.7, w)
    assert np.array_equal(w, x * 1.7)


def test_blas1_device_pointers(sg):
    torch = pytest.importorskip("torch")
    x = sg.uniform(100000, seed=1)
    y = sg.uniform(100000, seed=2)
    xd, yd = torch.from_numpy(x).cuda(), torch.from_numpy(y).cuda()
    assert sg.dot(xd, yd) == sg.dot(x, y)
    sg.axpy(2.0, xd, yd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), y + 2.0 * x)


# ------------------------------------------------------------------ set-up
@pytest.mark.parametrize("case", CASES)
def test_device_ilu_factors_bit_exact(sg, oracle, golden, case):
    A = golden_matrix(golden, case)
    pc = sg.ILU0Precond()
    pc.setup(to_sg(sg, A))
    f = pc.factors(0)
    assert np.array_equal(f["diag_ptr"], golden[f"{case}/ilu0_diag"])
    assert np.array_equal(f["lu_vals"], golden[f"{case}/ilu0_lu"])
    # every subdomain of a RAS set-up against the oracle's local factorisation
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pr = sg.RASPrecond(nparts, 2, part)
    pr.setup(to_sg(sg, A))
    po = oracle.precond("ras", A, nparts, 2, part)
    for s in range(nparts):
        rp, ci, lu, dg = po.sub_factor(s)
        g = pr.factors(s)
        assert np.array_equal(g["row_ptr"], rp) and np.array_equal(g["col_idx"], ci)
        assert np.array_equal(g["diag_ptr"], dg)
        assert np.array_equal(g["lu_vals"], lu)


@pytest.mark.parametrize("case", CASES)
def test_device_decomposition_and_coarse(sg, golden, case):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pc = sg.TwoLevelSchwarzPrecond(nparts, 1, sg.FineLevelType.RAS, part)
    pc.setup(to_sg(sg, A))
    d = pc.decomposition()
    for k in ("owned_ptr", "owned", "sub_ptr", "sub", "ownloc_ptr", "ownloc"):
        assert np.array_equal(d[k], golden[f"{case}/dd1/{k}"]), k
    assert np.array_equal(pc.coarse_a0(), golden[f"{case}/a0"])


# ------------------------------------------------------------------ applies
@pytest.mark.parametrize("case", CASES)
@pytest.mark.parametrize("kind", KINDS)
def test_apply_fp64_vs_reference(sg, golden, case, kind):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pc = make_pc(sg, kind, nparts, 1, part)
    pc.setup(to_sg(sg, A))
    y = pc.apply(golden[f"{case}/x"])
    ref = golden[f"{case}/apply/{kind}"]
    if kind in ("jacobi", "ilu0", "ras"):
        assert np.array_equal(y, ref)
    elif kind == "asm":
        assert rel(y, ref) <= 1e-14
    else:
        assert rel(y, ref) <= 1e-12


@pytest.mark.parametrize("kind", ["ilu0", "ras", "asm", "twolevel_ras"])
@pytest.mark.parametrize("dt", ["fp32", "bf16"])
def test_apply_low_precision(sg, oracle, kind, dt):
    A = sg.make_varcoef_3d(24, 20, 16, 1.0, 6.0, 2)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    part = sg.partition_graph(A, 8)
    x = sg.uniform(A.nrows, seed=4)
    fdt = sg.FP32 if dt == "fp32" else sg.BF16
    pc = make_pc(sg, kind, 8, 1, part, fdt, sg.FP32)
    pc.setup(A)
    y = pc.apply(x)
    ref = oracle.precond(kind, H, 8, 1, part).apply(x)
    assert rel(y, ref) <= (1e-5 if dt == "fp32" else 2e-2)


@pytest.mark.parametrize("kind", ["ilu0", "asm", "ras", "twolevel_ras"])
@pytest.mark.parametrize("dt", ["fp64", "fp32", "bf16"])
def test_sweep_variants_agree(sg, kind, dt):
    """The sync-free sweep, the level sweep (a barrier per level) and the
    TMA-fed level sweep -- at every block size the set-up autotuner may
    pick -- compute the same thing: bit-exact
    (same operations in the same order per row, coarse term summed in a
    block-size independent order), up to the atomic order of the ASM sums."""
    A = sg.make_varcoef_3d(20, 22, 18, 1.0, 5.0, 4)
    part = sg.partition_boxes(20, 22, 18, 12, 0.1, 2)
    x = sg.uniform(A.nrows, seed=9)
    fdt = {"fp64": sg.FP64, "fp32": sg.FP32, "bf16": sg.BF16}[dt]
    sdt = sg.FP64 if dt == "fp64" else sg.FP32
    ys = []
    for sweep, threads in (("tma", 0), ("tma", 512), ("tma", 256), ("tma", 128), ("tma", 64),
                           ("tma", 32), ("level", 0), ("syncfree", 0)):
        pc = make_pc(sg, kind, 12, 1, part, fdt, sdt, sweep=sweep, sweep_threads=threads)
        pc.setup(A)
        ch = pc.sweep_choice()
        assert ch["sweep"] == sweep
        if sweep == "tma" and threads:
            assert ch["threads"] == threads
        elif sweep == "tma":
            assert ch["threads"] in (128, 256, 384, 512)
        ys.append(pc.apply(x))
    for y in ys[1:]:
        if kind == "asm":
            assert rel(y, ys[0]) <= 1e-6
        else:
            assert np.array_equal(y, ys[0])


def test_apply_large_subdomains_and_many_parts(sg, oracle):
    """Uneven box partition, 64 parts, overlap 2 (the cfg2 shape at 32^3)."""
    A = sg.make_poisson_3d(32, 32, 32)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    part = sg.partition_boxes(32, 32, 32, 64, 0.08, 3)
    x = sg.uniform(A.nrows, seed=7)
    for kind in ("ras", "twolevel_ras"):
        pc = make_pc(sg, kind, 64, 2, part)
        pc.setup(A)
        ref = oracle.precond(kind, H, 64, 2, part).apply(x)
        y = pc.apply(x)
        if kind == "ras":
            assert np.array_equal(y, ref)
        else:
            assert rel(y, ref) <= 1e-12


def test_apply_device_pointers(sg):
    torch = pytest.importorskip("torch")
    A = sg.make_poisson_2d(40, 40)
    pc = sg.RASPrecond(4, 1)
    pc.setup(A)
    x = sg.uniform(A.nrows, seed=3)
    yd = torch.empty(A.nrows, dtype=torch.float64, device="cuda")
    pc.apply(torch.from_numpy(x).cuda(), yd)
    torch.cuda.synchronize()
    assert np.array_equal(yd.cpu().numpy(), pc.apply(x))


# ------------------------------------------------------------------ solves
@pytest.mark.parametrize("case", ["p2d_blocks", "p3d_slabs"])
@pytest.mark.parametrize("kind", KINDS)
@pytest.mark.parametrize("solver", ["gmres", "fgmres"])
@pytest.mark.parametrize("graph", [True, False])
def test_solve_reference_rule_vs_golden(sg, golden, case, kind, solver, graph):
    A = golden_matrix(golden, case)
    part = golden[f"{case}/part"]
    nparts = int(golden[f"{case}/nparts"])
    pc = make_pc(sg, kind, nparts, 1, part)
    As = to_sg(sg, A)
    pc.setup(As)
    b = golden[f"{case}/b"]
    x = np.zeros(A.nrows)
    fn = sg.gmres if solver == "gmres" else sg.fgmres
    p = sg.GMRESParams(restart=30, max_iter=500, tol=1e-10, use_graph=graph)
    r = fn(As, b, x, pc, p)
    key = f"{case}/{solver}/{kind}"
    assert r.converged == bool(golden[key + "/converged"])
    assert abs(r.iterations - int(golden[key + "/iterations"])) <= 3
    assert rel(x, golden[key + "/x"]) <= 1e-7
    assert len(r.residual_history) == r.iterations


def test_identity_kat(sg):
    """tests/test_gmres.cpp:27-44 on the GPU"""
    A = sg.make_identity(10)
    b = np.arange(1, 11, dtype=np.float64)
    x = np.zeros(10)
    r = sg.gmres(A, b, x, None, sg.GMRESParams(restart=10, tol=1e-12))
    assert r.converged and r.iterations <= 2
    assert np.abs(x - b).sum() < 1e-10


@pytest.mark.parametrize("kind", [None, "jacobi", "ilu0"])
def test_small_spd_kat(sg, kind):
    """tests/test_gmres.cpp:46-92 on the GPU"""
    A = sg.CSRMatrix(3, 3, [0, 2, 5, 7], [0, 1, 0, 1, 2, 1, 2], [4.0, 1, 1, 3, 1, 1, 2])
    xe = np.array([1.0, 2.0, 3.0])
    b = A.spmv(xe)
    pc = None if kind is None else make_pc(sg, kind, 1, 0, None)
    if pc is not None:
        pc.setup(A)
    x = np.zeros(3)
    r = sg.gmres(A, b, x, pc)
    assert r.converged and np.abs(x - xe).sum() < 1e-8


def test_poisson5_kat(sg):
    """tests/test_gmres.cpp:94-142 on the GPU"""
    A = sg.make_poisson_2d(5, 5)
    b = A.spmv(np.ones(25))
    pc = sg.ILU0Precond()
    pc.setup(A)
    x = np.zeros(25)
    r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=25, tol=1e-10))
    assert r.converged and r.residual_norm < 1e-10 and np.abs(x - 1).sum() < 1e-6


def _oracle_true_rel(oracle, H, b, pc, m, rtol, fgmres=False, max_cycles=400):
    """The oracle harness: the reference GMRES one cycle at a time (tol 0,
    max_iter = m, warm start) until ||b-Ax||/||b|| <= rtol in FP64."""
    x = np.zeros(H.nrows)
    bn = np.linalg.norm(b)
    its = 0
    fn = oracle.fgmres if fgmres else oracle.gmres
    for _ in range(max_cycles):
        r = fn(H, b, x, pc, restart=m, max_iter=m, tol=0.0)
        x = r["x"]
        its += r["iterations"]
        if np.linalg.norm(b - oracle.spmv(H, x)) / bn <= rtol:
            return x, its
    return x, its


def test_cfg1_poisson2d_ilu0_true_residual(sg, oracle):
    """128x128 5-point Poisson, x* ~ U[-1,1] seed 0, GMRES(30)+ILU(0), FP64
    true relative residual 1e-8."""
    A = sg.make_poisson_2d(128, 128)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    xs = sg.uniform(A.nrows, seed=0)
    b = A.spmv(xs)
    pc = sg.ILU0Precond()
    pc.setup(A)
    for kind in (sg.TOL_TRUE_REL_CYCLE, sg.TOL_TRUE_REL):
        x = np.zeros(A.nrows)
        r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=5000, tol=1e-8,
                                                  tol_kind=kind))
        assert r.converged and r.true_rel_residual <= 1e-8
        assert np.linalg.norm(b - A.spmv(x)) / np.linalg.norm(b) <= 1e-8
        xo, its = _oracle_true_rel(oracle, H, b, oracle.precond("ilu0", H), 30, 1e-8)
        if kind == sg.TOL_TRUE_REL_CYCLE:
            assert abs(r.iterations - its) <= 30
        # both solutions sit within the 1e-8 residual ball around x*
        assert rel(x, xo) <= 1e-5


@pytest.mark.parametrize("precision", ["fp64", "mixed", "mixed_bf16"])
def test_cfg2_shape_ras_true_residual(sg, oracle, precision):
    """7-point Poisson, RAS with graph-partitioned parts and overlap 2, GMRES(30)
    at FP64 true relative residual 1e-8 (40^3 here; full size in the config
    tests)."""
    A = sg.make_poisson_3d(40, 40, 40)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    xs = sg.uniform(A.nrows, seed=1)
    b = A.spmv(xs)
    part = sg.partition_graph(A, 16)
    if precision == "fp64":
        pc = sg.RASPrecond(16, 2, part)
        prec = sg.FP64
    else:
        pc = sg.RASPrecond(16, 2, part, sg.BF16 if precision == "mixed_bf16" else sg.FP32, sg.FP32)
        prec = sg.FP32
    pc.setup(A)
    x = np.zeros(A.nrows)
    r = sg.gmres(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=3000, tol=1e-8,
                                              tol_kind=sg.TOL_TRUE_REL, precision=prec))
    assert r.converged and r.true_rel_residual <= 1e-8
    assert np.linalg.norm(b - A.spmv(x)) / np.linalg.norm(b) <= 1e-8
    xo, _ = _oracle_true_rel(oracle, H, b, oracle.precond("ras", H, 16, 2, part), 30, 1e-8)
    assert rel(x, xo) <= 1e-5


@pytest.mark.parametrize("solver", ["gmres", "fgmres"])
def test_two_level_varcoef_true_residual(sg, oracle, solver):
    A = sg.make_varcoef_3d(32, 32, 32, 1.0, 8.0, 3)
    H = HostCSR(A.row_ptr, A.col_idx, A.vals)
    xs = sg.uniform(A.nrows, seed=2)
    b = A.spmv(xs)
    part = sg.partition_boxes(32, 32, 32, 32, 0.08, 5)
    for prec in (sg.FP64, sg.FP32):
        if prec == sg.FP64:
            pc = sg.TwoLevelSchwarzPrecond(32, 1, sg.FineLevelType.RAS, part)
        else:
            pc = sg.TwoLevelSchwarzPrecond(32, 1, sg.FineLevelType.RAS, part, sg.FP32, sg.FP32)
        pc.setup(A)
        x = np.zeros(A.nrows)
        fn = sg.gmres if solver == "gmres" else sg.fgmres
        r = fn(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=3000, tol=1e-8,
                                            tol_kind=sg.TOL_TRUE_REL, precision=prec))
        assert r.converged and r.true_rel_residual <= 1e-8
        xo, _ = _oracle_true_rel(oracle, H, b, oracle.precond("twolevel_ras", H, 32, 1, part),
                                 30, 1e-8, fgmres=solver == "fgmres")
        assert rel(x, xo) <= 1e-5


@pytest.mark.parametrize("solver", ["gmres", "fgmres"])
def test_mixed_keeps_fp64_iteration_count(sg, solver):
    """The FP32 inner Krylov cycle (CGS2 in FP32) keeps the basis orthogonal:
    on a 48^3 two-level problem it needs about the FP64 solver's iterations;
    a loss of orthogonality shows up as many extra iterations."""
    A = sg.make_varcoef_3d(48, 48, 48, 1.0, 8.0, 1)
    b = A.spmv(sg.uniform(A.nrows, seed=3))
    part = sg.partition_boxes(48, 48, 48, 27, 0.08, 2)
    its = {}
    for prec in (sg.FP64, sg.FP32):
        sd = sg.FP64 if prec == sg.FP64 else sg.FP32
        pc = sg.TwoLevelSchwarzPrecond(27, 1, sg.FineLevelType.RAS, part, sd, sd)
        pc.setup(A)
        x = np.zeros(A.nrows)
        fn = sg.gmres if solver == "gmres" else sg.fgmres
        r = fn(A, b, x, pc, sg.GMRESParams(restart=30, max_iter=3000, tol=1e-8,
                                            tol_kind=sg.TOL_TRUE_REL, precision=prec))
        assert r.converged and r.true_rel_residual <= 1e-8
        its[prec] = r.iterations
    assert its[sg.FP32] <= 1.15 * its[sg.FP64] + 5, its


def test_solve_device_pointers(sg):
    torch = pytest.importorskip("torch")
    A = sg.make_poisson_3d(24, 24, 24)
    b = A.spmv(sg.uniform(A.nrows, seed=5))
    pc = sg.RASPrecond(8, 1)
    pc.setup(A)
    xh = np.zeros(A.nrows)
    p = sg.GMRESParams(restart=30, max_iter=2000, tol=1e-8, tol_kind=sg.TOL_TRUE_REL)
    rh = sg.gmres(A, b, xh, pc, p)
    xd = torch.zeros(A.nrows, dtype=torch.float64, device="cuda")
    rd = sg.gmres(A, torch.from_numpy(b).cuda(), xd, pc, p)
    torch.cuda.synchronize()
    assert rh.iterations == rd.iterations
    assert np.array_equal(xd.cpu().numpy(), xh)


# ------------------------------------------------------------------ failure paths
def test_nonfinite_rhs_is_reported(sg):
    A = sg.make_poisson_2d(10, 10)
    b = np.ones(100)
    b[17] = np.nan
    with pytest.raises(sg.SgError) as e:
        sg.gmres(A, b, np.zeros(100), None, sg.GMRESParams(tol_kind=sg.TOL_TRUE_REL, tol=1e-8))
    assert e.value.status == 6


def test_singular_coarse_is_reported(sg):
    """Two parts with no coupling and zero blocks: A0 is singular
    (src/precond/coarse_solve.h:31-32 throws)."""
    n = 4
    A = sg.CSRMatrix(n, n, [0, 1, 2, 3, 4], [0, 1, 2, 3], [1.0, 1.0, 0.0, 0.0])
    pc = sg.TwoLevelSchwarzPrecond(2, 0, sg.FineLevelType.RAS, np.array([0, 0, 1, 1], np.int32))
    with pytest.raises(sg.SgError) as e:
        pc.setup(A)
    assert e.value.status == 4


def test_use_before_setup_and_bad_csr(sg):
    pc = sg.RASPrecond(2, 1)
    with pytest.raises(sg.SgError) as e:
        pc.apply(np.ones(4))
    assert e.value.status == 5
    bad = sg.CSRMatrix(2, 2, [0, 1, 3], [0, 5, 1], [1.0, 1.0, 1.0])
    with pytest.raises(sg.SgError) as e:
        bad.upload()
    assert e.value.status == 1


@pytest.mark.parametrize("kind", [sg_kind for sg_kind in ("twolevel_ras", "twolevel_asm")])
@pytest.mark.parametrize("dt", ["fp64", "bf16"])
def test_fused_restriction_same_bits(sg, kind, dt):
    """The coarse restriction computed inside the TMA-fed sweep (cooperative
    launch) and in a kernel of its own sum in the same order: the apply and a
    whole solve give the same bits either way."""
    A = sg.make_varcoef_3d(24, 20, 22, 1.0, 5.0, 6)
    part = sg.partition_boxes(24, 20, 22, 12, 0.1, 2)
    x = sg.uniform(A.nrows, seed=10)
    b = A.spmv(x)
    fdt = sg.FP64 if dt == "fp64" else sg.BF16
    sdt = sg.FP64 if dt == "fp64" else sg.FP32
    ft = sg.FineLevelType.RAS if kind == "twolevel_ras" else sg.FineLevelType.ASM
    ys, xs = [], []
    for fuse in (True, False):
        pc = sg.TwoLevelSchwarzPrecond(12, 1, ft, part, fdt, sdt, fuse_restrict=fuse)
        pc.setup(A)
        ys.append(pc.apply(x))
        if kind == "twolevel_ras":
            xx = np.zeros(A.nrows)
            r = sg.gmres(A, b, xx, pc, sg.GMRESParams(
                restart=30, max_iter=2000, tol=1e-9, tol_kind=sg.TOL_TRUE_REL,
                precision=sg.FP32 if dt == "bf16" else sg.FP64))
            assert r.converged
            xs.append(xx)
    if kind == "twolevel_ras":
        assert np.array_equal(ys[0], ys[1])
        assert np.array_equal(xs[0], xs[1])
    else:
        # ASM adds overlapping rows atomically: order of the adds may differ
        assert rel(ys[0], ys[1]) <= 1e-12 if dt == "fp64" else rel(ys[0], ys[1]) <= 1e-6
