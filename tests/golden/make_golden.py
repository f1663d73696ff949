"""Generate tests/golden/golden.npz from the reference's own sources.

Run here, where the reference tree is present:

    make -C oracle ref && python tests/golden/make_golden.py

It drives oracle/_ref/libref.so (the reference's src/core/gmres.cpp,
src/core/fgmres.cpp and headers, compiled unmodified with the metis.h seam)
on small inputs and stores inputs and outputs.  The GPU parity tests and the
oracle pin tests read the fixture; nothing reads the reference at test time.
"""
from __future__ import annotations

import os
import sys

import numpy as np

# one OpenMP thread: the reference's ASM adds overlap entries under
# `omp critical` in arrival order, so more threads give run-to-run rounding
# differences in those fixtures
os.environ["OMP_NUM_THREADS"] = "1"

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle.oracle import Reference  # noqa: E402

KINDS = ["jacobi", "ilu0", "asm", "ras", "twolevel_asm", "twolevel_ras"]


class CSR:
    def __init__(self, rp, ci, v):
        self.row_ptr, self.col_idx, self.vals = rp, ci, v
        self.nrows = self.ncols = len(rp) - 1


def vec(n, seed):
    """Deterministic test vector independent of any RNG library."""
    i = np.arange(n, dtype=np.float64)
    return np.sin(0.7 * i + seed) + 0.25 * np.cos(1.3 * i * (seed + 1))


def add_case(out, R, name, A, part, nparts, overlaps=(0, 1, 2), solve=True):
    n = A.nrows
    out[f"{name}/row_ptr"] = A.row_ptr
    out[f"{name}/col_idx"] = A.col_idx
    out[f"{name}/vals"] = A.vals
    out[f"{name}/part"] = part
    out[f"{name}/nparts"] = np.array(nparts)
    x = vec(n, 1)
    out[f"{name}/x"] = x
    out[f"{name}/spmv"] = R.spmv(A, x)
    lu, dg = R.ilu0_factor(A)
    out[f"{name}/ilu0_lu"] = lu
    out[f"{name}/ilu0_diag"] = dg
    for ov in overlaps:
        d = R.decompose(A, part, nparts, ov)
        for k, v in d.items():
            out[f"{name}/dd{ov}/{k}"] = v
    out[f"{name}/a0"] = R.coarse_a0(A, part, nparts, 1)
    b = vec(n, 2)
    out[f"{name}/b"] = b
    for kind in KINDS:
        pc = R.precond(kind, A, nparts, 1, part)
        out[f"{name}/apply/{kind}"] = pc.apply(x)
        if not solve:
            continue
        for solver in ("gmres", "fgmres"):
            fn = R.gmres if solver == "gmres" else R.fgmres
            r = fn(A, b, np.zeros(n), pc, restart=30, max_iter=500, tol=1e-10, hist_cap=600)
            key = f"{name}/{solver}/{kind}"
            out[key + "/x"] = r["x"]
            out[key + "/iterations"] = np.array(r["iterations"])
            out[key + "/converged"] = np.array(r["converged"])
            out[key + "/residual_norm"] = np.array(r["residual_norm"])
            out[key + "/history"] = r["history"]


MTX = {
    # general real matrix, entries out of order, a comment between header lines
    # (no comment between entries: the reference reader parses such a line as
    # an entry with undefined indices)
    "general": ("%%MatrixMarket matrix coordinate real general\n% made for the reader test\n"
                "4 5 7\n3 2 -1.5\n1 1 4\n"
                "4 5 2.25e-1\n1 3 -2\n2 2 5\n4 1 1e3\n3 3 6\n"),
    # symmetric: lower triangle stored, off-diagonal entries mirrored
    "symmetric": ("%%MatrixMarket matrix coordinate real symmetric\n5 5 8\n1 1 4\n2 1 -1\n"
                  "2 2 4\n3 2 -1\n3 3 4\n4 3 -1\n5 4 -1\n5 5 4\n"),
    # pattern + symmetric: no values (read as 1.0)
    "pattern": ("%%MatrixMarket matrix coordinate pattern symmetric\n4 4 5\n1 1\n2 1\n"
                "3 3\n4 2\n4 4\n"),
    # duplicates are kept, not summed (the reference reader does not dedupe)
    "duplicates": ("%%MatrixMarket matrix coordinate real general\n3 3 6\n1 1 1\n"
                   "2 3 2\n1 1 3\n3 1 4\n2 3 5\n3 3 6\n"),
}


def add_io_cases(out, R):
    """Matrix Market files read by the reference reader, and convergence
    metrics / .conv.jsonl records of the reference's analysis code."""
    import tempfile
    d = os.path.join(HERE, "mtx")
    os.makedirs(d, exist_ok=True)
    for name, text in MTX.items():
        path = os.path.join(d, f"{name}.mtx")
        with open(path, "w") as f:
            f.write(text)
        nr, nc, rp, ci, v = R.read_mm(path)
        out[f"mm/{name}/shape"] = np.array([nr, nc])
        out[f"mm/{name}/row_ptr"], out[f"mm/{name}/col_idx"], out[f"mm/{name}/vals"] = rp, ci, v
    hists = {
        "gmres": out["p2d_blocks/gmres/ilu0/history"],
        "stagnating": np.concatenate([np.geomspace(1.0, 1e-3, 15), np.full(30, 1e-3) *
                                      (1 - 1e-5 * np.arange(30))]),
        "single": np.array([0.5]),
        "empty": np.zeros(0),
    }
    for name, h in hists.items():
        conv = name == "gmres"
        m = R.conv_metrics(h, conv)
        out[f"conv/{name}/history"] = h
        out[f"conv/{name}/converged"] = np.array(conv)
        out[f"conv/{name}/metrics"] = np.array([m["initial_residual"], m["final_residual"],
                                                m["asymptotic_rate"]])
        out[f"conv/{name}/imetrics"] = np.array([m["iterations"], m["stagnation_start"]])
        out[f"conv/{name}/rates"] = m["rates"]
        with tempfile.TemporaryDirectory() as t:
            path = os.path.join(t, "o.conv.jsonl")
            R.conv_write(path, "poisson_12", "ilu0", 4, 1, h, conv)
            out[f"conv/{name}/jsonl"] = np.frombuffer(open(path, "rb").read(), np.uint8)


def add_solver_cases(out, R, name, A, part, nparts, kinds):
    """BiCGSTAB and the Lanczos / power-iteration estimates of the reference
    on the same inputs as the GMRES cases."""
    n = A.nrows
    b = out[f"{name}/b"]
    for kind in kinds:
        pc = R.precond(kind, A, nparts, 1, part)
        r = R.bicgstab(A, b, np.zeros(n), pc, max_iter=500, tol=1e-10, hist_cap=600)
        key = f"{name}/bicgstab/{kind}"
        out[key + "/x"] = r["x"]
        out[key + "/iterations"] = np.array(r["iterations"])
        out[key + "/converged"] = np.array(r["converged"])
        out[key + "/residual_norm"] = np.array(r["residual_norm"])
        out[key + "/history"] = r["history"]
        c = R.condition(A, pc, 80, 42)
        out[f"{name}/condition/{kind}"] = np.array([c["lambda_min"], c["lambda_max"],
                                                    c["kappa"], c["lanczos_steps"], c["valid"]])
        sp = R.spectral(A, pc, 200, 1e-6, 123)
        out[f"{name}/spectral/{kind}"] = np.array([sp["spectral_radius"], sp["power_iters"],
                                                   sp["convergence_ok"]])


def main():
    R = Reference()
    out = {}
    # 2D Poisson 12x12, contiguous blocks and a scattered partition
    rp, ci, v = R.poisson2d(12, 12)
    A = CSR(rp, ci, v)
    n = A.nrows
    add_case(out, R, "p2d_blocks", A, (np.arange(n) * 4 // n).astype(np.int32), 4)
    add_case(out, R, "p2d_scatter", A, ((np.arange(n) * 7919) % 5).astype(np.int32), 5,
             solve=False)
    # 3D Poisson 6x7x5 in 6 slabs
    rp, ci, v = R.poisson3d(6, 7, 5)
    A = CSR(rp, ci, v)
    n = A.nrows
    add_case(out, R, "p3d_slabs", A, (np.arange(n) * 6 // n).astype(np.int32), 6)
    # BiCGSTAB and the analysis tools (none = the unpreconditioned operator)
    solver_kinds = ["none", "jacobi", "ilu0", "ras", "twolevel_ras"]
    rp, ci, v = R.poisson2d(12, 12)
    A = CSR(rp, ci, v)
    add_solver_cases(out, R, "p2d_blocks", A, (np.arange(A.nrows) * 4 // A.nrows)
                     .astype(np.int32), 4, solver_kinds)
    rp, ci, v = R.poisson3d(6, 7, 5)
    A = CSR(rp, ci, v)
    add_solver_cases(out, R, "p3d_slabs", A, (np.arange(A.nrows) * 6 // A.nrows)
                     .astype(np.int32), 6, solver_kinds)
    add_io_cases(out, R)
    # the reference's own known-answer cases (tests/test_gmres.cpp:27-142)
    out["kat/p2d5/row_ptr"], out["kat/p2d5/col_idx"], out["kat/p2d5/vals"] = R.poisson2d(5, 5)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
