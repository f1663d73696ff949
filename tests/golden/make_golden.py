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
    # the reference's own known-answer cases (tests/test_gmres.cpp:27-142)
    out["kat/p2d5/row_ptr"], out["kat/p2d5/col_idx"], out["kat/p2d5/vals"] = R.poisson2d(5, 5)
    np.savez_compressed(os.path.join(HERE, "golden.npz"), **out)
    print(f"wrote {len(out)} arrays")


if __name__ == "__main__":
    main()
