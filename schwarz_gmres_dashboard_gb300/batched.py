"""Batched solves: many independent systems (uneven sizes, several right-hand
sides each) in one call of libsgmres's batched GMRES (sg_solve_batched).

    prob = make_aniso_batch(512, seed=0)       # 2D anisotropic 9-point systems
    M = RASPrecond(prob.nparts, 1, partition=prob.partition,
                   factor_dtype=FP32, sweep_dtype=FP32)
    M.setup(prob.A)                            # one set-up for every subdomain
    B = uniform(4 * prob.n, seed=1).reshape(4, prob.n)
    X = np.zeros_like(B)
    res, t = solve_batched(prob.A, M, prob.sys_row_ptr, 4, B, X,
                           GMRESParams(restart=30, tol=1e-8, tol_kind=TOL_TRUE_REL,
                                       precision=FP32))

The systems are stacked as one block-diagonal matrix; every (system, rhs)
pair is an independent GMRES with its own Krylov space and stopping test.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional

import numpy as np

from . import _lib as L
from . import (CSRMatrix, FP32, GMRESParams, Preconditioner, TOL_TRUE_REL, _vec,
               default_context, make_aniso_2d, partition_boxes, uniform)

_clib = L.load()


@dataclass
class BatchProblem:
    A: CSRMatrix                 # block-diagonal union of the systems
    sys_row_ptr: np.ndarray      # [nsys + 1] row offsets
    sizes: np.ndarray            # grid edge n of every system (n x n)
    eps: np.ndarray
    theta: np.ndarray
    parts: np.ndarray            # subdomains of every system
    partition: np.ndarray        # global partition (parts never cross systems)

    @property
    def n(self) -> int:
        return self.A.nrows

    @property
    def nsys(self) -> int:
        return len(self.sizes)

    @property
    def nparts(self) -> int:
        return int(self.parts.sum())


def make_aniso_batch(nsys: int, seed: int = 0, nmin: int = 32, nmax: int = 256,
                     eps_range=(1e-3, 1.0), rows_per_part: int = 4096, min_parts: int = 4,
                     max_parts: int = 16, spread: float = 0.08) -> BatchProblem:
    """nsys systems -div(K grad u) on n x n grids, n ~ U{nmin..nmax},
    eps ~ LogUniform(eps_range), theta ~ U[0, pi), all from SplitMix64(seed);
    each split into clamp(round(n^2 / rows_per_part), min_parts, max_parts)
    seeded boxes."""
    u = uniform(3 * nsys, seed, 0.0, 1.0).reshape(nsys, 3)
    sizes = nmin + np.minimum((u[:, 0] * (nmax - nmin + 1)).astype(np.int64), nmax - nmin)
    lo, hi = np.log10(eps_range[0]), np.log10(eps_range[1])
    eps = 10.0 ** (lo + (hi - lo) * u[:, 1])
    theta = np.pi * u[:, 2]
    parts = np.clip(np.rint(sizes.astype(float) ** 2 / rows_per_part), min_parts,
                    max_parts).astype(np.int64)
    rps, cis, vals, pts = [], [], [], []
    row_ptr = [0]
    nnz_off = 0
    part_off = 0
    for s in range(nsys):
        n = int(sizes[s])
        As = make_aniso_2d(n, n, float(eps[s]), float(theta[s]))
        rps.append(As.row_ptr[:-1] + nnz_off)
        cis.append(As.col_idx + row_ptr[-1])
        vals.append(As.vals)
        nnz_off += As.nnz()
        p = partition_boxes(n, n, 1, int(parts[s]), spread, seed * 1000003 + s)
        pts.append(p + part_off)
        part_off += int(parts[s])
        row_ptr.append(row_ptr[-1] + n * n)
    rp = np.concatenate(rps + [np.array([nnz_off])]).astype(np.int32)
    A = CSRMatrix(row_ptr[-1], row_ptr[-1], rp, np.concatenate(cis).astype(np.int32),
                  np.concatenate(vals))
    return BatchProblem(A=A, sys_row_ptr=np.asarray(row_ptr, np.int32), sizes=sizes, eps=eps,
                        theta=theta, parts=parts,
                        partition=np.concatenate(pts).astype(np.int32))


def solve_batched(A: CSRMatrix, M: Optional[Preconditioner], sys_row_ptr, nrhs: int, B, X,
                  params: Optional[GMRESParams] = None):
    """Solve every (system, rhs) pair; B and X are [nrhs, n] (numpy or CUDA
    arrays), X holds x0 on entry and the solutions on exit.  Returns
    (results, seconds): results a structured array with iterations, cycles,
    converged, status and true_rel_residual per pair i = rhs * nsys + s."""
    params = params or GMRESParams(restart=30, tol=1e-8, tol_kind=TOL_TRUE_REL, precision=FP32)
    ctx = M.ctx if M is not None else default_context()
    dev = A.device(ctx)
    srp = np.ascontiguousarray(sys_row_ptr, dtype=np.int32)
    nsys = len(srp) - 1
    n = A.nrows
    pb, mb, _kb = _vec(B, n * nrhs)
    px, mx, _kx = _vec(X, n * nrhs, writable=True)
    if mb != mx:
        raise TypeError("B and X must both be host or both be device arrays")
    p = L.SolveParams()
    p.restart = params.restart
    p.max_iter = params.max_iter
    p.tol = params.tol
    p.tol_kind = params.tol_kind
    p.precision = params.precision
    p.use_graph = 1 if params.use_graph else 0
    res = (L.BatchResult * (nsys * nrhs))()
    t = C.c_double(0.0)
    L.check(_clib.sg_solve_batched(ctx.handle, dev, M.handle if M is not None else None, nsys,
                                   srp.ctypes.data, nrhs, pb, px, mx, C.byref(p), res,
                                   C.byref(t)))
    out = np.zeros(nsys * nrhs, dtype=[("iterations", np.int32), ("cycles", np.int32),
                                       ("converged", np.int32), ("status", np.int32),
                                       ("true_rel_residual", np.float64)])
    for i in range(nsys * nrhs):
        out[i] = (res[i].iterations, res[i].cycles, res[i].converged, res[i].status,
                  res[i].true_rel_residual)
    return out, t.value
