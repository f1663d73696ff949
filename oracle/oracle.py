"""ctypes wrapper over the oracle libraries -- TEST INFRASTRUCTURE ONLY.

`Oracle` wraps ``oracle/_build/liboracle.so`` (the CPU restatement in
``oracle.c``); `Reference` wraps ``oracle/_ref/libref.so`` (the reference's own
sources compiled by ``make ref`` where the reference tree is present).  Only
the tests, ``__graft_entry__.smoke()`` and the cpu_baseline leg of ``bench.py``
import this module; it is the checker, never the thing measured or shipped.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_SO = os.path.join(HERE, "_build", "liboracle.so")
REF_SO = os.path.join(HERE, "_ref", "libref.so")

PC_KINDS = {"none": 0, "jacobi": 1, "ilu0": 2, "asm": 3, "ras": 4,
            "twolevel_asm": 5, "twolevel_ras": 6}

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")


def build(ref: bool = False) -> None:
    """Compile the oracle (and, when asked and the reference tree exists, the
    reference shim) with the committed Makefile."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref"], check=True)


def _csr_args(A):
    rp = np.ascontiguousarray(A.row_ptr, dtype=np.int32)
    ci = np.ascontiguousarray(A.col_idx, dtype=np.int32)
    v = np.ascontiguousarray(A.vals, dtype=np.float64)
    return rp, ci, v


class _Lib:
    def __init__(self, path):
        if not os.path.exists(path):
            raise FileNotFoundError(path)
        self.lib = C.CDLL(path)


class Oracle(_Lib):
    """CPU restatement of the reference (oracle.c)."""

    def __init__(self, path: str = ORACLE_SO):
        if not os.path.exists(path):
            build()
        super().__init__(path)
        L = self.lib
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_get_threads.restype = C.c_int
        L.orc_spmv.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.orc_ilu0_factor.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _i32p]
        L.orc_ilu0_solve.argtypes = [C.c_int, _i32p, _i32p, _f64p, _i32p, _f64p, _f64p]
        L.orc_levels_lower.argtypes = [C.c_int, _i32p, _i32p, _i32p]
        L.orc_levels_lower.restype = C.c_int
        L.orc_levels_upper.argtypes = [C.c_int, _i32p, _i32p, _i32p, _i32p]
        L.orc_levels_upper.restype = C.c_int
        pp = C.POINTER(C.POINTER(C.c_int))
        L.orc_decompose.argtypes = [C.c_int, _i32p, _i32p, _i32p, C.c_int, C.c_int,
                                    pp, pp, pp, pp, pp, pp]
        L.orc_decompose.restype = C.c_int
        L.orc_free.argtypes = [C.c_void_p]
        L.orc_pc_create.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_int,
                                    C.c_int, C.c_void_p, C.POINTER(C.c_int)]
        L.orc_pc_create.restype = C.c_void_p
        L.orc_pc_apply.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int]
        L.orc_pc_destroy.argtypes = [C.c_void_p]
        L.orc_pc_coarse.argtypes = [C.c_void_p, C.c_void_p]
        L.orc_pc_coarse.restype = C.c_int
        L.orc_pc_sub_factor.argtypes = [C.c_void_p, C.c_int, C.POINTER(C.c_int),
                                        C.POINTER(C.POINTER(C.c_int)),
                                        C.POINTER(C.POINTER(C.c_int)),
                                        C.POINTER(C.POINTER(C.c_double)),
                                        C.POINTER(C.POINTER(C.c_int))]
        L.orc_pc_sub_factor.restype = C.c_int
        for fn in (L.orc_gmres, L.orc_fgmres):
            fn.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_void_p,
                           C.c_int, C.c_int, C.c_double, C.POINTER(C.c_int),
                           C.POINTER(C.c_double), C.c_void_p, C.c_int, C.POINTER(C.c_int)]
            fn.restype = C.c_int
        L.orc_poisson2d.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_poisson2d.restype = C.c_int
        L.orc_poisson3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                    C.c_void_p]
        L.orc_poisson3d.restype = C.c_int
        L.orc_bicgstab.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p, C.c_void_p,
                                   C.c_int, C.c_double, C.POINTER(C.c_int),
                                   C.POINTER(C.c_double), C.c_void_p, C.c_int,
                                   C.POINTER(C.c_int)]
        L.orc_bicgstab.restype = C.c_int
        L.orc_condition.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, C.c_uint,
                                    _f64p, _i32p]
        L.orc_condition.restype = C.c_int
        L.orc_spectral.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_void_p, C.c_int, C.c_double,
                                   C.c_uint, _f64p, _i32p]
        L.orc_uniform.argtypes = [C.c_uint64, C.c_int, C.c_double, C.c_double, _f64p]
        L.orc_partition_boxes.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                          C.c_uint64, _i32p]
        L.orc_partition_boxes.restype = C.c_int
        L.orc_varcoef3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                    C.c_uint64, C.c_void_p, C.c_void_p, C.c_void_p]
        L.orc_varcoef3d.restype = C.c_int

    # -- threads
    def set_threads(self, n: int) -> None:
        self.lib.orc_set_threads(int(n))

    def threads(self) -> int:
        return int(self.lib.orc_get_threads())

    # -- kernels
    def spmv(self, A, x):
        rp, ci, v = _csr_args(A)
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(A.nrows, dtype=np.float64)
        self.lib.orc_spmv(A.nrows, rp, ci, v, x, y)
        return y

    def ilu0_factor(self, A):
        rp, ci, v = _csr_args(A)
        lu = np.empty_like(v)
        diag = np.empty(A.nrows, dtype=np.int32)
        self.lib.orc_ilu0_factor(A.nrows, rp, ci, v, lu, diag)
        return lu, diag

    def ilu0_solve(self, A, lu, diag, x):
        rp, ci, _ = _csr_args(A)
        y = np.empty(A.nrows, dtype=np.float64)
        self.lib.orc_ilu0_solve(A.nrows, rp, ci, np.ascontiguousarray(lu), diag,
                                np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def levels(self, A, diag):
        rp, ci, _ = _csr_args(A)
        lo = np.zeros(A.nrows, dtype=np.int32)
        up = np.zeros(A.nrows, dtype=np.int32)
        self.lib.orc_levels_lower(A.nrows, rp, ci, lo)
        self.lib.orc_levels_upper(A.nrows, rp, ci, np.ascontiguousarray(diag, dtype=np.int32), up)
        return lo, up

    def decompose(self, A, part, nparts, overlap):
        rp, ci, _ = _csr_args(A)
        part = np.ascontiguousarray(part, dtype=np.int32)
        ptrs = [C.POINTER(C.c_int)() for _ in range(6)]
        rc = self.lib.orc_decompose(A.nrows, rp, ci, part, nparts, overlap,
                                    *[C.byref(p) for p in ptrs])
        if rc:
            raise ValueError(f"orc_decompose failed ({rc})")
        owned_ptr = np.ctypeslib.as_array(ptrs[0], (nparts + 1,)).copy()
        owned = np.ctypeslib.as_array(ptrs[1], (max(int(owned_ptr[-1]), 1),))[: owned_ptr[-1]].copy()
        sub_ptr = np.ctypeslib.as_array(ptrs[2], (nparts + 1,)).copy()
        sub = np.ctypeslib.as_array(ptrs[3], (max(int(sub_ptr[-1]), 1),))[: sub_ptr[-1]].copy()
        ol_ptr = np.ctypeslib.as_array(ptrs[4], (nparts + 1,)).copy()
        ol = np.ctypeslib.as_array(ptrs[5], (max(int(ol_ptr[-1]), 1),))[: ol_ptr[-1]].copy()
        for p in ptrs:
            self.lib.orc_free(C.cast(p, C.c_void_p))
        return dict(owned_ptr=owned_ptr, owned=owned, sub_ptr=sub_ptr, sub=sub,
                    ownloc_ptr=ol_ptr, ownloc=ol)

    def precond(self, kind, A, nparts=4, overlap=1, part=None):
        return OraclePC(self, kind, A, nparts, overlap, part)

    def _solve(self, fn, A, b, x0, pc, restart, max_iter, tol, hist_cap=0):
        rp, ci, v = _csr_args(A)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        it = C.c_int(0)
        res = C.c_double(0.0)
        hl = C.c_int(0)
        hist = np.zeros(max(hist_cap, 1), dtype=np.float64)
        conv = fn(A.nrows, rp, ci, v, b, x, pc.handle if pc is not None else None,
                  restart, max_iter, tol, C.byref(it), C.byref(res),
                  hist.ctypes.data if hist_cap else None, hist_cap, C.byref(hl))
        return dict(x=x, converged=bool(conv), iterations=it.value, residual_norm=res.value,
                    history=hist[: min(hl.value, hist_cap)].copy())

    def gmres(self, A, b, x0, pc=None, restart=30, max_iter=1000, tol=1e-10, hist_cap=0):
        return self._solve(self.lib.orc_gmres, A, b, x0, pc, restart, max_iter, tol, hist_cap)

    def fgmres(self, A, b, x0, pc=None, restart=30, max_iter=1000, tol=1e-10, hist_cap=0):
        return self._solve(self.lib.orc_fgmres, A, b, x0, pc, restart, max_iter, tol, hist_cap)

    def bicgstab(self, A, b, x0, pc=None, max_iter=1000, tol=1e-10, hist_cap=0):
        rp, ci, v = _csr_args(A)
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        it, res, hl = C.c_int(0), C.c_double(0.0), C.c_int(0)
        hist = np.zeros(max(hist_cap, 1))
        conv = self.lib.orc_bicgstab(A.nrows, rp, ci, v, b, x,
                                     pc.handle if pc is not None else None, max_iter, tol,
                                     C.byref(it), C.byref(res),
                                     hist.ctypes.data if hist_cap else None, hist_cap,
                                     C.byref(hl))
        return dict(x=x, converged=bool(conv), iterations=it.value, residual_norm=res.value,
                    history=hist[: min(hl.value, hist_cap)].copy(), history_len=hl.value)

    def condition(self, A, pc=None, k=80, seed=42):
        rp, ci, v = _csr_args(A)
        out = np.zeros(3)
        iout = np.zeros(2, np.int32)
        self.lib.orc_condition(A.nrows, rp, ci, v, pc.handle if pc is not None else None, k,
                               seed, out, iout)
        return dict(lambda_min=out[0], lambda_max=out[1], kappa=out[2],
                    lanczos_steps=int(iout[0]), valid=bool(iout[1]))

    def spectral(self, A, pc=None, max_iter=200, tol=1e-6, seed=123):
        rp, ci, v = _csr_args(A)
        out = np.zeros(1)
        iout = np.zeros(2, np.int32)
        self.lib.orc_spectral(A.nrows, rp, ci, v, pc.handle if pc is not None else None,
                              max_iter, tol, seed, out, iout)
        return dict(spectral_radius=out[0], power_iters=int(iout[0]),
                    convergence_ok=bool(iout[1]))

    def poisson2d(self, nx, ny):
        nz = self.lib.orc_poisson2d(nx, ny, None, None, None)
        rp = np.empty(nx * ny + 1, np.int32)
        ci = np.empty(nz, np.int32)
        v = np.empty(nz, np.float64)
        self.lib.orc_poisson2d(nx, ny, rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
        return rp, ci, v

    def poisson3d(self, nx, ny, nz_):
        nz = self.lib.orc_poisson3d(nx, ny, nz_, None, None, None)
        rp = np.empty(nx * ny * nz_ + 1, np.int32)
        ci = np.empty(nz, np.int32)
        v = np.empty(nz, np.float64)
        self.lib.orc_poisson3d(nx, ny, nz_, rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
        return rp, ci, v


    # -- benchmark inputs (the project's generators, restated)
    def uniform(self, n, seed, lo=-1.0, hi=1.0):
        out = np.empty(n, np.float64)
        self.lib.orc_uniform(seed, n, lo, hi, out)
        return out

    def partition_boxes(self, nx, ny, nz, nparts, spread, seed):
        part = np.empty(nx * ny * nz, np.int32)
        rc = self.lib.orc_partition_boxes(nx, ny, nz, nparts, spread, seed, part)
        if rc:
            raise ValueError(f"orc_partition_boxes failed ({rc})")
        return part

    def varcoef3d(self, nx, ny, nz, sigma, corr, seed):
        nnz = self.lib.orc_varcoef3d(nx, ny, nz, sigma, corr, seed, None, None, None)
        rp = np.empty(nx * ny * nz + 1, np.int32)
        ci = np.empty(nnz, np.int32)
        v = np.empty(nnz, np.float64)
        self.lib.orc_varcoef3d(nx, ny, nz, sigma, corr, seed, rp.ctypes.data, ci.ctypes.data,
                               v.ctypes.data)
        return HostMatrix(rp, ci, v)

    def solve_true_rel(self, A, b, pc, restart, rtol, fgmres=False, max_cycles=400,
                       on_cycle=None):
        """The oracle harness for an FP64 true-relative-residual target: the
        reference's GMRES (or FGMRES) one restart cycle at a time (tol 0,
        max_iter = restart, warm start through x) until ||b - A x|| / ||b||
        <= rtol, checked in FP64 between cycles.  Returns (x, iterations,
        cycles, relative residual)."""
        x = np.zeros(A.nrows)
        bn = np.linalg.norm(b)
        its = cycles = 0
        rel = 1.0
        fn = self.fgmres if fgmres else self.gmres
        for _ in range(max_cycles):
            r = fn(A, b, x, pc, restart=restart, max_iter=restart, tol=0.0)
            x = r["x"]
            its += r["iterations"]
            cycles += 1
            rel = float(np.linalg.norm(b - self.spmv(A, x)) / bn)
            if on_cycle:
                on_cycle(cycles, rel)
            if rel <= rtol:
                break
        return x, its, cycles, rel


class HostMatrix:
    """A CSR matrix in host memory (int32 row_ptr / col_idx, FP64 values),
    the layout of src/core/sparse_matrix.h:13-18."""

    def __init__(self, row_ptr, col_idx, vals):
        self.row_ptr = np.ascontiguousarray(row_ptr, np.int32)
        self.col_idx = np.ascontiguousarray(col_idx, np.int32)
        self.vals = np.ascontiguousarray(vals, np.float64)
        self.nrows = self.ncols = len(self.row_ptr) - 1

    def nnz(self) -> int:
        return int(self.row_ptr[-1])


class OraclePC:
    def __init__(self, orc, kind, A, nparts, overlap, part):
        self.orc = orc
        self.n = A.nrows
        self.nparts = nparts
        rp, ci, v = _csr_args(A)
        err = C.c_int(0)
        pp = None
        if part is not None:
            self._part = np.ascontiguousarray(part, dtype=np.int32)
            pp = self._part.ctypes.data
        k = PC_KINDS[kind] if isinstance(kind, str) else int(kind)
        self.handle = orc.lib.orc_pc_create(k, A.nrows, rp, ci, v, nparts, overlap, pp,
                                            C.byref(err))
        if err.value:
            orc.lib.orc_pc_destroy(self.handle)
            self.handle = None
            raise RuntimeError({2: "invalid partition", 3: "Coarse matrix is singular"}
                               .get(err.value, f"oracle setup error {err.value}"))

    def apply(self, x):
        y = np.empty(self.n, dtype=np.float64)
        self.orc.lib.orc_pc_apply(self.handle, np.ascontiguousarray(x, dtype=np.float64), y,
                                  self.n)
        return y

    def coarse_a0(self):
        nc = self.orc.lib.orc_pc_coarse(self.handle, None)
        a0 = np.empty(nc * nc, dtype=np.float64)
        self.orc.lib.orc_pc_coarse(self.handle, a0.ctypes.data)
        return a0.reshape(nc, nc)

    def sub_factor(self, s):
        nnz = C.c_int(0)
        rp = C.POINTER(C.c_int)()
        ci = C.POINTER(C.c_int)()
        lu = C.POINTER(C.c_double)()
        dg = C.POINTER(C.c_int)()
        n = self.orc.lib.orc_pc_sub_factor(self.handle, s, C.byref(nnz), C.byref(rp),
                                           C.byref(ci), C.byref(lu), C.byref(dg))
        if n < 0:
            raise IndexError(s)
        z = nnz.value
        return (np.ctypeslib.as_array(rp, (n + 1,)).copy(),
                np.ctypeslib.as_array(ci, (max(z, 1),))[:z].copy(),
                np.ctypeslib.as_array(lu, (max(z, 1),))[:z].copy(),
                np.ctypeslib.as_array(dg, (max(n, 1),))[:n].copy())

    def __del__(self):
        if getattr(self, "handle", None):
            self.orc.lib.orc_pc_destroy(self.handle)
            self.handle = None


class Reference(_Lib):
    """The reference's own sources (oracle/_ref/libref.so)."""

    def __init__(self, path: str = REF_SO):
        super().__init__(path)
        L = self.lib
        L.ref_set_partition.argtypes = [_i32p, C.c_int, C.c_int]
        L.ref_spmv.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _f64p]
        L.ref_poisson2d.argtypes = [C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_poisson2d.restype = C.c_int
        L.ref_poisson3d.argtypes = [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]
        L.ref_poisson3d.restype = C.c_int
        L.ref_ilu0.argtypes = [C.c_int, _i32p, _i32p, _f64p, _f64p, _i32p]
        L.ref_decompose.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int] + [C.c_void_p] * 6
        L.ref_decompose.restype = C.c_int
        L.ref_coarse_a0.argtypes = [C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int, C.c_void_p]
        L.ref_coarse_a0.restype = C.c_int
        L.ref_pc_create.argtypes = [C.c_int, C.c_int, _i32p, _i32p, _f64p, C.c_int, C.c_int]
        L.ref_pc_create.restype = C.c_void_p
        L.ref_pc_apply.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int]
        L.ref_pc_destroy.argtypes = [C.c_void_p]
        for fn in (L.ref_gmres, L.ref_fgmres):
            fn.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int, C.c_int, C.c_double,
                           C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p, C.c_int,
                           C.POINTER(C.c_int)]
            fn.restype = C.c_int
        L.ref_bicgstab.argtypes = [C.c_void_p, _f64p, _f64p, C.c_int, C.c_double,
                                   C.POINTER(C.c_int), C.POINTER(C.c_double), C.c_void_p,
                                   C.c_int, C.POINTER(C.c_int)]
        L.ref_bicgstab.restype = C.c_int
        L.ref_read_mm.argtypes = [C.c_char_p, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                  C.POINTER(C.c_int), C.c_void_p, C.c_void_p, C.c_void_p,
                                  C.c_int]
        L.ref_read_mm.restype = C.c_int
        L.ref_conv_metrics.argtypes = [_f64p, C.c_int, C.c_int, _f64p, _i32p, C.c_void_p]
        L.ref_conv_write.argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int, C.c_int,
                                     _f64p, C.c_int, C.c_int]
        L.ref_condition.argtypes = [C.c_void_p, C.c_int, C.c_uint, _f64p, _i32p]
        L.ref_spectral.argtypes = [C.c_void_p, C.c_int, C.c_double, C.c_uint, _f64p, _i32p]

    def set_partition(self, part, nparts):
        part = np.ascontiguousarray(part, dtype=np.int32)
        self.lib.ref_set_partition(part, len(part), nparts)

    def spmv(self, A, x):
        rp, ci, v = _csr_args(A)
        y = np.empty(A.nrows, dtype=np.float64)
        self.lib.ref_spmv(A.nrows, rp, ci, v, np.ascontiguousarray(x, dtype=np.float64), y)
        return y

    def poisson2d(self, nx, ny):
        nz = self.lib.ref_poisson2d(nx, ny, None, None, None)
        rp = np.empty(nx * ny + 1, np.int32); ci = np.empty(nz, np.int32); v = np.empty(nz)
        self.lib.ref_poisson2d(nx, ny, rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
        return rp, ci, v

    def poisson3d(self, nx, ny, nz_):
        nz = self.lib.ref_poisson3d(nx, ny, nz_, None, None, None)
        rp = np.empty(nx * ny * nz_ + 1, np.int32); ci = np.empty(nz, np.int32); v = np.empty(nz)
        self.lib.ref_poisson3d(nx, ny, nz_, rp.ctypes.data, ci.ctypes.data, v.ctypes.data)
        return rp, ci, v

    def ilu0_factor(self, A):
        rp, ci, v = _csr_args(A)
        lu = np.empty_like(v); dg = np.empty(A.nrows, np.int32)
        self.lib.ref_ilu0(A.nrows, rp, ci, v, lu, dg)
        return lu, dg

    def decompose(self, A, part, nparts, overlap):
        self.set_partition(part, nparts)
        rp, ci, v = _csr_args(A)
        tot = self.lib.ref_decompose(A.nrows, rp, ci, v, nparts, overlap, *([None] * 6))
        if tot < 0:
            raise RuntimeError("reference decomposition failed")
        sub_ptr = np.empty(nparts + 1, np.int32); sub = np.empty(max(tot, 1), np.int32)
        ol_ptr = np.empty(nparts + 1, np.int32); ol = np.empty(max(A.nrows, 1), np.int32)
        ow_ptr = np.empty(nparts + 1, np.int32); ow = np.empty(max(A.nrows, 1), np.int32)
        self.lib.ref_decompose(A.nrows, rp, ci, v, nparts, overlap, sub_ptr.ctypes.data,
                               sub.ctypes.data, ol_ptr.ctypes.data, ol.ctypes.data,
                               ow_ptr.ctypes.data, ow.ctypes.data)
        return dict(owned_ptr=ow_ptr, owned=ow[: ow_ptr[-1]], sub_ptr=sub_ptr, sub=sub[:tot],
                    ownloc_ptr=ol_ptr, ownloc=ol[: ol_ptr[-1]])

    def coarse_a0(self, A, part, nparts, overlap):
        self.set_partition(part, nparts)
        rp, ci, v = _csr_args(A)
        a0 = np.empty(nparts * nparts)
        nc = self.lib.ref_coarse_a0(A.nrows, rp, ci, v, nparts, overlap, a0.ctypes.data)
        if nc < 0:
            raise RuntimeError("reference coarse build failed")
        return a0.reshape(nparts, nparts)

    def precond(self, kind, A, nparts=4, overlap=1, part=None):
        return RefPC(self, kind, A, nparts, overlap, part)

    def _solve(self, fn, A, b, x0, pc, restart, max_iter, tol, hist_cap=0):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        it = C.c_int(0); res = C.c_double(0.0); hl = C.c_int(0)
        hist = np.zeros(max(hist_cap, 1))
        if pc is None:
            pc = RefPC(self, "none", A, 1, 0, None)
        conv = fn(pc.handle, b, x, restart, max_iter, tol, C.byref(it), C.byref(res),
                  hist.ctypes.data if hist_cap else None, hist_cap, C.byref(hl))
        return dict(x=x, converged=bool(conv), iterations=it.value, residual_norm=res.value,
                    history=hist[: min(hl.value, hist_cap)].copy())

    def gmres(self, A, b, x0, pc=None, restart=30, max_iter=1000, tol=1e-10, hist_cap=0):
        return self._solve(self.lib.ref_gmres, A, b, x0, pc, restart, max_iter, tol, hist_cap)

    def fgmres(self, A, b, x0, pc=None, restart=30, max_iter=1000, tol=1e-10, hist_cap=0):
        return self._solve(self.lib.ref_fgmres, A, b, x0, pc, restart, max_iter, tol, hist_cap)


def _ref_methods(cls):
    def read_mm(self, path):
        nr, nc, nz = C.c_int(0), C.c_int(0), C.c_int(0)
        if self.lib.ref_read_mm(path.encode(), C.byref(nr), C.byref(nc), C.byref(nz), None,
                                None, None, 0):
            raise RuntimeError("reference read_matrix_market threw")
        rp = np.empty(nr.value + 1, np.int32)
        ci = np.empty(max(nz.value, 1), np.int32)
        v = np.empty(max(nz.value, 1))
        self.lib.ref_read_mm(path.encode(), C.byref(nr), C.byref(nc), C.byref(nz),
                             rp.ctypes.data, ci.ctypes.data, v.ctypes.data, ci.size)
        return nr.value, nc.value, rp, ci[: nz.value], v[: nz.value]

    def conv_metrics(self, hist, converged):
        h = np.ascontiguousarray(hist, np.float64)
        d = np.zeros(3)
        i = np.zeros(2, np.int32)
        rates = np.zeros(max(len(h), 1))
        self.lib.ref_conv_metrics(h, len(h), int(converged), d, i, rates.ctypes.data)
        return dict(initial_residual=d[0], final_residual=d[1], asymptotic_rate=d[2],
                    iterations=int(i[0]), stagnation_start=int(i[1]), rates=rates[: len(h)])

    def conv_write(self, path, matrix, precond, nparts, overlap, hist, converged):
        h = np.ascontiguousarray(hist, np.float64)
        self.lib.ref_conv_write(path.encode(), matrix.encode(), precond.encode(), nparts,
                                overlap, h, len(h), int(converged))

    def bicgstab(self, A, b, x0, pc=None, max_iter=1000, tol=1e-10, hist_cap=0):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.array(x0, dtype=np.float64, copy=True)
        it, res, hl = C.c_int(0), C.c_double(0.0), C.c_int(0)
        hist = np.zeros(max(hist_cap, 1))
        if pc is None:
            pc = RefPC(self, "none", A, 1, 0, None)
        conv = self.lib.ref_bicgstab(pc.handle, b, x, max_iter, tol, C.byref(it), C.byref(res),
                                     hist.ctypes.data if hist_cap else None, hist_cap,
                                     C.byref(hl))
        return dict(x=x, converged=bool(conv), iterations=it.value, residual_norm=res.value,
                    history=hist[: min(hl.value, hist_cap)].copy(), history_len=hl.value)

    def condition(self, A, pc=None, k=80, seed=42):
        if pc is None:
            pc = RefPC(self, "none", A, 1, 0, None)
        out = np.zeros(3)
        iout = np.zeros(2, np.int32)
        self.lib.ref_condition(pc.handle, k, seed, out, iout)
        return dict(lambda_min=out[0], lambda_max=out[1], kappa=out[2],
                    lanczos_steps=int(iout[0]), valid=bool(iout[1]))

    def spectral(self, A, pc=None, max_iter=200, tol=1e-6, seed=123):
        if pc is None:
            pc = RefPC(self, "none", A, 1, 0, None)
        out = np.zeros(1)
        iout = np.zeros(2, np.int32)
        self.lib.ref_spectral(pc.handle, max_iter, tol, seed, out, iout)
        return dict(spectral_radius=out[0], power_iters=int(iout[0]),
                    convergence_ok=bool(iout[1]))

    for f in (read_mm, conv_metrics, conv_write, bicgstab, condition, spectral):
        setattr(cls, f.__name__, f)
    return cls


Reference = _ref_methods(Reference)


class RefPC:
    def __init__(self, ref, kind, A, nparts, overlap, part):
        self.ref = ref
        self.n = A.nrows
        if part is not None:
            ref.set_partition(part, nparts)
        rp, ci, v = _csr_args(A)
        k = PC_KINDS[kind] if isinstance(kind, str) else int(kind)
        self.handle = ref.lib.ref_pc_create(k, A.nrows, rp, ci, v, nparts, overlap)
        if not self.handle:
            raise RuntimeError("reference preconditioner setup threw")

    def apply(self, x):
        y = np.empty(self.n)
        self.ref.lib.ref_pc_apply(self.handle, np.ascontiguousarray(x, dtype=np.float64), y, self.n)
        return y

    def __del__(self):
        if getattr(self, "handle", None):
            self.ref.lib.ref_pc_destroy(self.handle)
            self.handle = None
