"""schwarz_gmres_dashboard_gb300 -- GB300 (sm_103a) solve path of schwarz-gmres.

Python mirror of the reference's C++ interface (src/core/sparse_matrix.h,
src/precond/*.h, src/core/gmres.h, src/core/fgmres.h) over the C ABI of
libsgmres.so.  Same names, argument meaning and error behaviour:

    A = make_poisson_2d(20, 20)
    M = RASPrecond(4, 1); M.setup(A)
    x = np.zeros(A.nrows)
    res = gmres(A, b, x, M, GMRESParams(restart=30, tol=1e-10))

Every numerical step runs on the GPU; there is no CPU fallback -- without the
built library the import fails, without a device the calls raise.
Vectors may be numpy arrays (host) or CUDA tensors / objects exposing
``__cuda_array_interface__`` (used in place on the device).
"""
from __future__ import annotations

import ctypes as C
import enum
from dataclasses import dataclass, field
from typing import List, Optional

import numpy as np

from . import _lib as L
from ._lib import SgError

_clib = L.load()

__all__ = [
    "SgError", "Context", "default_context", "CSRMatrix", "make_identity", "make_poisson_2d",
    "read_matrix_market", "convergence_metrics", "write_convergence_jsonl", "bicgstab",
    "estimate_condition", "estimate_spectral_radius", "HostPreconditioner",
    "make_poisson_3d", "make_varcoef_3d", "uniform", "partition_graph", "partition_boxes",
    "schwarz_structure", "dot", "norm2", "axpy", "scale",
    "Preconditioner", "NoPrecond", "JacobiPrecond", "ILU0Precond", "ASMPrecond", "RASPrecond",
    "TwoLevelSchwarzPrecond", "FineLevelType", "GMRESParams", "GMRESResult", "gmres", "fgmres",
    "FP64", "FP32", "BF16", "TOL_REF_ABS", "TOL_TRUE_REL_CYCLE", "TOL_TRUE_REL",
    "LearnedCorrection", "collect_pairs", "make_aniso_2d", "BatchProblem", "make_aniso_batch",
    "solve_batched",
]

FP64, FP32, BF16 = L.FP64, L.FP32, L.BF16
TOL_REF_ABS, TOL_TRUE_REL_CYCLE, TOL_TRUE_REL = L.TOL_REF_ABS, L.TOL_TRUE_REL_CYCLE, L.TOL_TRUE_REL


def _check(st):
    L.check(st)


# ---------------------------------------------------------------- context
class Context:
    """One device and one stream (replaces CudaHandles, src/gpu/cuda_common.h:42-107)."""

    def __init__(self, device: int = 0):
        h = C.c_void_p()
        _check(_clib.sg_ctx_create(int(device), C.byref(h)))
        self.handle = h
        self.device = device

    def set_stream(self, stream_ptr: int | None) -> None:
        _check(_clib.sg_ctx_set_stream(self.handle, C.c_void_p(stream_ptr or 0)))

    @property
    def stream(self) -> int:
        s = C.c_void_p()
        _check(_clib.sg_ctx_get_stream(self.handle, C.byref(s)))
        return s.value or 0

    def synchronize(self) -> None:
        _check(_clib.sg_ctx_synchronize(self.handle))

    TIMER_KINDS = ("spmv", "residual", "precond", "ortho", "update", "learned")

    def set_timing(self, on: bool) -> None:
        """Kernel-class CUDA-event timers for solves run without a graph."""
        _check(_clib.sg_ctx_set_timing(self.handle, 1 if on else 0))

    def timing(self) -> dict:
        out = {}
        for k, nm in enumerate(self.TIMER_KINDS):
            ms, cnt = C.c_double(0.0), C.c_longlong(0)
            _check(_clib.sg_ctx_get_timing(self.handle, k, C.byref(ms), C.byref(cnt)))
            out[nm] = (ms.value, int(cnt.value))
        return out

    @property
    def launch_count(self) -> int:
        """Kernels launched through this context so far."""
        c = C.c_longlong(0)
        _check(_clib.sg_ctx_get_launch_count(self.handle, C.byref(c)))
        return int(c.value)

    @property
    def capture_count(self) -> int:
        """Restart cycles captured as CUDA graphs so far (a solve reuses the
        previous capture while its inputs are unchanged)."""
        c = C.c_longlong(0)
        _check(_clib.sg_ctx_get_capture_count(self.handle, C.byref(c)))
        return int(c.value)

    def close(self) -> None:
        if getattr(self, "handle", None):
            _clib.sg_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_default_ctx: Optional[Context] = None


def default_context() -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(0)
    return _default_ctx


def _vec(a, n: int, writable: bool = False):
    """(pointer, mem, keepalive) for a host numpy array or a device array."""
    cai = getattr(a, "__cuda_array_interface__", None)
    if cai is not None:
        ptr = cai["data"][0]
        typestr = cai["typestr"]
        if typestr not in ("<f8", "=f8"):
            raise TypeError("device vectors must be float64")
        if cai.get("strides") not in (None, (8,)):
            raise TypeError("device vectors must be contiguous")
        if int(np.prod(cai["shape"])) < n:
            raise ValueError("device vector too short")
        return C.c_void_p(ptr), L.MEM_DEVICE, a
    if not isinstance(a, np.ndarray) or a.dtype != np.float64 or not a.flags.c_contiguous:
        if writable:
            raise TypeError("output vectors must be contiguous float64 numpy arrays")
        a = np.ascontiguousarray(a, dtype=np.float64)
    if a.size < n:
        raise ValueError("vector too short")
    return C.c_void_p(a.ctypes.data), L.MEM_HOST, a


# ---------------------------------------------------------------- matrix
class CSRMatrix:
    """CSRMatrix of src/core/sparse_matrix.h:13-84: int32 row_ptr/col_idx,
    float64 vals, 0-based.  The device copy is made on first use (or by
    ``upload()``); call ``upload()`` again after changing the arrays."""

    def __init__(self, nrows=0, ncols=0, row_ptr=None, col_idx=None, vals=None):
        self.nrows = int(nrows)
        self.ncols = int(ncols)
        self.row_ptr = np.zeros(self.nrows + 1, np.int32) if row_ptr is None else \
            np.ascontiguousarray(row_ptr, dtype=np.int32)
        self.col_idx = np.zeros(0, np.int32) if col_idx is None else \
            np.ascontiguousarray(col_idx, dtype=np.int32)
        self.vals = np.zeros(0, np.float64) if vals is None else \
            np.ascontiguousarray(vals, dtype=np.float64)
        self._dev = None
        self._ctx = None

    def nnz(self) -> int:
        return int(self.vals.size)

    def upload(self, ctx: Context | None = None):
        ctx = ctx or default_context()
        self.release()
        h = C.c_void_p()
        _check(_clib.sg_csr_create(ctx.handle, self.nrows, self.ncols, self.nnz(),
                                  self.row_ptr.ctypes.data, self.col_idx.ctypes.data,
                                  self.vals.ctypes.data, L.MEM_HOST, C.byref(h)))
        self._dev, self._ctx = h, ctx
        return self

    def device(self, ctx: Context | None = None):
        if self._dev is None or (ctx is not None and ctx is not self._ctx):
            self.upload(ctx)
        return self._dev

    def release(self):
        if self._dev is not None:
            _clib.sg_csr_destroy(self._dev)
            self._dev = None

    def __del__(self):
        try:
            self.release()
        except Exception:
            pass

    def spmv(self, x, y=None):
        """y = A x on the GPU (sparse_matrix.h:30-37), bit-identical to the
        reference's row loop."""
        dev = self.device()
        if y is None:
            y = np.empty(self.nrows, np.float64)
        px, mx, _kx = _vec(x, self.ncols)
        py, my, _ky = _vec(y, self.nrows, writable=True)
        if mx != my:
            raise TypeError("x and y must both be host or both be device arrays")
        _check(_clib.sg_csr_spmv(dev, px, py, mx))
        return y

    @property
    def format(self) -> int:
        """SpMV storage: 0 autotune (not decided yet), 1 CSR, 2 SELL-32,
        3 SELL-32 with 16-bit column offsets."""
        f = C.c_int(0)
        _check(_clib.sg_csr_get_format(self.device(), C.byref(f)))
        return f.value

    @format.setter
    def format(self, fmt: int) -> None:
        _check(_clib.sg_csr_set_format(self.device(), int(fmt)))

    def spmv_choice(self) -> dict:
        """The autotuner's SpMV choice for the FP64 values and the FP32 copy."""
        f, v, f32, v32 = C.c_int(0), C.c_int(0), C.c_int(0), C.c_int(0)
        _check(_clib.sg_csr_get_spmv_choice(self.device(), C.byref(f), C.byref(v), C.byref(f32),
                                           C.byref(v32)))
        return {"format": f.value, "variant": v.value, "format32": f32.value,
                "variant32": v32.value}

    def set_spmv_variant(self, variant: int) -> None:
        """Force one SELL launch variant of the autotuner's set (testing)."""
        _check(_clib.sg_csr_set_spmv_variant(self.device(), int(variant)))

    def diagonal(self, i: int) -> float:
        for e in range(self.row_ptr[i], self.row_ptr[i + 1]):
            if self.col_idx[e] == i:
                return float(self.vals[e])
        return 0.0


def make_identity(n: int) -> CSRMatrix:
    """make_identity (src/core/sparse_matrix.h:86-96)"""
    return CSRMatrix(n, n, np.arange(n + 1, dtype=np.int32), np.arange(n, dtype=np.int32),
                     np.ones(n))


def _gen(fn, dims, n, *extra):
    nnz = C.c_int(0)
    _check(fn(*dims, *extra, None, None, None, C.byref(nnz)))
    rp = np.empty(n + 1, np.int32)
    ci = np.empty(nnz.value, np.int32)
    v = np.empty(nnz.value, np.float64)
    _check(fn(*dims, *extra, rp.ctypes.data, ci.ctypes.data, v.ctypes.data, C.byref(nnz)))
    return CSRMatrix(n, n, rp, ci, v)


def make_poisson_2d(nx: int, ny: int) -> CSRMatrix:
    """5-point Laplacian, Dirichlet (src/mesh/poisson.h:10-38)."""
    return _gen(_clib.sg_gen_poisson2d, (nx, ny), nx * ny)


def make_poisson_3d(nx: int, ny: int, nz: int) -> CSRMatrix:
    """7-point Laplacian, Dirichlet (src/mesh/poisson.h:41-74)."""
    return _gen(_clib.sg_gen_poisson3d, (nx, ny, nz), nx * ny * nz)


def make_varcoef_3d(nx: int, ny: int, nz: int, sigma: float = 1.0, corr_len: float = 8.0,
                    seed: int = 0) -> CSRMatrix:
    """-div(k grad u), 7-point, k = exp(sigma * g), g a seeded unit-variance
    Gaussian random field with squared-exponential correlation length
    `corr_len` cells; harmonic-mean face coefficients."""
    return _gen(_clib.sg_gen_varcoef3d, (nx, ny, nz), nx * ny * nz,
                C.c_double(sigma), C.c_double(corr_len), C.c_uint64(seed))


def make_aniso_2d(nx: int, ny: int, eps: float, theta: float) -> CSRMatrix:
    """-div(K grad u), K = R(theta) diag(1, eps) R(theta)^T, 9-point stencil,
    Dirichlet, on an nx*ny grid."""
    return _gen(_clib.sg_gen_aniso2d, (nx, ny), nx * ny, C.c_double(eps), C.c_double(theta))


def uniform(n: int, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    """Seeded U[lo,hi) values from SplitMix64 ((x >> 11) * 2^-53)."""
    out = np.empty(n, np.float64)
    _check(_clib.sg_gen_uniform(C.c_uint64(seed), n, C.c_double(lo), C.c_double(hi),
                               out.ctypes.data))
    return out


def read_matrix_market(path: str) -> CSRMatrix:
    """read_matrix_market (src/io/matrix_market.h:14-92): the same reading
    rules (symmetric mirrored, pattern read as 1.0, duplicates kept)."""
    nr, nc, nz = C.c_int(0), C.c_int(0), C.c_int(0)
    _check(_clib.sg_read_matrix_market(path.encode(), C.byref(nr), C.byref(nc), C.byref(nz),
                                       None, None, None, 0))
    rp = np.empty(nr.value + 1, np.int32)
    ci = np.empty(max(nz.value, 1), np.int32)
    v = np.empty(max(nz.value, 1), np.float64)
    _check(_clib.sg_read_matrix_market(path.encode(), C.byref(nr), C.byref(nc), C.byref(nz),
                                       rp.ctypes.data, ci.ctypes.data, v.ctypes.data, ci.size))
    return CSRMatrix(nr.value, nc.value, rp, ci[: nz.value], v[: nz.value])


def convergence_metrics(history, converged: bool) -> dict:
    """ConvergenceMetrics (src/analysis/convergence_analysis.h:15-65) of a
    residual history."""
    h = np.ascontiguousarray(history, np.float64)
    out = L.Convergence()
    rates = np.zeros(max(h.size, 1))
    _check(_clib.sg_convergence_metrics(h.ctypes.data, h.size, int(bool(converged)),
                                        C.byref(out), rates.ctypes.data))
    return dict(iterations=out.iterations, converged=bool(out.converged),
                stagnation_start=out.stagnation_start, initial_residual=out.initial_residual,
                final_residual=out.final_residual, asymptotic_rate=out.asymptotic_rate,
                rates=rates[: h.size])


def write_convergence_jsonl(path: str, matrix: str, precond: str, nparts: int, overlap: int,
                            history, converged: bool) -> None:
    """Appends the <output>.conv.jsonl record of the reference CLI
    (src/analysis/convergence_analysis.h:69-93)."""
    h = np.ascontiguousarray(history, np.float64)
    _check(_clib.sg_write_convergence_jsonl(path.encode(), matrix.encode(), precond.encode(),
                                            nparts, overlap, h.ctypes.data, h.size,
                                            int(bool(converged))))


def partition_graph(A: CSRMatrix, nparts: int) -> np.ndarray:
    """Built-in graph partitioner (takes METIS_PartGraphKway's place)."""
    part = np.empty(A.nrows, np.int32)
    _check(_clib.sg_partition_graph(A.nrows, A.row_ptr.ctypes.data, A.col_idx.ctypes.data,
                                   nparts, part.ctypes.data))
    return part


def partition_boxes(nx: int, ny: int, nz: int, nparts: int, spread: float = 0.0,
                    seed: int = 0) -> np.ndarray:
    """Boxes of a grid from recursive coordinate bisection with seeded uneven cuts."""
    part = np.empty(nx * ny * nz, np.int32)
    _check(_clib.sg_partition_boxes(nx, ny, nz, nparts, C.c_double(spread), C.c_uint64(seed),
                                   part.ctypes.data))
    return part


STRUCTURE_NAMES = ["partition", "owned_ptr", "owned", "sub_ptr", "sub", "ownloc_ptr", "ownloc",
                   "local_row_ptr", "local_col_idx", "diag_ptr", "level_lower", "level_upper"]


def schwarz_structure(A: CSRMatrix, part, nparts: int, overlap: int) -> dict:
    """Host-side integer set-up of the Schwarz/ILU(0) preconditioners (the part
    of setup() that runs before any device work); no GPU needed."""
    part = np.ascontiguousarray(part, dtype=np.int32)
    out = {}
    for which, nm in enumerate(STRUCTURE_NAMES):
        ln = C.c_int(0)
        _check(_clib.sg_schwarz_structure(A.nrows, A.row_ptr.ctypes.data, A.col_idx.ctypes.data,
                                         part.ctypes.data, nparts, overlap, which, None, 0,
                                         C.byref(ln)))
        arr = np.empty(max(ln.value, 1), np.int32)
        _check(_clib.sg_schwarz_structure(A.nrows, A.row_ptr.ctypes.data, A.col_idx.ctypes.data,
                                         part.ctypes.data, nparts, overlap, which,
                                         arr.ctypes.data, arr.size, C.byref(ln)))
        out[nm] = arr[: ln.value]
    return out


# ---------------------------------------------------------------- BLAS-1
def dot(a, b, ctx: Context | None = None) -> float:
    """dot (src/core/vector.h:11-16) on the GPU, FP64, deterministic order."""
    ctx = ctx or default_context()
    n = len(a) if not hasattr(a, "__cuda_array_interface__") else a.__cuda_array_interface__["shape"][0]
    pa, ma, _ka = _vec(a, n)
    pb, mb, _kb = _vec(b, n)
    if ma != mb:
        raise TypeError("a and b must both be host or both be device arrays")
    out = C.c_double(0.0)
    _check(_clib.sg_dot(ctx.handle, pa, pb, n, ma, C.byref(out)))
    return out.value


def norm2(a, ctx: Context | None = None) -> float:
    """norm2 (src/core/vector.h:23-25)."""
    ctx = ctx or default_context()
    n = len(a) if not hasattr(a, "__cuda_array_interface__") else a.__cuda_array_interface__["shape"][0]
    pa, ma, _ka = _vec(a, n)
    out = C.c_double(0.0)
    _check(_clib.sg_norm2(ctx.handle, pa, n, ma, C.byref(out)))
    return out.value


def axpy(alpha: float, x, y, ctx: Context | None = None):
    """y += alpha x in place (src/core/vector.h:31-34)."""
    ctx = ctx or default_context()
    n = len(y) if not hasattr(y, "__cuda_array_interface__") else y.__cuda_array_interface__["shape"][0]
    px, mx, _kx = _vec(x, n)
    py, my, _ky = _vec(y, n, writable=True)
    if mx != my:
        raise TypeError("x and y must both be host or both be device arrays")
    _check(_clib.sg_axpy(ctx.handle, C.c_double(alpha), px, py, n, my))
    return y


def scale(alpha: float, x, ctx: Context | None = None):
    """x *= alpha in place (src/core/vector.h:40-44)."""
    ctx = ctx or default_context()
    n = len(x) if not hasattr(x, "__cuda_array_interface__") else x.__cuda_array_interface__["shape"][0]
    px, mx, _kx = _vec(x, n, writable=True)
    _check(_clib.sg_scale(ctx.handle, C.c_double(alpha), px, n, mx))
    return x


# ---------------------------------------------------------------- preconditioners
class FineLevelType(enum.Enum):
    """src/precond/two_level_schwarz.h:21"""
    ASM = 0
    RAS = 1


class Preconditioner:
    """Preconditioner plugin of src/precond/preconditioner.h:7-20:
    setup(A) then apply(x) -> y = M^{-1} x (overwrites all of y)."""

    kind = "none"

    def __init__(self, nparts: int = 1, overlap: int = 0, partition=None,
                 factor_dtype: int = FP64, sweep_dtype: int = FP64,
                 ctx: Context | None = None, generic_sweep: bool = False,
                 sweep: str = "tma", sweep_threads: int = 0, fuse_restrict: bool = True,
                 group_bytes: int = 0, sweep_launch: str = "auto", setup: str = "device"):
        # sweep variant (testing/comparison): "tma" (default: TMA-fed level
        # records), "level" (factors read from global memory), "syncfree"
        if generic_sweep:
            sweep = "level"
        self.sweep = sweep
        self.ctx = ctx or default_context()
        self.nparts = int(nparts)
        self.overlap = int(overlap)
        self.partition = None if partition is None else np.ascontiguousarray(partition, np.int32)
        self.factor_dtype = factor_dtype
        self.sweep_dtype = sweep_dtype
        opts = L.PrecondOpts()
        opts.nparts = self.nparts
        opts.overlap = self.overlap
        opts.factor_dtype = factor_dtype
        opts.sweep_dtype = sweep_dtype
        opts.partition = self.partition.ctypes.data if self.partition is not None else None
        opts.reserved[0] = {"tma": 0, "level": 1, "syncfree": 4}[self.sweep]
        # threads per CTA of the TMA-fed sweep (0: timed at set-up)
        opts.reserved[1] = int(sweep_threads)
        # two-level: coarse restriction inside the TMA-fed sweep when all the
        # subdomains' CTAs fit at once (False: a kernel of its own; same bits)
        opts.reserved[2] = 0 if fuse_restrict else 1
        # largest group of level records the TMA-fed sweep copies at once
        # (0: 8 or 16 KB, timed at set-up; same results either way)
        opts.reserved[3] = int(group_bytes)
        # launch shape of the TMA-fed sweep: "auto" (timed), "per_subdomain"
        # (one CTA each), "persistent" (resident CTAs loop over subdomains)
        # or an int k > 2 (persistent with at most k CTAs)
        opts.reserved[4] = (int(sweep_launch) if isinstance(sweep_launch, int) else
                            {"auto": 0, "per_subdomain": 1, "persistent": 2}[sweep_launch])
        # integer set-up: "device" (kernels; host threads when its bitmaps
        # would not fit) or "host" (threads); same results
        opts.reserved[5] = {"device": 0, "host": 1}[setup]
        self._opts = opts
        h = C.c_void_p()
        _check(_clib.sg_precond_create(self.ctx.handle, L.PC_KINDS[self.kind], C.byref(opts),
                                      C.byref(h)))
        self.handle = h
        self.n = 0

    def setup(self, A: CSRMatrix) -> None:
        _check(_clib.sg_precond_setup(self.handle, A.device(self.ctx)))
        self.n = A.nrows

    def apply(self, x, y=None):
        if y is None:
            y = np.empty(self.n, np.float64)
        px, mx, _kx = _vec(x, self.n)
        py, my, _ky = _vec(y, self.n, writable=True)
        if mx != my:
            raise TypeError("x and y must both be host or both be device arrays")
        _check(_clib.sg_precond_apply(self.handle, px, py, self.n, mx))
        return y

    # ---- set-up read-back (parity checks)
    def decomposition(self) -> dict:
        names = ["partition", "owned_ptr", "owned", "sub_ptr", "sub", "ownloc_ptr", "ownloc"]
        out = {}
        for which, nm in enumerate(names):
            ln = C.c_int(0)
            _check(_clib.sg_precond_get_decomposition(self.handle, which, None, 0, C.byref(ln)))
            arr = np.empty(max(ln.value, 1), np.int32)
            _check(_clib.sg_precond_get_decomposition(self.handle, which, arr.ctypes.data,
                                                     arr.size, C.byref(ln)))
            out[nm] = arr[: ln.value]
        return out

    def factors(self, s: int = 0) -> dict:
        ns, nz = C.c_int(0), C.c_int(0)
        _check(_clib.sg_precond_get_factors(self.handle, s, C.byref(ns), C.byref(nz), None, None,
                                           None, None, None, None))
        rp = np.empty(ns.value + 1, np.int32)
        ci = np.empty(max(nz.value, 1), np.int32)
        lu = np.empty(max(nz.value, 1), np.float64)
        dg = np.empty(max(ns.value, 1), np.int32)
        lo = np.empty(max(ns.value, 1), np.int32)
        up = np.empty(max(ns.value, 1), np.int32)
        _check(_clib.sg_precond_get_factors(self.handle, s, C.byref(ns), C.byref(nz),
                                           rp.ctypes.data, ci.ctypes.data, lu.ctypes.data,
                                           dg.ctypes.data, lo.ctypes.data, up.ctypes.data))
        k, z = ns.value, nz.value
        return dict(row_ptr=rp, col_idx=ci[:z], lu_vals=lu[:z], diag_ptr=dg[:k],
                    level_lower=lo[:k], level_upper=up[:k])

    def coarse_a0(self) -> np.ndarray:
        nc = C.c_int(0)
        _check(_clib.sg_precond_get_coarse(self.handle, None, 0, C.byref(nc)))
        a0 = np.empty(nc.value * nc.value, np.float64)
        _check(_clib.sg_precond_get_coarse(self.handle, a0.ctypes.data, a0.size, C.byref(nc)))
        return a0.reshape(nc.value, nc.value)

    def sweep_choice(self) -> dict:
        """The subdomain sweep chosen at set-up: kind ("tma", "level",
        "syncfree" or "none") and threads per CTA of the TMA-fed sweep."""
        k, t = C.c_int(0), C.c_int(0)
        _check(_clib.sg_precond_get_sweep(self.handle, C.byref(k), C.byref(t)))
        kinds = {0: "tma", 1: "level", 2: "syncfree", -1: "none"}
        rb, gb = C.c_int(0), C.c_int(0)
        _check(_clib.sg_precond_get_sweep_ring(self.handle, C.byref(rb), C.byref(gb)))
        return {"sweep": kinds[k.value], "threads": t.value, "ring_bytes": rb.value,
                "group_bytes": gb.value}

    def setup_on_device(self) -> bool:
        """True when the last set-up's integer part ran on the device."""
        v = C.c_int(0)
        _check(_clib.sg_precond_get_setup_path(self.handle, C.byref(v)))
        return bool(v.value)

    def schedule(self, which: int) -> np.ndarray:
        """Read-back of a subdomain schedule array (sg_precond_get_schedule)."""
        ln = C.c_longlong(0)
        _check(_clib.sg_precond_get_schedule(self.handle, int(which), None, 0, C.byref(ln)))
        out = np.empty(ln.value, np.int32)
        _check(_clib.sg_precond_get_schedule(self.handle, int(which), out.ctypes.data, out.size,
                                             C.byref(ln)))
        return out

    def check(self, plant: bool = False) -> int:
        """Checked mode of the TMA-fed sweep: the number of violated
        invariants of its level records and ring schedule (0: all hold).
        plant=True first corrupts one column slot of the host copy."""
        v = C.c_longlong(-1)
        _check(_clib.sg_precond_check(self.handle, 1 if plant else 0, C.byref(v)))
        return v.value

    def set_wait_test(self, mode: int) -> None:
        """Test hook of the bounded device waits: 1 makes every sweep CTA's
        first record wait run out, 2 the fused coarse restriction's wait
        (~1 ms each; applies and solves then raise SgError with
        SG_ERR_DEVICE_TIMEOUT); 0 restores the normal waits."""
        _check(_clib.sg_precond_set_wait_test(self.handle, int(mode)))

    def close(self):
        if getattr(self, "handle", None):
            _clib.sg_precond_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class HostPreconditioner(Preconditioner):
    """A Preconditioner plug-in of the caller's own (src/precond/
    preconditioner.h:7-20), or FGMRES's flexible apply (FlexApply,
    src/core/fgmres.h:37): fn(x, y) receives numpy views of the input and the
    output (n doubles) and must fill y.  Inside a solve it runs in stream
    order on a CUDA host-function thread, so it must not call into CUDA (nor
    into this package's GPU functions).  An exception inside fn makes the
    call raise SgError (SG_ERR_CALLBACK) carrying the message."""

    kind = "host"

    def __init__(self, fn, n: int, ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.n = int(n)
        self.fn = fn
        self.error = None

        def call(_user, x, y, m):
            try:
                fn(np.ctypeslib.as_array(x, (m,)), np.ctypeslib.as_array(y, (m,)))
                return 0
            except Exception as e:  # reported through the status
                self.error = f"{type(e).__name__}: {e}"
                return 1

        self._cb = L.HOST_APPLY_FN(call)  # kept alive with the object
        h = C.c_void_p()
        _check(_clib.sg_precond_create_host(self.ctx.handle, C.cast(self._cb, C.c_void_p), None,
                                           self.n, C.byref(h)))
        self.handle = h

    def setup(self, A: CSRMatrix) -> None:
        if A.nrows != self.n:
            raise ValueError("size mismatch")


class NoPrecond(Preconditioner):
    kind = "none"


class JacobiPrecond(Preconditioner):
    """src/precond/jacobi.h:10-27"""
    kind = "jacobi"

    def __init__(self, sweep_dtype: int = FP64, ctx: Context | None = None, **kw):
        super().__init__(1, 0, None, FP64 if sweep_dtype == FP64 else FP32, sweep_dtype, ctx, **kw)


class ILU0Precond(Preconditioner):
    """src/precond/ilu0.h:11-93"""
    kind = "ilu0"

    def __init__(self, factor_dtype: int = FP64, sweep_dtype: int = FP64,
                 ctx: Context | None = None, **kw):
        super().__init__(1, 0, None, factor_dtype, sweep_dtype, ctx, **kw)


class ASMPrecond(Preconditioner):
    """src/precond/asm.h:13-71"""
    kind = "asm"

    def __init__(self, nparts: int, overlap: int, partition=None, factor_dtype: int = FP64,
                 sweep_dtype: int = FP64, ctx: Context | None = None, **kw):
        super().__init__(nparts, overlap, partition, factor_dtype, sweep_dtype, ctx, **kw)


class RASPrecond(Preconditioner):
    """src/precond/ras.h:16-82"""
    kind = "ras"

    def __init__(self, nparts: int, overlap: int, partition=None, factor_dtype: int = FP64,
                 sweep_dtype: int = FP64, ctx: Context | None = None, **kw):
        super().__init__(nparts, overlap, partition, factor_dtype, sweep_dtype, ctx, **kw)


class TwoLevelSchwarzPrecond(Preconditioner):
    """src/precond/two_level_schwarz.h:23-75 (fine ASM or RAS + piecewise-constant
    coarse space with an FP64 LU)."""

    def __init__(self, nparts: int, overlap: int, fine_type: FineLevelType = FineLevelType.RAS,
                 partition=None, factor_dtype: int = FP64, sweep_dtype: int = FP64,
                 ctx: Context | None = None, **kw):
        self.kind = "twolevel_asm" if fine_type == FineLevelType.ASM else "twolevel_ras"
        self.fine_type = fine_type
        super().__init__(nparts, overlap, partition, factor_dtype, sweep_dtype, ctx, **kw)


# ---------------------------------------------------------------- solvers
@dataclass
class GMRESParams:
    """GMRESParams (src/core/gmres.h:20-24) plus the GPU options."""
    restart: int = 30
    max_iter: int = 1000
    tol: float = 1e-10
    tol_kind: int = TOL_REF_ABS
    precision: int = FP64
    use_graph: bool = True
    # 0: CGS2 in the fewest passes (two for linear GMRES cycles, restart < 32);
    # 1: classic three-pass CGS2
    ortho: int = 0


@dataclass
class GMRESResult:
    """GMRESResult (src/core/gmres.h:12-18) plus true_rel_residual / cycles."""
    iterations: int = 0
    residual_norm: float = 0.0
    converged: bool = False
    time_solve_s: float = 0.0
    residual_history: List[float] = field(default_factory=list)
    true_rel_residual: float = 0.0
    cycles: int = 0


def _solve(solver: int, A: CSRMatrix, b, x, M: Optional[Preconditioner],
           params: Optional[GMRESParams], history: bool = True) -> GMRESResult:
    params = params or GMRESParams()
    ctx = M.ctx if M is not None else default_context()
    dev = A.device(ctx)
    n = A.nrows
    pb, mb, _kb = _vec(b, n)
    px, mx, _kx = _vec(x, n, writable=True)
    if mb != mx:
        raise TypeError("b and x must both be host or both be device arrays")
    p = L.SolveParams()
    p.restart = params.restart
    p.max_iter = params.max_iter
    p.tol = params.tol
    p.tol_kind = params.tol_kind
    p.precision = params.precision
    p.use_graph = 1 if params.use_graph else 0
    p.ortho = params.ortho
    hist = None
    if history:
        cap = max(params.max_iter, 0) + params.restart + 1
        hist = np.zeros(cap, np.float64)
        p.history = hist.ctypes.data
        p.history_cap = cap
    r = L.SolveResult()
    st = _clib.sg_solve(ctx.handle, solver, dev, M.handle if M is not None else None, pb, px, n,
                       mx, C.byref(p), C.byref(r))
    if st == L.SG_ERR_CALLBACK and getattr(M, "error", None):
        msg, M.error = M.error, None
        raise SgError(st, msg)
    _check(st)
    hl = min(r.history_len, hist.size) if hist is not None else 0
    return GMRESResult(iterations=r.iterations, residual_norm=r.residual_norm,
                       converged=bool(r.converged), time_solve_s=r.time_solve_s,
                       residual_history=list(hist[:hl]) if hist is not None else [],
                       true_rel_residual=r.true_rel_residual, cycles=r.cycles)


def gmres(A: CSRMatrix, b, x, M: Optional[Preconditioner] = None,
          params: Optional[GMRESParams] = None) -> GMRESResult:
    """Restarted GMRES(m), left preconditioning (src/core/gmres.h:28-33).
    x holds x0 on entry and the solution on exit."""
    return _solve(L.GMRES, A, b, x, M, params)


def fgmres(A: CSRMatrix, b, x, M: Optional[Preconditioner] = None,
           params: Optional[GMRESParams] = None) -> GMRESResult:
    """FGMRES(m), right preconditioning (src/core/fgmres.h:42-47)."""
    return _solve(L.FGMRES, A, b, x, M, params)


def bicgstab(A: CSRMatrix, b, x, M: Optional[Preconditioner] = None,
             params: Optional[GMRESParams] = None) -> GMRESResult:
    """BiCGSTAB, right preconditioning (src/core/bicgstab.h:57-204), FP64.
    params.restart is unused; the reference rule (TOL_REF_ABS) stops on
    ||r|| < tol ||r0||."""
    return _solve(L.BICGSTAB, A, b, x, M, params)


def estimate_condition(A: CSRMatrix, M: Optional[Preconditioner] = None, k: int = 80,
                       seed: int = 42) -> dict:
    """estimate_condition (src/analysis/condition_estimator.h:94-191): k
    Lanczos steps on M^{-1}A on the GPU; extreme Ritz values and kappa."""
    ctx = M.ctx if M is not None else default_context()
    out = L.ConditionEstimate()
    _check(_clib.sg_estimate_condition(ctx.handle, A.device(ctx),
                                       M.handle if M is not None else None, k, seed,
                                       C.byref(out)))
    return dict(lambda_min=out.lambda_min, lambda_max=out.lambda_max, kappa=out.kappa,
                lanczos_steps=out.lanczos_steps, valid=bool(out.valid))


def estimate_spectral_radius(A: CSRMatrix, M: Optional[Preconditioner] = None,
                             max_iter: int = 200, tol: float = 1e-6, seed: int = 123,
                             eigenvector: bool = False) -> dict:
    """estimate_spectral_radius (src/analysis/spectral_analysis.h:30-97):
    power iteration on I - M^{-1}A on the GPU."""
    ctx = M.ctx if M is not None else default_context()
    out = L.SpectralResult()
    ev = np.zeros(A.nrows) if eigenvector else None
    _check(_clib.sg_estimate_spectral_radius(ctx.handle, A.device(ctx),
                                             M.handle if M is not None else None, max_iter,
                                             tol, seed, ev.ctypes.data if ev is not None else None,
                                             C.byref(out)))
    res = dict(spectral_radius=out.spectral_radius, power_iters=out.power_iters,
               convergence_ok=bool(out.convergence_ok))
    if ev is not None:
        res["eigenvector"] = ev
    return res


from .learned import LearnedCorrection, collect_pairs  # noqa: E402  (uses the names above)
from .batched import BatchProblem, make_aniso_batch, solve_batched  # noqa: E402
