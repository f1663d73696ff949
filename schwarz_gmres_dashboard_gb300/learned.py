"""Learned coarse-correction stage for FGMRES + Schwarz (no counterpart in the
reference; its FGMRES, src/core/fgmres.cpp:164-172, accepts any
preconditioner, which is where the stage plugs in).

    stage = LearnedCorrection(96)              # 96^3 grid, 48^3 network grid
    stage.set_matrix(A)
    stage.init_weights(seed=0)
    for seed in fields:                        # plain solves -> training pairs
        collect_pairs(stage, A_seed, M_seed, x_star)
    stage.train(0, stage.num_samples, epochs=30, batch=8, lr=1e-3)
    stage.attach(M, stagnation=0.5)            # z = M v + learned correction
    fgmres(A, b, x, M, GMRESParams(restart=40, tol=1e-8, tol_kind=TOL_TRUE_REL))

Every step (pair restriction, forward, backward, Adam) runs on the GPU
through libsgmres; the stage is nonlinear and is accepted by FGMRES only.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional, Sequence

import numpy as np

from . import _lib as L
from . import (CSRMatrix, Context, GMRESParams, Preconditioner, TOL_TRUE_REL_CYCLE, FP32,
               default_context, fgmres)

_clib = L.load()

NUM_PARAMS = int(_clib.sg_learned_num_params())
CHANNELS = 16
TAPS = 27
LAYERS = 4
LAYER_P = TAPS * CHANNELS * CHANNELS + CHANNELS


def _check(st):
    L.check(st)


class LearnedCorrection:
    """4-layer 3x3x3 CNN (16 channels, ReLU, BF16 weights, FP32 accumulation)
    on the half-resolution grid of an nx^3 grid (nx a multiple of 16)."""

    def __init__(self, nx: int, ny: Optional[int] = None, nz: Optional[int] = None,
                 ctx: Context | None = None):
        self.ctx = ctx or default_context()
        self.nx, self.ny, self.nz = nx, ny or nx, nz or nx
        h = C.c_void_p()
        _check(_clib.sg_learned_create(self.ctx.handle, self.nx, self.ny, self.nz, C.byref(h)))
        self.handle = h
        self.nc = (self.nx // 2) * (self.ny // 2) * (self.nz // 2)
        self._A = None
        self._M = None

    # ---- operator and weights
    def set_matrix(self, A: CSRMatrix) -> None:
        _check(_clib.sg_learned_set_matrix(self.handle, A.device(self.ctx)))
        self._A = A  # the stage keeps A's device copy by pointer

    def init_weights(self, seed: int = 0) -> None:
        _check(_clib.sg_learned_init_weights(self.handle, C.c_uint64(seed)))

    @property
    def weights(self) -> np.ndarray:
        w = np.empty(NUM_PARAMS, np.float32)
        _check(_clib.sg_learned_get_weights(self.handle, w.ctypes.data, NUM_PARAMS))
        return w

    @weights.setter
    def weights(self, w) -> None:
        w = np.ascontiguousarray(w, dtype=np.float32)
        if w.size != NUM_PARAMS:
            raise ValueError(f"expected {NUM_PARAMS} parameters, got {w.size}")
        _check(_clib.sg_learned_set_weights(self.handle, w.ctypes.data, NUM_PARAMS))

    def save(self, path: str) -> None:
        """Raw little-endian float32 weights (the format `schwarz_solve --learned` reads)."""
        self.weights.astype("<f4").tofile(path)

    def load(self, path: str) -> None:
        self.weights = np.fromfile(path, dtype="<f4")

    # ---- training data
    def add_pair(self, M: Preconditioner, r, e) -> None:
        """(residual r = b - A x_k, error e = x* - x_k) of a plain solve."""
        from . import _vec
        n = M.n
        pr, mr, _kr = _vec(r, n)
        pe, me, _ke = _vec(e, n)
        if mr != me:
            raise TypeError("r and e must both be host or both be device arrays")
        _check(_clib.sg_learned_add_pair(self.handle, M.handle, pr, pe, n, mr))

    @property
    def num_samples(self) -> int:
        c = C.c_int(0)
        _check(_clib.sg_learned_num_samples(self.handle, C.byref(c)))
        return c.value

    def clear_samples(self) -> None:
        _check(_clib.sg_learned_clear_samples(self.handle))

    def sample(self, i: int):
        """(input R r1 / s, feature f, target R(e - M r) / s) of stored sample i."""
        a = np.empty(self.nc, np.float32)
        f = np.empty(self.nc, np.float32)
        t = np.empty(self.nc, np.float32)
        _check(_clib.sg_learned_get_sample(self.handle, i, a.ctypes.data, f.ctypes.data,
                                           t.ctypes.data))
        return a, f, t

    def sample_fine(self, i: int):
        """(fine energy target e1 / s, its energy in A, field index) of sample i."""
        n = self.nx * self.ny * self.nz
        err = np.empty(n, np.float32)
        en = np.zeros(1, np.float32)
        fld = np.zeros(1, np.int32)
        _check(_clib.sg_learned_get_sample_fine(self.handle, i, err.ctypes.data, en.ctypes.data,
                                                fld.ctypes.data))
        return err, float(en[0]), int(fld[0])

    # ---- training
    LOSSES = {"energy": 0, "mse": 1}

    def set_loss(self, kind: str) -> None:
        """"energy" (default): ||e1/s - c P y||_A^2 / ||e1/s||_A^2; "mse": coarse MSE."""
        _check(_clib.sg_learned_set_loss(self.handle, self.LOSSES[kind]))

    def sample_gradient(self, first: int, count: int):
        """(loss, parameter gradient) of stored samples [first, first+count) as one batch."""
        g = np.empty(NUM_PARAMS - 1, np.float32)
        loss = C.c_double(0.0)
        _check(_clib.sg_learned_sample_gradient(self.handle, first, count, g.ctypes.data,
                                                C.byref(loss)))
        return loss.value, g

    def train(self, first: int, count: int, epochs: int, batch: int = 8, lr: float = 1e-3,
              seed: int = 0) -> np.ndarray:
        """Adam over samples [first, first+count); returns the mean batch loss
        of every epoch."""
        losses = np.zeros(max(epochs, 1), np.float64)
        _check(_clib.sg_learned_train(self.handle, first, count, epochs, batch, float(lr),
                                      C.c_uint64(seed), losses.ctypes.data))
        return losses[:epochs]

    def eval(self, first: int, count: int) -> float:
        out = C.c_double(0.0)
        _check(_clib.sg_learned_eval(self.handle, first, count, C.byref(out)))
        return out.value

    def forward(self, x: np.ndarray) -> np.ndarray:
        """Network alone: x [batch, nc, 2] float32 -> y [batch, nc]."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        b = x.shape[0]
        if x.shape != (b, self.nc, 2):
            raise ValueError(f"x must be [batch, {self.nc}, 2]")
        y = np.empty((b, self.nc), np.float32)
        _check(_clib.sg_learned_forward(self.handle, x.ctypes.data, b, y.ctypes.data))
        return y

    def gradient(self, x: np.ndarray, t: np.ndarray):
        """(loss, gradient of the network parameters) of mean (y - t)^2."""
        x = np.ascontiguousarray(x, dtype=np.float32)
        t = np.ascontiguousarray(t, dtype=np.float32)
        b = x.shape[0]
        if x.shape != (b, self.nc, 2) or t.shape != (b, self.nc):
            raise ValueError("shape mismatch")
        g = np.empty(NUM_PARAMS - 1, np.float32)
        loss = C.c_double(0.0)
        _check(_clib.sg_learned_gradient(self.handle, x.ctypes.data, t.ctypes.data, b,
                                         g.ctypes.data, C.byref(loss)))
        return loss.value, g

    # ---- use inside FGMRES
    def attach(self, M: Preconditioner, stagnation: float = 0.5) -> None:
        """Apply the stage after M (its applies and FGMRES solves).  The monitor
        falls back to plain M for the rest of a solve when a restart cycle
        reduces the true residual by less than `stagnation` (0: never)."""
        _check(_clib.sg_precond_set_learned(M.handle, self.handle, float(stagnation)))
        self._M = M

    def detach(self) -> None:
        if self._M is not None and getattr(self._M, "handle", None):
            _check(_clib.sg_precond_set_learned(self._M.handle, None, 0.0))
        self._M = None

    @property
    def enabled(self) -> bool:
        return bool(self.state()["enabled"])

    @enabled.setter
    def enabled(self, on: bool) -> None:
        _check(_clib.sg_learned_set_enabled(self.handle, 1 if on else 0))

    def set_wait_test(self, mode: int) -> None:
        """Testing: 1 / 2 make the convolutions' copy / MMA waits give up at
        once (the next call raises SgError with SG_ERR_DEVICE_TIMEOUT); 0
        restores the normal budget."""
        _check(_clib.sg_learned_set_wait_test(self.handle, int(mode)))

    def state(self) -> dict:
        en, fb, ap = C.c_int(0), C.c_int(0), C.c_longlong(0)
        _check(_clib.sg_learned_get_state(self.handle, C.byref(en), C.byref(fb), C.byref(ap)))
        return dict(enabled=en.value, fallback_cycle=fb.value, applies=ap.value)

    def close(self):
        if getattr(self, "handle", None):
            _clib.sg_learned_destroy(self.handle)
            self.handle = None
            self._M = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def collect_pairs(stage: LearnedCorrection, A: CSRMatrix, M: Preconditioner, x_star,
                  snapshots: Sequence[int] = (2, 5, 9, 14, 20, 28),
                  precision: int = FP32) -> int:
    """Training pairs from plain FGMRES solves of A x = A x_star: for every k in
    `snapshots` one restart cycle of k steps from x0 = 0 gives x_k, and the
    pair (b - A x_k, x_star - x_k) is added.  M must not have a learned stage
    attached.  Returns the number of pairs added."""
    if stage._M is M:
        raise ValueError("detach the learned stage from M before collecting plain-solve pairs")
    stage.set_matrix(A)
    x_star = np.ascontiguousarray(x_star, dtype=np.float64)
    b = A.spmv(x_star)
    for k in snapshots:
        x = np.zeros(A.nrows)
        fgmres(A, b, x, M, GMRESParams(restart=int(k), max_iter=int(k), tol=0.0,
                                       tol_kind=TOL_TRUE_REL_CYCLE, precision=precision,
                                       use_graph=False))
        r = b - A.spmv(x)
        stage.add_pair(M, r, x_star - x)
    return len(snapshots)
