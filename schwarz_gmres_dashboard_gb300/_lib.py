"""ctypes binding of libsgmres.so (the C ABI of include/sgmres.h).

The library is built in-tree by ``schwarz_gmres_dashboard_gb300.build``; this
module never falls back to anything else: when the shared object is missing
or fails to load, importing the package raises.
"""
from __future__ import annotations

import ctypes as C
import os

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsgmres.so")

SG_OK = 0
STATUS = {0: "SG_OK", 1: "SG_ERR_INVALID_ARG", 2: "SG_ERR_CUDA", 3: "SG_ERR_OOM",
          4: "SG_ERR_SINGULAR", 5: "SG_ERR_NOT_SETUP", 6: "SG_ERR_NONFINITE",
          7: "SG_ERR_DEVICE_TIMEOUT", 8: "SG_ERR_UNSUPPORTED", 9: "SG_ERR_INTERNAL",
          10: "SG_ERR_CALLBACK"}
SG_ERR_CALLBACK = 10

MEM_HOST, MEM_DEVICE = 0, 1
FP64, FP32, BF16 = 0, 1, 2
GMRES, FGMRES, BICGSTAB = 0, 1, 2
TOL_REF_ABS, TOL_TRUE_REL_CYCLE, TOL_TRUE_REL = 0, 1, 2
PC_KINDS = {"none": 0, "jacobi": 1, "ilu0": 2, "asm": 3, "ras": 4,
            "twolevel_asm": 5, "twolevel_ras": 6}


class SgError(RuntimeError):
    """A libsgmres call returned a non-OK status (the reference throws
    std::runtime_error in the same places)."""

    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS.get(status, status)}: {msg}")
        self.status = status


class PrecondOpts(C.Structure):
    _fields_ = [("nparts", C.c_int), ("overlap", C.c_int), ("factor_dtype", C.c_int),
                ("sweep_dtype", C.c_int), ("partition", C.c_void_p),
                ("reserved", C.c_int * 8)]


class SolveParams(C.Structure):
    _fields_ = [("restart", C.c_int), ("max_iter", C.c_int), ("tol", C.c_double),
                ("tol_kind", C.c_int), ("precision", C.c_int), ("use_graph", C.c_int),
                ("history", C.c_void_p), ("history_cap", C.c_int), ("ortho", C.c_int),
                ("reserved", C.c_int * 7)]


class BatchResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("cycles", C.c_int), ("converged", C.c_int),
                ("status", C.c_int), ("true_rel_residual", C.c_double)]


# int fn(void* user, const double* x, double* y, int n)
HOST_APPLY_FN = C.CFUNCTYPE(C.c_int, C.c_void_p, C.POINTER(C.c_double), C.POINTER(C.c_double),
                            C.c_int)


class Convergence(C.Structure):
    _fields_ = [("iterations", C.c_int), ("converged", C.c_int), ("stagnation_start", C.c_int),
                ("reserved", C.c_int), ("initial_residual", C.c_double),
                ("final_residual", C.c_double), ("asymptotic_rate", C.c_double)]


class ConditionEstimate(C.Structure):
    _fields_ = [("lambda_min", C.c_double), ("lambda_max", C.c_double), ("kappa", C.c_double),
                ("lanczos_steps", C.c_int), ("valid", C.c_int)]


class SpectralResult(C.Structure):
    _fields_ = [("spectral_radius", C.c_double), ("power_iters", C.c_int),
                ("convergence_ok", C.c_int)]


class SolveResult(C.Structure):
    _fields_ = [("iterations", C.c_int), ("cycles", C.c_int), ("converged", C.c_int),
                ("history_len", C.c_int), ("residual_norm", C.c_double),
                ("true_rel_residual", C.c_double), ("time_solve_s", C.c_double),
                ("reserved", C.c_double * 4)]


_vp, _ip, _dp = C.c_void_p, C.POINTER(C.c_int), C.POINTER(C.c_double)

# name -> (restype, argtypes)
PROTOTYPES = {
    "sg_abi_version": (C.c_int, []),
    "sg_last_error": (C.c_char_p, []),
    "sg_status_string": (C.c_char_p, [C.c_int]),
    "sg_ctx_create": (C.c_int, [C.c_int, C.POINTER(_vp)]),
    "sg_ctx_destroy": (C.c_int, [_vp]),
    "sg_ctx_set_stream": (C.c_int, [_vp, _vp]),
    "sg_ctx_get_stream": (C.c_int, [_vp, C.POINTER(_vp)]),
    "sg_ctx_synchronize": (C.c_int, [_vp]),
    "sg_ctx_get_launch_count": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "sg_ctx_get_capture_count": (C.c_int, [_vp, C.POINTER(C.c_longlong)]),
    "sg_ctx_set_timing": (C.c_int, [_vp, C.c_int]),
    "sg_ctx_get_timing": (C.c_int, [_vp, C.c_int, _dp, C.POINTER(C.c_longlong)]),
    "sg_csr_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, C.c_int,
                                C.POINTER(_vp)]),
    "sg_csr_destroy": (C.c_int, [_vp]),
    "sg_csr_set_format": (C.c_int, [_vp, C.c_int]),
    "sg_csr_get_format": (C.c_int, [_vp, _ip]),
    "sg_csr_set_spmv_variant": (C.c_int, [_vp, C.c_int]),
    "sg_csr_get_spmv_choice": (C.c_int, [_vp, _ip, _ip, _ip, _ip]),
    "sg_csr_spmv": (C.c_int, [_vp, _vp, _vp, C.c_int]),
    "sg_precond_create": (C.c_int, [_vp, C.c_int, C.POINTER(PrecondOpts), C.POINTER(_vp)]),
    "sg_precond_setup": (C.c_int, [_vp, _vp]),
    "sg_precond_apply": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int]),
    "sg_precond_destroy": (C.c_int, [_vp]),
    "sg_precond_get_decomposition": (C.c_int, [_vp, C.c_int, _vp, C.c_int, _ip]),
    "sg_precond_get_factors": (C.c_int, [_vp, C.c_int, _ip, _ip, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sg_precond_get_coarse": (C.c_int, [_vp, _vp, C.c_int, _ip]),
    "sg_precond_get_sweep": (C.c_int, [_vp, _ip, _ip]),
    "sg_precond_get_sweep_ring": (C.c_int, [_vp, _ip, _ip]),
    "sg_precond_check": (C.c_int, [_vp, C.c_int, C.POINTER(C.c_longlong)]),
    "sg_precond_get_setup_path": (C.c_int, [_vp, _ip]),
    "sg_precond_get_schedule": (C.c_int, [_vp, C.c_int, C.c_void_p, C.c_longlong,
                                          C.POINTER(C.c_longlong)]),
    "sg_precond_set_wait_test": (C.c_int, [_vp, C.c_int]),
    "sg_precond_create_host": (C.c_int, [_vp, _vp, _vp, C.c_int, C.POINTER(_vp)]),
    "sg_estimate_condition": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_uint,
                                        C.POINTER(ConditionEstimate)]),
    "sg_estimate_spectral_radius": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_double, C.c_uint, _vp,
                                              C.POINTER(SpectralResult)]),
    "sg_read_matrix_market": (C.c_int, [C.c_char_p, _ip, _ip, _ip, _vp, _vp, _vp, C.c_int]),
    "sg_convergence_metrics": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _vp]),
    "sg_write_convergence_jsonl": (C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int,
                                             C.c_int, _vp, C.c_int, C.c_int]),
    "sg_solve": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp, _vp, C.c_int, C.c_int,
                           C.POINTER(SolveParams), C.POINTER(SolveResult)]),
    "sg_solve_batched": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, C.c_int, _vp, _vp, C.c_int,
                                   C.POINTER(SolveParams), _vp, _dp]),
    "sg_dot": (C.c_int, [_vp, _vp, _vp, C.c_int, C.c_int, _dp]),
    "sg_norm2": (C.c_int, [_vp, _vp, C.c_int, C.c_int, _dp]),
    "sg_axpy": (C.c_int, [_vp, C.c_double, _vp, _vp, C.c_int, C.c_int]),
    "sg_scale": (C.c_int, [_vp, C.c_double, _vp, C.c_int, C.c_int]),
    "sg_dot_noalloc": (C.c_int, [_vp, _vp, C.c_int, _vp, _vp]),
    "sg_gen_poisson2d": (C.c_int, [C.c_int, C.c_int, _vp, _vp, _vp, _ip]),
    "sg_gen_poisson3d": (C.c_int, [C.c_int, C.c_int, C.c_int, _vp, _vp, _vp, _ip]),
    "sg_gen_varcoef3d": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_uint64, _vp, _vp, _vp, _ip]),
    "sg_gen_uniform": (C.c_int, [C.c_uint64, C.c_int, C.c_double, C.c_double, _vp]),
    "sg_gen_aniso2d": (C.c_int, [C.c_int, C.c_int, C.c_double, C.c_double, _vp, _vp, _vp, _ip]),
    "sg_partition_graph": (C.c_int, [C.c_int, _vp, _vp, C.c_int, _vp]),
    "sg_partition_boxes": (C.c_int, [C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                     C.c_uint64, _vp]),
    "sg_schwarz_structure": (C.c_int, [C.c_int, _vp, _vp, _vp, C.c_int, C.c_int, C.c_int, _vp,
                                       C.c_int, _ip]),
    "sg_learned_num_params": (C.c_int, []),
    "sg_learned_create": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.POINTER(_vp)]),
    "sg_learned_destroy": (C.c_int, [_vp]),
    "sg_learned_set_matrix": (C.c_int, [_vp, _vp]),
    "sg_learned_init_weights": (C.c_int, [_vp, C.c_uint64]),
    "sg_learned_set_weights": (C.c_int, [_vp, _vp, C.c_int]),
    "sg_learned_get_weights": (C.c_int, [_vp, _vp, C.c_int]),
    "sg_learned_add_pair": (C.c_int, [_vp, _vp, _vp, _vp, C.c_int, C.c_int]),
    "sg_learned_num_samples": (C.c_int, [_vp, _ip]),
    "sg_learned_clear_samples": (C.c_int, [_vp]),
    "sg_learned_get_sample": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "sg_learned_get_sample_fine": (C.c_int, [_vp, C.c_int, _vp, _vp, _vp]),
    "sg_learned_set_loss": (C.c_int, [_vp, C.c_int]),
    "sg_learned_sample_gradient": (C.c_int, [_vp, C.c_int, C.c_int, _vp, _dp]),
    "sg_learned_train": (C.c_int, [_vp, C.c_int, C.c_int, C.c_int, C.c_int, C.c_double,
                                   C.c_uint64, _vp]),
    "sg_learned_eval": (C.c_int, [_vp, C.c_int, C.c_int, _dp]),
    "sg_learned_forward": (C.c_int, [_vp, _vp, C.c_int, _vp]),
    "sg_learned_gradient": (C.c_int, [_vp, _vp, _vp, C.c_int, _vp, _dp]),
    "sg_learned_set_enabled": (C.c_int, [_vp, C.c_int]),
    "sg_learned_set_wait_test": (C.c_int, [_vp, C.c_int]),
    "sg_learned_get_state": (C.c_int, [_vp, _ip, _ip, C.POINTER(C.c_longlong)]),
    "sg_precond_set_learned": (C.c_int, [_vp, _vp, C.c_double]),
}

_lib = None


def load(path: str = LIB_PATH):
    """Load libsgmres.so and bind every prototype.  Raises when it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(path):
        raise ImportError(
            f"libsgmres.so not found at {path}; build it with "
            "`python -m schwarz_gmres_dashboard_gb300.build` (needs nvcc)")
    lib = C.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != SG_OK:
        msg = _lib.sg_last_error().decode(errors="replace") if _lib else ""
        raise SgError(status, msg)
