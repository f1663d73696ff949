// kernels.h -- host-side launchers of the CUDA kernels of libsgmres.
#pragma once

#include "sg_internal.h"

namespace sg {

// ---------------------------------------------------------------- spmv.cu
// y = scale * (A x) (scale may be null = 1).  `exact` (FP64 only) keeps the
// reference's product/sum rounding and order.  `active`: when non-null and
// *active == 0 the kernel does nothing (finished solve inside a graph).
template <class TV, class TX, class TY>
void launch_spmv(sg_ctx* ctx, int n, const int* rp, const int* ci, const TV* val, const TX* x,
                 TY* y, const double* scale, const int* active);
// Matrix-level SpMV: SELL or CSR as chosen for A (same bits in FP64).
// fp32 selects the FP32 copy of the values (inner Krylov).
template <class TV, class TX, class TY>
void launch_spmv_a(sg_ctx* ctx, const sg_csr* A, const TX* x, TY* y, const double* scale,
                   const int* active);
// Times both formats on A and keeps the faster one (autotuner).
void spmv_autotune(sg_ctx* ctx, sg_csr* A);
// r = b - A x in FP64 with ||r||; the last block updates the solve state
// (rnorm, true-residual convergence test).
void launch_residual(sg_ctx* ctx, const sg_csr* A, const double* b, const double* x, double* r,
                     SolveState* st);
// ||v|| of a FP64 vector into st->bnorm (solve start); flags non-finite input.
void launch_bnorm(sg_ctx* ctx, const double* v, int n, SolveState* st);

// ---------------------------------------------------------------- krylov.cu
// Cycle start: beta = ||raw0||, g = beta e1, vscale[0] = 1/beta, reference
// stopping test on beta.
template <class TV>
void launch_cycle_init(sg_ctx* ctx, const TV* raw0, int n, SolveState* st, int m, bool flexible);
// One CGS2 Arnoldi step on raw[j+1] against raw[0..j] (with the Givens
// update of the least-squares problem done by the last block); lagged: the
// two-pass variant with the second projection carried to the next step
// (st->lagged must be set for the whole solve, m < SG_LAGM).
template <class TV>
void launch_cgs2(sg_ctx* ctx, TV* raw, size_t ldv, int n, int j, int m, SolveState* st,
                 bool lagged);
// y = H^{-1} g (k x k upper triangle) by one thread.
void launch_backsolve(sg_ctx* ctx, SolveState* st, int m);
// x += sum_k y_k * vscale_k * basis_k  (k < st->kcount)
template <class TV>
void launch_update_x(sg_ctx* ctx, const TV* basis, size_t ldv, int n, double* x, SolveState* st);
// y = x with type conversion (no preconditioner)
template <class TI, class TO>
void launch_copy(sg_ctx* ctx, const TI* x, TO* y, int n, const int* active);
// BLAS-1 (src/core/vector.h): dot into device memory, axpy, scale
void launch_dot(sg_ctx* ctx, const double* x, const double* y, int n, double* out_dev);
void launch_axpy(sg_ctx* ctx, double alpha, const double* x, double* y, int n);
void launch_scale(sg_ctx* ctx, double alpha, double* x, int n);
int dot_grid(int num_sms, int n);
// the dot kernel with caller-provided scratch (blocks partial sums) and stream
void launch_dot_scratch(cudaStream_t stream, const double* x, const double* y, int n,
                        int blocks, double* partials, unsigned* counter, double* out_dev);
// cycle bookkeeping after the update: cycles++, out-of-iterations test
void launch_cycle_end(sg_ctx* ctx, SolveState* st);

// ---------------------------------------------------------------- bicgstab.cu
// BiCGSTAB (src/core/bicgstab.h:57-204) on device vectors b, x (x0 on entry)
void solve_bicgstab_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, const double* b,
                           double* x, const sg_solve_params& prm, sg_solve_result* res);
// ---------------------------------------------------------------- analysis.cu
// Lanczos estimate of the extreme eigenvalues of M^{-1}A and power iteration
// on I - M^{-1}A (src/analysis/condition_estimator.h, spectral_analysis.h)
void estimate_condition_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int k,
                               unsigned seed, sg_condition_estimate* out);
void estimate_spectral_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int max_iter,
                              double tol, unsigned seed, double* eigvec_host,
                              sg_spectral_result* out);

// ---------------------------------------------------------------- host_precond.cu
// a caller's host function as preconditioner (kind SG_PC_HOST): set-up, and
// the stream-ordered apply (D2H copy, host function, H2D copy); `scale`
// (device, optional) is the input's scale, applied before the function and
// divided out after it (FGMRES directions)
void host_precond_init(sg_precond* pc, sg_host_apply_fn fn, void* user, int n);
template <class TI, class TO>
void host_precond_apply(sg_precond* pc, const TI* x, TO* y, const int* active,
                        const double* scale);
int host_precond_status(sg_precond* pc);  // first nonzero return since the last read
long long host_precond_calls(const sg_precond* pc);

// ---------------------------------------------------------------- schwarz.cu
void precond_setup_device(sg_precond* pc, const sg_csr* A);
// exact: FP64 sweeps round each product and difference (reference bits);
// otherwise they use fused multiply-adds (the solver's FP64 mode)
template <class TI, class TO>
void precond_apply_device(sg_precond* pc, const TI* x, TO* y, const int* active,
                          bool exact = true);

// ---------------------------------------------------------------- sweep.cu
void rec_setup_device(sg_precond* pc);
template <class TI, class TO>
bool sweep_tma(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse, bool exact,
               const int* active);
// reads the sweeps' error word (0: none) and clears it
int sweep_error(sg_precond* pc);
// four right-hand sides ld apart at once (RAS, FP32 sweeps); false: use four
// single applies
template <class TI, class TO>
bool sweep_tma4(sg_precond* pc, const TI* x, TO* y, long long ld, const int* sub_on);
bool sweep_plan4(sg_precond* pc);  // plans that sweep (outside stream capture)
long long sweep_check(sg_precond* pc, int plant);
// whether sg_precond_set_wait_test's mode applies to this set-up
bool sweep_wait_test_supported(const sg_precond* pc, int mode);
// the TMA sweep computes the coarse restriction itself (no k_restrict launch)
bool sweep_fuses_restrict(const sg_precond* pc);
// ---------------------------------------------------------------- learned.cu
// y += learned correction of the preconditioned vector y = M x (x: the
// vector M was applied to; n: its length, checked against the stage's grid)
template <class TI, class TO>
void learned_apply(sg_learned* L, const TI* x, TO* y, int n, const int* active);
// solve start (stage on, monitor reset) and the per-cycle stagnation monitor
void learned_begin(sg_learned* L, SolveState* st);
void learned_monitor(sg_learned* L, SolveState* st);
void learned_detach(sg_learned* L);
uint64_t learned_gen(const sg_learned* L);  // changes when the stage's matrix changes
int learned_error(sg_learned* L);  // a convolution's bounded wait ran out (read and cleared)

// ---------------------------------------------------------------- batched.cu
// nsys independent systems (block-diagonal A, rows of system s at
// [sys_row_ptr[s], sys_row_ptr[s+1])) x nrhs right-hand sides in the layout
// [rhs][rows]; b and x may be host or device pointers
void solve_batched_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int nsys,
                          const int* sys_row_ptr, int nrhs, const double* b, double* x,
                          const sg_solve_params& prm, sg_batch_result* results, double* time_s);

// copy the FP64 factors of subdomain s back to the host
void precond_read_factors(sg_precond* pc, int s, double* lu_out);
void precond_read_coarse(sg_precond* pc, double* a0_out);

}  // namespace sg
