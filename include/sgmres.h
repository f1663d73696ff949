/*
 * sgmres.h -- C ABI of libsgmres.so, the GB300 (sm_103a) solve path of
 * schwarz-gmres: restarted GMRES(m) / FGMRES preconditioned by Jacobi,
 * ILU(0), one-level ASM/RAS and two-level Schwarz with ILU(0) subdomain
 * solves, all resident on one GPU.
 *
 * Conventions
 *  - Every entry point returns sg_status; on failure sg_last_error() returns a
 *    thread-local message (the reference throws std::runtime_error instead:
 *    src/gpu/cuda_common.h:13-40, src/precond/coarse_solve.h:31-32,
 *    src/decomp/domain_decomp.h:54-55).
 *  - Indices are 0-based int32, values FP64, CSR column indices ascending
 *    within a row (as src/core/sparse_matrix.h:13-18 and every reference
 *    generator produce them).
 *  - Vectors passed with SG_MEM_HOST are host pointers (copied in/out inside
 *    the call); with SG_MEM_DEVICE they are device pointers on the context's
 *    device, used in place on the context's stream.
 *  - No entry point falls back to the CPU: without a usable CUDA device the
 *    calls that compute return SG_ERR_CUDA.
 */
#ifndef SGMRES_H
#define SGMRES_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SG_ABI_VERSION 1

typedef enum sg_status {
    SG_OK = 0,
    SG_ERR_INVALID_ARG = 1, /* bad size, pointer, option or CSR structure */
    SG_ERR_CUDA = 2,        /* CUDA runtime failure or no device */
    SG_ERR_OOM = 3,         /* device allocation failed */
    SG_ERR_SINGULAR = 4,    /* coarse matrix singular, missing ILU diagonal */
    SG_ERR_NOT_SETUP = 5,   /* preconditioner used before sg_precond_setup */
    SG_ERR_NONFINITE = 6,   /* NaN/Inf in the right-hand side or the iteration */
    SG_ERR_DEVICE_TIMEOUT = 7, /* a bounded device wait gave up */
    SG_ERR_UNSUPPORTED = 8, /* option combination not provided */
    SG_ERR_INTERNAL = 9,
    SG_ERR_CALLBACK = 10    /* a host preconditioner function returned nonzero */
} sg_status;

typedef enum sg_mem { SG_MEM_HOST = 0, SG_MEM_DEVICE = 1 } sg_mem;

/* Preconditioners of the reference CLI (src/main.cpp:44, :190-208). */
typedef enum sg_precond_kind {
    SG_PC_NONE = 0,
    SG_PC_JACOBI = 1,       /* src/precond/jacobi.h:10-27 */
    SG_PC_ILU0 = 2,         /* src/precond/ilu0.h:11-93 */
    SG_PC_ASM = 3,          /* src/precond/asm.h:13-71 */
    SG_PC_RAS = 4,          /* src/precond/ras.h:16-82 */
    SG_PC_TWOLEVEL_ASM = 5, /* src/precond/two_level_schwarz.h:23-75, FineLevelType::ASM */
    SG_PC_TWOLEVEL_RAS = 6, /* src/precond/two_level_schwarz.h:23-75, FineLevelType::RAS */
    SG_PC_HOST = 7          /* a caller's host function (sg_precond_create_host only) */
} sg_precond_kind;

/* Arithmetic / storage types. */
typedef enum sg_dtype { SG_FP64 = 0, SG_FP32 = 1, SG_BF16 = 2 } sg_dtype;

typedef struct sg_precond_opts {
    int nparts;        /* subdomains (reference default 4, src/main.cpp:75) */
    int overlap;       /* overlap layers (reference default 1, src/main.cpp:74) */
    int factor_dtype;  /* storage of ILU factors: SG_FP64, SG_FP32 or SG_BF16 */
    int sweep_dtype;   /* triangular sweeps: SG_FP64 or SG_FP32 (FP32 accumulate) */
    const int* partition; /* optional host array [n] of part ids in [0,nparts);
                             NULL = built-in graph partitioner. Takes the place
                             of METIS_PartGraphKway (src/decomp/domain_decomp.h:23-58) */
    int reserved[8];  /* reserved[0]: sweep variant (testing/comparison): 0 the
                         TMA-fed level sweep, 1 a level sweep reading factors
                         from global memory, 4 the sync-free sweep (per-row
                         ready flags); reserved[1]: threads per CTA of the
                         TMA-fed sweep (32, 64, 128, 256, 384 or 512; 0 =
                         the fastest of 128-512, timed at set-up);
                         reserved[2]: two-level
                         preconditioners compute the coarse restriction
                         inside the TMA-fed sweep when all subdomains' CTAs
                         fit on the GPU at once (0), or in a kernel of its
                         own (1; same results); reserved[3]: largest group
                         of level records the TMA-fed sweep copies at once
                         (0 = 8 or 16 KB, timed at set-up, else a multiple
                         of 16 in [1024, 65536]; same results); reserved[4]:
                         launch shape of the TMA-fed sweep (0 = timed, 1 one
                         CTA per subdomain, 2 persistent: resident CTAs take
                         subdomains largest first from a work counter, k > 2
                         persistent with k CTAs at most; same results);
                         reserved[5]: integer set-up (decomposition,
                         overlap, local matrices, level schedules) on the
                         device (0; host threads when its bitmaps would not
                         fit) or on host threads (1); same results; other
                         entries must be 0 */
} sg_precond_opts;

typedef struct sg_ctx sg_ctx;
typedef struct sg_csr sg_csr;
typedef struct sg_precond sg_precond;

/* ---- context / errors ------------------------------------------------- */
int sg_abi_version(void);
const char* sg_last_error(void);
const char* sg_status_string(sg_status st);
/* Replaces CudaHandles::init (src/gpu/cuda_common.h:48-56): a device, one
 * stream, no library handles. */
sg_status sg_ctx_create(int device, sg_ctx** out);
sg_status sg_ctx_destroy(sg_ctx* ctx);
/* Run all work of this context on an existing cudaStream_t (NULL = the
 * context's own stream). */
sg_status sg_ctx_set_stream(sg_ctx* ctx, void* cuda_stream);
sg_status sg_ctx_get_stream(sg_ctx* ctx, void** cuda_stream);
sg_status sg_ctx_synchronize(sg_ctx* ctx);
/* Kernels launched through this context so far (a CUDA-graph launch adds
 * the kernel nodes it replays).  No counterpart in the reference. */
sg_status sg_ctx_get_launch_count(sg_ctx* ctx, long long* count);
/* Restart cycles captured as a CUDA graph so far.  A solve reuses the
 * previous capture when the matrix, preconditioner (and its learned stage),
 * vectors, restart length and precision are the same objects in the same
 * state; a re-set-up, format change or new buffer captures again.  No
 * counterpart in the reference. */
sg_status sg_ctx_get_capture_count(sg_ctx* ctx, long long* count);
/* Kernel-class timers: with timing on, solves that run without a CUDA graph
 * record a CUDA event pair on the context stream around every kernel class:
 * kind 0 Krylov SpMV, 1 FP64 residual, 2 preconditioner, 3 orthogonalisation
 * (CGS2 passes, Givens), 4 back-solve and update, 5 the learned stage (also
 * counted inside kind 2).  get_timing returns the
 * accumulated milliseconds and the number of timed launches of a kind.
 * Turning timing on resets the sums.  No counterpart in the reference. */
sg_status sg_ctx_set_timing(sg_ctx* ctx, int on);
sg_status sg_ctx_get_timing(sg_ctx* ctx, int kind, double* ms, long long* count);

/* ---- matrix ----------------------------------------------------------- */
/* Copies a CSR matrix to the device (CSRMatrix, src/core/sparse_matrix.h:13-28;
 * DeviceCSRMatrix::upload, src/gpu/cuda_sparse.h:15-51). Arrays are host or
 * device pointers per `mem`. */
sg_status sg_csr_create(sg_ctx* ctx, int nrows, int ncols, int nnz, const int* row_ptr,
                        const int* col_idx, const double* vals, sg_mem mem, sg_csr** out);
sg_status sg_csr_destroy(sg_csr* A);
/* SpMV storage used by this matrix: 0 = decided by the autotuner on first
 * use (times every available format, keeps the fastest), 1 = CSR,
 * 2 = SELL-C-sigma (C = 32), 3 = SELL-32 with 16-bit column offsets from the
 * row (when every |column - row| <= 32767).  All give the same bits.  No counterpart in the reference (cuSPARSE's
 * CUSPARSE_SPMV_ALG_DEFAULT, src/gpu/cuda_sparse.h:64-68, has no choice). */
sg_status sg_csr_set_format(sg_csr* A, int format);
/* Forces one SELL launch variant of the autotuner's set (testing and
 * comparison): column width, resident blocks, grid and the software-pipelined
 * kernel; SG_ERR_UNSUPPORTED when the matrix does not allow it. */
sg_status sg_csr_set_spmv_variant(sg_csr* A, int variant);
/* The autotuner's choice: format and SELL launch variant (-1: default) for
 * the FP64 values and for the FP32 copy (0 until the first solve or SpMV). */
sg_status sg_csr_get_spmv_choice(sg_csr* A, int* format, int* variant, int* format32,
                                 int* variant32);
sg_status sg_csr_get_format(sg_csr* A, int* format);
/* y = A x (CSRMatrix::spmv, src/core/sparse_matrix.h:30-37; replaces
 * DeviceCSRMatrix::spmv, src/gpu/cuda_sparse.h:53-74). FP64, same summation
 * order as the reference row loop. */
sg_status sg_csr_spmv(sg_csr* A, const double* x, double* y, sg_mem mem);

/* ---- preconditioner plugin (src/precond/preconditioner.h:7-20) ------- */
sg_status sg_precond_create(sg_ctx* ctx, sg_precond_kind kind, const sg_precond_opts* opts,
                            sg_precond** out);
/* Preconditioner::setup(const CSRMatrix&).  A second set-up with a matrix of
 * the same sparsity pattern (and the same partition and options) keeps the
 * host integer set-up (decomposition, local structures, level schedules) and
 * redoes only the device factorisation -- e.g. a new coefficient field. */
sg_status sg_precond_setup(sg_precond* pc, const sg_csr* A);
/* Preconditioner::apply(const double* x, double* y, int n) const:
 * overwrites all of y with M^{-1} x. */
sg_status sg_precond_apply(sg_precond* pc, const double* x, double* y, int n, sg_mem mem);
sg_status sg_precond_destroy(sg_precond* pc);

/* Read back set-up data for parity checks (host arrays).
 * which: 0 partition[n], 1 owned_ptr[P+1], 2 owned[n], 3 sub_ptr[P+1],
 *        4 sub[sum n_s], 5 ownloc_ptr[P+1], 6 ownloc[n]
 * (DomainDecomposition, src/decomp/domain_decomp.h:12-20; RASPrecond::
 * owned_local_indices_, src/precond/ras.h:34-41).  Returns the length in
 * *len; out may be NULL to query the length. */
sg_status sg_precond_get_decomposition(sg_precond* pc, int which, int* out, int cap, int* len);
/* ILU(0) factors of subdomain s as computed on the device, in the local CSR
 * layout of ILU0Precond (src/precond/ilu0.h:81-85): row_ptr[n_s+1],
 * col_idx[nnz_s], lu_vals[nnz_s] (FP64), diag_ptr[n_s]; plus the forward and
 * backward sweep level of every local row.  Any array may be NULL. */
sg_status sg_precond_get_factors(sg_precond* pc, int s, int* n_s, int* nnz_s, int* row_ptr,
                                 int* col_idx, double* lu_vals, int* diag_ptr,
                                 int* level_lower, int* level_upper);
/* Coarse operator A0 (P x P, row-major) of a two-level preconditioner as
 * built on the device (CoarseSpace::A0, src/precond/coarse_space.h:43-60). */
sg_status sg_precond_get_coarse(sg_precond* pc, double* a0, int cap, int* nc);
/* The subdomain sweep the set-up chose (ILU0Precond::apply's triangular
 * solves, src/precond/ilu0.h:54-79, run per subdomain): *sweep 0 TMA-fed
 * level records, 1 a barrier per level, 2 sync-free, -1 none (Jacobi);
 * *threads the threads per CTA of the TMA-fed sweep (0 otherwise).  Either
 * pointer may be NULL. */
sg_status sg_precond_get_sweep(sg_precond* pc, int* sweep, int* threads);
/* Bytes of the TMA-fed sweep's shared-memory record ring and the largest
 * group of level records it copies at once (0 and 0 without that sweep;
 * no counterpart in the reference).  Either pointer may be NULL. */
sg_status sg_precond_get_sweep_ring(sg_precond* pc, int* ring_bytes, int* group_bytes);
/* Checked mode of the TMA-fed sweep (no counterpart in the reference, which
 * has no debug checks): reads the level records back and checks on the host
 * what bounds asserts in the kernel would -- every row and column slot inside
 * the subdomain's shared vector, every column computed by an earlier level
 * of its sweep, every record inside its ring group and the ring, every group
 * issued before the level that waits for it and never over bytes or an
 * mbarrier still in use.  *violations = 0 when all hold.  plant = 1 (tests
 * of the check) first corrupts one column slot of the host copy.  0
 * violations and SG_OK without that sweep. */
sg_status sg_precond_check(sg_precond* pc, int plant, long long* violations);
/* Where the integer set-up of the last sg_precond_setup ran (no
 * counterpart in the reference, which sets up on the host): *on_device 1
 * for the device kernels, 0 for host threads. */
sg_status sg_precond_get_setup_path(sg_precond* pc, int* on_device);
/* Read-back of the subdomain schedule the set-up built (no counterpart in
 * the reference; for tests and inspection): which 0/1 level pointers of the
 * forward/backward sweeps (per subdomain nlev + 1 entries, concatenated),
 * 2/3 rows in level order, 4 slot-layout shift per subdomain, 5 global entry
 * of every local entry, 6 local row pointers (n_s + 1 per subdomain), 7
 * diagonal entry per local row, 8 local columns, 9/10 forward/backward level
 * per local row, 11 per subdomain (lower width, upper width, forward levels,
 * backward levels), 12 launch order of the subdomains.  out may be NULL to
 * query *len. */
sg_status sg_precond_get_schedule(sg_precond* pc, int which, int* out, long long cap,
                                  long long* len);

/* A preconditioner that is a caller's host function: FGMRES's flexible apply
 * (FlexApply / fgmres_flex, src/core/fgmres.h:37, src/core/fgmres.cpp:164-172)
 * and any Preconditioner plugin that is not one of the GPU kinds
 * (src/precond/preconditioner.h:7-20).  fn(user, x, y, n) must write all of
 * y = M^{-1} x (host arrays of n doubles) and return 0, or nonzero to report
 * an error (the call then returns SG_ERR_CALLBACK).  Inside sg_solve the
 * function runs in stream order on a CUDA host-function thread (between a
 * device-to-host and a host-to-device copy of pinned buffers, so a restart
 * cycle with it still runs without host synchronisation and may be replayed
 * as a CUDA graph): it must not call CUDA itself.  FGMRES applies it to the
 * normalised basis vector, as the reference does.  The object is set up on
 * creation (n rows) and is used with SG_GMRES, SG_FGMRES, SG_BICGSTAB,
 * sg_precond_apply and the analysis calls; the batched solver rejects it. */
typedef int (*sg_host_apply_fn)(void* user, const double* x, double* y, int n);
sg_status sg_precond_create_host(sg_ctx* ctx, sg_host_apply_fn fn, void* user, int n,
                                 sg_precond** out);

/* Test hook of the bounded device waits (no counterpart in the reference).
 * mode 1: the TMA-fed sweep copies no subdomain's first level-record group,
 * so every CTA's first record wait runs out after ~1 ms; mode 2: no CTA
 * counts its coarse restriction, so the wait of the sweep's fused
 * restriction runs out after ~1 ms (two-level preconditioners whose sweep
 * computes the restriction itself).  Either way each CTA drains the copies
 * it did issue and returns without writing y; sg_precond_apply and sg_solve
 * then return SG_ERR_DEVICE_TIMEOUT, and the error state is cleared for the
 * next call.  mode 0 restores the normal waits (~1 s budget).
 * SG_ERR_UNSUPPORTED when this set-up has no such wait. */
sg_status sg_precond_set_wait_test(sg_precond* pc, int mode);

/* ---- solvers ---------------------------------------------------------- */
typedef enum sg_solver {
    SG_GMRES = 0, /* left preconditioned, src/core/gmres.cpp:34-160 */
    SG_FGMRES = 1, /* right preconditioned storing V and Z, src/core/fgmres.cpp:28-144 */
    /* right preconditioned BiCGSTAB, src/core/bicgstab.h:57-204 (FP64; restart
     * is unused; SG_TOL_REF_ABS is the reference rule ||r|| < tol ||r0|| on the
     * recursive residual; the true-residual kinds restart from the current x
     * while ||b - A x|| / ||b|| > tol and iterations remain) */
    SG_BICGSTAB = 2
} sg_solver;

typedef enum sg_tol_kind {
    /* the reference rule: stop when |g_{j+1}| < tol (the preconditioned
     * residual for GMRES, src/core/gmres.cpp:318; unpreconditioned for FGMRES,
     * src/core/fgmres.cpp:170), or when the cycle-start norm < tol */
    SG_TOL_REF_ABS = 0,
    /* FP64 true relative residual ||b-Ax||/||b|| <= tol, checked at every
     * restart only (the cycle granularity of the oracle harness) */
    SG_TOL_TRUE_REL_CYCLE = 1,
    /* FP64 true relative residual <= tol; a cycle stops early once the
     * Arnoldi estimate says so, and the restart recomputes b-Ax in FP64 */
    SG_TOL_TRUE_REL = 2
} sg_tol_kind;

typedef struct sg_solve_params {
    int restart;     /* m (GMRESParams::restart, default 30) */
    int max_iter;    /* GMRESParams::max_iter (default 1000) */
    double tol;      /* GMRESParams::tol (default 1e-10) */
    int tol_kind;    /* sg_tol_kind */
    int precision;   /* SG_FP64: all-FP64 Krylov; SG_FP32: FP32 inner Krylov
                        with FP64 true residual, update and least squares
                        (GMRES-IR); the preconditioner uses its own dtypes */
    int use_graph;   /* 1: launch each restart cycle as a CUDA graph */
    double* history; /* optional host array receiving |g_{j+1}| per iteration */
    int history_cap;
    /* orthogonalisation of the Arnoldi step (the reference uses modified
     * Gram-Schmidt, src/core/gmres.cpp:288-292): 0 = CGS2 in the fewest
     * streaming passes -- two (second projection deferred by one step) when
     * the cycle's operator is linear (GMRES, restart < 32), else three;
     * 1 = classic CGS2, three passes per step */
    int ortho;
    int reserved[7];
} sg_solve_params;

typedef struct sg_solve_result {
    int iterations;           /* GMRESResult::iterations */
    int cycles;
    int converged;            /* GMRESResult::converged */
    int history_len;
    double residual_norm;     /* GMRESResult::residual_norm (last |g_{j+1}|) */
    double true_rel_residual; /* ||b - A x||_2 / ||b||_2 in FP64 at exit */
    double time_solve_s;      /* GMRESResult::time_solve_s */
    double reserved[4];
} sg_solve_result;

/* gmres()/fgmres() (src/core/gmres.h:28-33, src/core/fgmres.h:42-47).
 * x holds x0 on entry and the solution on exit.  pc may be NULL. */
sg_status sg_solve(sg_ctx* ctx, sg_solver solver, const sg_csr* A, sg_precond* pc,
                   const double* b, double* x, int n, sg_mem mem,
                   const sg_solve_params* params, sg_solve_result* result);

/* ---- batched solve ---------------------------------------------------- */
/* No single reference counterpart (its benches loop over problems,
 * bench/*.cpp).  nsys independent systems of uneven sizes stacked as one
 * block-diagonal A (rows of system s at [sys_row_ptr[s], sys_row_ptr[s+1]),
 * no entry outside its system's block), each with nrhs right-hand sides: b
 * and x are [nrhs][n] (n = rows of A), host or device pointers per `mem`, x
 * holding x0 on entry.  Every (system, rhs) pair i = rhs * nsys + s is an
 * independent left-preconditioned GMRES(restart <= 32) with its own Krylov
 * space and stopping test (params as sg_solve; default restart 30, tol 1e-8,
 * SG_TOL_TRUE_REL, SG_FP32 basis, graph on).  pc (may be NULL) is set up on A
 * with a partition whose parts each lie inside one system, so one set-up and
 * one sweep launch serve every subdomain of every system.  results (optional,
 * nsys*nrhs entries) receive each pair's outcome; time_s the wall time. */
typedef struct sg_batch_result {
    int iterations;
    int cycles;
    int converged;
    int status;               /* SG_OK or SG_ERR_NONFINITE */
    double true_rel_residual; /* FP64 ||b - A x|| / ||b|| at exit */
} sg_batch_result;
sg_status sg_solve_batched(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int nsys,
                           const int* sys_row_ptr, int nrhs, const double* b, double* x,
                           sg_mem mem, const sg_solve_params* params, sg_batch_result* results,
                           double* time_s);

/* ---- analysis (the reference CLI's --analyze, src/main.cpp:213-224) ---- */
/* ConditionEstimate (src/analysis/condition_estimator.h:32-38). */
typedef struct sg_condition_estimate {
    double lambda_min;
    double lambda_max;
    double kappa;      /* lambda_max / lambda_min (1e30 when |lambda_min| <= 1e-14) */
    int lanczos_steps; /* 0: no estimate */
    int valid;         /* lambda_min > 0 (meaningful for an SPD operator) */
} sg_condition_estimate;
/* estimate_condition (condition_estimator.h:94-191): k Lanczos steps on
 * M^{-1}A (A when pc is NULL) from the reference's seeded start vector, the
 * extreme eigenvalues of the tridiagonal.  k <= 1024. */
sg_status sg_estimate_condition(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int k,
                                unsigned seed, sg_condition_estimate* out);
/* SpectralResult (src/analysis/spectral_analysis.h:21-27). */
typedef struct sg_spectral_result {
    double spectral_radius; /* rho(I - M^{-1}A) */
    int power_iters;
    int convergence_ok;     /* rho < 1 */
} sg_spectral_result;
/* estimate_spectral_radius (spectral_analysis.h:30-97): power iteration on
 * I - M^{-1}A until the Rayleigh quotient changes by less than
 * tol (1 + |mu|); eigenvector (optional host array [n]) receives the last
 * normalised iterate. */
sg_status sg_estimate_spectral_radius(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int max_iter,
                                      double tol, unsigned seed, double* eigenvector,
                                      sg_spectral_result* out);

/* ---- BLAS-1 (src/core/vector.h:11-44) --------------------------------- */
/* dot (vector.h:11-16), FP64, deterministic order (block partial sums added
 * in block order); the value is returned to the host in *result. */
sg_status sg_dot(sg_ctx* ctx, const double* x, const double* y, int n, sg_mem mem,
                 double* result);
/* norm2 (vector.h:23-25) = sqrt(dot(x, x)) */
sg_status sg_norm2(sg_ctx* ctx, const double* x, int n, sg_mem mem, double* result);
/* axpy y += alpha x (vector.h:31-34), same bits as the reference loop */
sg_status sg_axpy(sg_ctx* ctx, double alpha, const double* x, double* y, int n, sg_mem mem);
/* scale x *= alpha (vector.h:40-44), same bits as the reference loop */
sg_status sg_scale(sg_ctx* ctx, double alpha, double* x, int n, sg_mem mem);

/* ---- allocation-free dot product -------------------------------------- */
/* No counterpart in the reference.  For callers that cannot allocate device
 * memory when they need a reduction: plug-ins hosted by an application that
 * owns all device memory through its own pool and forbids raw cudaMalloc,
 * and real-time loops that cannot pay cudaMalloc's latency or cudaFree's
 * device-wide synchronisation.  (sg_dot takes its scratch from an sg_ctx,
 * whose creation allocates.)
 * Computes *result = dot(x, y) like sg_dot, but takes its per-block partial
 * sums from a fixed 64 KiB array inside the library instead of a context,
 * needs no sg_ctx, and calls no allocator.  x, y and result are device
 * pointers on the current device; the kernel runs on `stream` (NULL: the
 * default stream) and the call does not wait for it.
 * Limits: n <= SG_DOT_NOALLOC_MAX_N, else SG_ERR_INVALID_ARG and nothing runs.
 * All calls on a device share the array: calls whose kernels overlap on the
 * GPU race and return wrong sums.  The first call on a device (with that
 * device current) looks up the array's device address and keeps it for the
 * life of the process; make that first call before any stream capture, and
 * do not call the function again after cudaDeviceReset on that device. */
#define SG_DOT_NOALLOC_MAX_N 33554432
sg_status sg_dot_noalloc(const double* x, const double* y, int n, double* result, void* stream);

/* ---- learned coarse-correction stage ---------------------------------- */
/* No counterpart in the reference (its FGMRES accepts any preconditioner,
 * src/core/fgmres.cpp:164-172, which is where this stage plugs in).
 * Attached to a Schwarz preconditioner M, an apply becomes
 *   z1 = M v;  r1 = v - A z1;  s = rms(R r1);
 *   z  = z1 + s * c * P(CNN([R r1 / s, f]))
 * with R the mean over 2x2x2 cells (an nx^3 grid, nx a multiple of 16, to
 * (nx/2)^3), f the standardised restricted log A_ii, CNN four 3x3x3
 * convolutions with 16 channels and ReLU (BF16 weights and activations,
 * FP32 accumulation, tensor cores), c an output scale and P cell-centred
 * trilinear prolongation.  The stage is nonlinear: sg_solve accepts it with
 * SG_FGMRES only.  After every restart cycle a device monitor switches it
 * off for the rest of the solve when the cycle reduced the FP64 true
 * residual by less than the stagnation ratio (the plain M is the fallback).
 *
 * Parameters: sg_learned_num_params() floats = 4 layers x (27*16*16 weights
 * in [tap][c_in][c_out] order, tap = (dz+1)*9 + (dy+1)*3 + (dx+1), then 16
 * biases), then c.  Padded channels (inputs 2-15 of layer 1, outputs 1-15 of
 * layer 4) are kept at 0. */
typedef struct sg_learned sg_learned;
int sg_learned_num_params(void);
sg_status sg_learned_create(sg_ctx* ctx, int nx, int ny, int nz, sg_learned** out);
/* Detaches it from its preconditioner first. */
sg_status sg_learned_destroy(sg_learned* L);
/* The operator of the residual r1 and the source of the feature f; kept by
 * pointer (it must outlive its use by the stage). */
sg_status sg_learned_set_matrix(sg_learned* L, const sg_csr* A);
/* Seeded He-uniform initialisation (last layer x0.1); resets Adam. */
sg_status sg_learned_init_weights(sg_learned* L, uint64_t seed);
sg_status sg_learned_set_weights(sg_learned* L, const float* w, int count);
sg_status sg_learned_get_weights(sg_learned* L, float* w, int count);
/* Training pair from a plain solve: residual r = b - A x_k and error
 * e = x* - x_k.  Stores on the device the input R r1 / s, the feature f, the
 * coarse target R(e1) / s and the fine target e1 / s with e1 = e - M r (M: pc
 * without any learned stage), and the current matrix's FP32 values once per
 * sg_learned_set_matrix (every pair's matrix must share one pattern). */
sg_status sg_learned_add_pair(sg_learned* L, sg_precond* pc, const double* r, const double* e,
                              int n, sg_mem mem);
sg_status sg_learned_num_samples(sg_learned* L, int* count);
sg_status sg_learned_clear_samples(sg_learned* L);
/* Copies stored sample i (each array nc = (nx/2)^3 floats; NULL skips). */
sg_status sg_learned_get_sample(sg_learned* L, int i, float* input, float* feature,
                                float* target);
/* Fine-grid data of stored sample i: the energy target e1 / s (n floats),
 * its energy (e1/s)^T A (e1/s) and the index of its field (NULL skips). */
sg_status sg_learned_get_sample_fine(sg_learned* L, int i, float* err, float* energy, int* field);
/* Training loss: 0 (default) the energy norm of the field's A,
 *   mean over samples of ||e1/s - c P y||_A^2 / ||e1/s||_A^2;
 * 1 the mean squared error between y and the coarse target / c. */
sg_status sg_learned_set_loss(sg_learned* L, int kind);
/* Loss and parameter gradient of the current network over stored samples
 * [first, first+count) as one batch (count <= 64). */
sg_status sg_learned_sample_gradient(sg_learned* L, int first, int count, float* grad,
                                     double* loss);
/* Adam (lr, betas 0.9/0.999, eps 1e-8) on the training loss over samples
 * [first, first+count), in shuffled mini-batches (SplitMix64(seed)
 * Fisher-Yates per epoch); sets c to the rms of those samples' coarse
 * targets first.  epoch_loss (optional) receives the mean batch loss of
 * every epoch. */
sg_status sg_learned_train(sg_learned* L, int first, int count, int epochs, int batch, double lr,
                           uint64_t seed, double* epoch_loss);
/* Mean loss of the current network over samples [first, first+count). */
sg_status sg_learned_eval(sg_learned* L, int first, int count, double* loss);
/* The network alone on host inputs x [batch][nc][2] (channel-last FP32,
 * rounded to BF16 on the device): y [batch][nc]. */
sg_status sg_learned_forward(sg_learned* L, const float* x, int batch, float* y);
/* loss = mean over batch*nc of (y - t)^2 and its gradient with respect to the
 * network parameters (grad: sg_learned_num_params() - 1 floats). */
sg_status sg_learned_gradient(sg_learned* L, const float* x, const float* t, int batch,
                              float* grad, double* loss);
/* Switch the stage on/off for later applies and solves. */
sg_status sg_learned_set_enabled(sg_learned* L, int on);
/* Testing of the bounded device waits: mode 1 (2) makes every convolution's
 * wait for its halo copies (for its tensor-core MMAs) impossible to satisfy
 * with a ~1 ms budget; the kernel drains what is in flight, leaves its tile
 * unwritten and the call returns SG_ERR_DEVICE_TIMEOUT.  0: normal waits. */
sg_status sg_learned_set_wait_test(sg_learned* L, int mode);
/* enabled: 1 while on; fallback_cycle: restart cycle after which the monitor
 * switched it off in the last solve (-1: never); applies: stage applies so far. */
sg_status sg_learned_get_state(sg_learned* L, int* enabled, int* fallback_cycle,
                               long long* applies);
/* Attach L after pc's apply (ASM/RAS and two-level kinds), with the monitor's
 * stagnation ratio (0: no monitor); L == NULL detaches.  A learned stage
 * serves one preconditioner at a time. */
sg_status sg_precond_set_learned(sg_precond* pc, sg_learned* L, double stagnation);

/* ---- file formats (host side, no device work) ------------------------- */
/* read_matrix_market (src/io/matrix_market.h:14-92), same reading rules:
 * '%' comment lines mentioning "symmetric" mirror every off-diagonal entry,
 * "pattern" reads entries as 1.0; duplicates are kept; rows and columns end
 * up ascending (duplicates in file order).  Blank lines are skipped; an
 * index outside the declared size is SG_ERR_INVALID_ARG.  Call with
 * row_ptr == NULL for the sizes, then with arrays of nrows+1 / cap / cap
 * entries (cap >= nnz). */
sg_status sg_read_matrix_market(const char* path, int* nrows, int* ncols, int* nnz, int* row_ptr,
                                int* col_idx, double* vals, int cap);
/* ConvergenceMetrics (src/analysis/convergence_analysis.h:15-65) of a
 * residual history: rate_k = (r_k / r_0)^(1/k), the mean of the last (up to)
 * 20 rates, and the first 20-iteration window with a relative reduction
 * below 1e-3 (-1: none).  rates (optional) receives len values. */
typedef struct sg_convergence {
    int iterations;
    int converged;
    int stagnation_start;
    int reserved;
    double initial_residual;
    double final_residual;
    double asymptotic_rate;
} sg_convergence;
sg_status sg_convergence_metrics(const double* history, int len, int converged,
                                 sg_convergence* out, double* rates);
/* Appends the record ConvergenceMetrics::write_jsonl writes
 * (convergence_analysis.h:69-93; the CLI's <output>.conv.jsonl, src/main.cpp:
 * 251-258): same keys, order and 6-significant-digit numbers. */
sg_status sg_write_convergence_jsonl(const char* path, const char* matrix, const char* precond,
                                     int nparts, int overlap, const double* history, int len,
                                     int converged);

/* ---- problem generators and partitions (host side, deterministic) ----- */
/* make_poisson_2d / make_poisson_3d (src/mesh/poisson.h:10-74).  Call with
 * NULL arrays to get nnz, then with arrays of n+1 / nnz / nnz entries. */
sg_status sg_gen_poisson2d(int nx, int ny, int* row_ptr, int* col_idx, double* vals, int* nnz);
sg_status sg_gen_poisson3d(int nx, int ny, int nz, int* row_ptr, int* col_idx, double* vals,
                           int* nnz);
/* -div(k grad u) on an nx*ny*nz grid, 7-point, Dirichlet, k = exp(sigma*g)
 * with g a unit-variance Gaussian random field of squared-exponential
 * correlation length `corr_len` cells (white noise from SplitMix64(seed)
 * convolved with a separable Gaussian kernel); face coefficients are the
 * harmonic mean of the two cell values.  Same index order as
 * make_poisson_3d. */
sg_status sg_gen_varcoef3d(int nx, int ny, int nz, double sigma, double corr_len,
                           uint64_t seed, int* row_ptr, int* col_idx, double* vals, int* nnz);
/* -div(K grad u) on an nx*ny grid, K = R(theta) diag(1, eps) R(theta)^T,
 * 9-point stencil (central difference for the cross term), Dirichlet; row
 * index iy*nx + ix, columns ascending.  Same calling convention as
 * sg_gen_poisson2d (row_ptr == NULL: only *nnz). */
sg_status sg_gen_aniso2d(int nx, int ny, double eps, double theta, int* row_ptr, int* col_idx,
                         double* vals, int* nnz);
/* n values uniform in [lo,hi): u = (SplitMix64(seed) >> 11) * 2^-53. */
sg_status sg_gen_uniform(uint64_t seed, int n, double lo, double hi, double* out);
/* Built-in graph partitioner used when no partition is given: recursive
 * bisection of the CSR graph by breadth-first level structures. */
sg_status sg_partition_graph(int n, const int* row_ptr, const int* col_idx, int nparts,
                             int* part);
/* Boxes of an nx*ny*nz grid from recursive coordinate bisection with cut
 * fractions drawn from [0.5-spread, 0.5+spread] (seeded): uneven parts. */
sg_status sg_partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed,
                             int* part);
/* Host-only integer set-up of a Schwarz/ILU(0) preconditioner, exactly as
 * sg_precond_setup computes it before any device work: decomposition
 * (build_decomposition, src/decomp/domain_decomp.h:61-93), owned-local map
 * (src/precond/ras.h:34-41), local CSR of A[dofs,dofs] (src/core/
 * sparse_matrix.h:53-83), ILU(0) diagonal positions (src/precond/ilu0.h:
 * 19-29) and sweep levels.  which: 0-6 as sg_precond_get_decomposition;
 * 7 local row_ptr (n_s+1 per subdomain, concatenated), 8 local col_idx,
 * 9 diag_ptr, 10 forward level, 11 backward level. */
sg_status sg_schwarz_structure(int n, const int* row_ptr, const int* col_idx, const int* part,
                               int nparts, int overlap, int which, int* out, int cap, int* len);

#ifdef __cplusplus
}
#endif
#endif
