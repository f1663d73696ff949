/*
 * oracle.h -- CPU restatement of the schwarz-gmres solve path.
 *
 * TEST INFRASTRUCTURE ONLY.  This library is the checker: the parity tests,
 * __graft_entry__.smoke() and the cpu_baseline leg of bench.py call it to
 * produce the answers the CUDA path is compared against.  Nothing in the
 * product (libsgmres.so, the Python mirror, the CLI) links or calls it.
 *
 * Every function restates one function of the reference C++ sources
 * (izbassarn7/schwarz-gmres-dashboard, paths relative to that project) and
 * cites the file:line it follows.  Floating-point operations are kept in the
 * reference's order and the file is compiled with -ffp-contract=off so that,
 * on the same host, results are bit-identical to the reference build
 * (oracle/_ref) -- the golden-vector tests check exactly that.
 *
 * The reference partitions with METIS_PartGraphKway (src/decomp/
 * domain_decomp.h:23-58); METIS is not available, so every entry point that
 * builds a decomposition takes the partition vector explicitly (the same
 * vector is injected into the reference build through its metis.h seam).
 */
#ifndef SG_ORACLE_H
#define SG_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Preconditioner kinds, in the order of the reference CLI's --precond list
 * (src/main.cpp:44, :190-208). */
enum {
    ORC_PC_NONE = 0,
    ORC_PC_JACOBI = 1,
    ORC_PC_ILU0 = 2,
    ORC_PC_ASM = 3,
    ORC_PC_RAS = 4,
    ORC_PC_TWOLEVEL_ASM = 5,
    ORC_PC_TWOLEVEL_RAS = 6
};

typedef struct orc_pc orc_pc;

void orc_set_threads(int nthreads);
int orc_get_threads(void);

/* y = A x  (src/core/sparse_matrix.h:30-37) */
void orc_spmv(int n, const int* rp, const int* ci, const double* v,
              const double* x, double* y);

/* A[idx, idx]; two calls: with out arrays NULL returns the nnz.
 * (src/core/sparse_matrix.h:53-83) */
int orc_extract(int nrows, int ncols, const int* rp, const int* ci, const double* v,
                const int* idx, int nidx, int* rp_out, int* ci_out, double* v_out);

/* ILU(0) factorisation in place on a copy of the values; diag_out[i] is the
 * position of the diagonal (-1 if absent).  (src/precond/ilu0.h:13-54) */
void orc_ilu0_factor(int n, const int* rp, const int* ci, const double* v,
                     double* lu_out, int* diag_out);
/* forward/backward sweep (src/precond/ilu0.h:57-79) */
void orc_ilu0_solve(int n, const int* rp, const int* ci, const double* lu,
                    const int* diag, const double* x, double* y);

/* Decomposition from a partition (src/decomp/domain_decomp.h:61-93) plus the
 * owned-local map of RAS (src/precond/ras.h:34-41).  Returns 0 on success.
 * Output arrays are allocated by the oracle; free with orc_free. */
int orc_decompose(int n, const int* rp, const int* ci, const int* part, int nparts,
                  int overlap, int** owned_ptr, int** owned, int** sub_ptr, int** sub,
                  int** ownloc_ptr, int** ownloc);
void orc_free(void* p);

/* Level of each row for the forward (lower) and backward (upper) sweeps of
 * ILU(0): level = 1 + max level of the rows the sweep reads. The reference
 * sweeps rows one by one (src/precond/ilu0.h:62-76); this is the dependency
 * structure of that order, used to pin the device level schedules. */
int orc_levels_lower(int n, const int* rp, const int* ci, int* level);
int orc_levels_upper(int n, const int* rp, const int* ci, const int* diag, int* level);

/* Preconditioner objects.  part may be NULL for JACOBI/ILU0. */
orc_pc* orc_pc_create(int kind, int n, const int* rp, const int* ci, const double* v,
                      int nparts, int overlap, const int* part, int* err);
void orc_pc_apply(const orc_pc* pc, const double* x, double* y, int n);
void orc_pc_destroy(orc_pc* pc);
/* coarse data of a two-level preconditioner: A0 (n_coarse^2, row-major) */
int orc_pc_coarse(const orc_pc* pc, double* a0_out);
/* ILU factors of subdomain s (or the global ILU0): returns n_s, nnz via out */
int orc_pc_sub_factor(const orc_pc* pc, int s, int* nnz_out, const int** rp,
                      const int** ci, const double** lu, const int** diag);

/* Restarted GMRES(m), left preconditioning (src/core/gmres.cpp:34-160).
 * hist may be NULL.  Returns converged flag. */
int orc_gmres(int n, const int* rp, const int* ci, const double* v, const double* b,
              double* x, const orc_pc* pc, int restart, int max_iter, double tol,
              int* iters, double* res_norm, double* hist, int hist_cap, int* hist_len);
/* FGMRES(m), right preconditioning storing V and Z (src/core/fgmres.cpp:28-144). */
int orc_fgmres(int n, const int* rp, const int* ci, const double* v, const double* b,
               double* x, const orc_pc* pc, int restart, int max_iter, double tol,
               int* iters, double* res_norm, double* hist, int hist_cap, int* hist_len);

/* Poisson generators (src/mesh/poisson.h:10-74): returns nnz; arrays may be
 * NULL on the sizing call. */
int orc_poisson2d(int nx, int ny, int* rp, int* ci, double* v);
int orc_poisson3d(int nx, int ny, int nz, int* rp, int* ci, double* v);

/* BiCGSTAB, right preconditioned (src/core/bicgstab.h:57-204); pc may be
 * NULL.  Returns the converged flag. */
int orc_bicgstab(int n, const int* rp, const int* ci, const double* v, const double* b,
                 double* x, const orc_pc* pc, int max_iter, double tol, int* iters,
                 double* res_norm, double* hist, int hist_cap, int* hist_len);
/* estimate_condition (src/analysis/condition_estimator.h:94-191): out =
 * lambda_min, lambda_max, kappa; iout = Lanczos steps, valid. */
int orc_condition(int n, const int* rp, const int* ci, const double* v, const orc_pc* pc, int k,
                  unsigned seed, double* out, int* iout);
/* estimate_spectral_radius (src/analysis/spectral_analysis.h:30-97): out =
 * rho(I - M^{-1}A); iout = power iterations, rho < 1. */
void orc_spectral(int n, const int* rp, const int* ci, const double* v, const orc_pc* pc,
                  int max_iter, double tol, unsigned seed, double* out, int* iout);

/* Benchmark inputs the project generates (no reference counterpart),
 * restated from the package so the CPU baseline needs nothing else:
 * uniform vectors (SplitMix64, (u >> 11) * 2^-53), uneven box partitions
 * (returns 0 on success) and the 3D variable-coefficient 7-point operator
 * k = exp(sigma g) (returns nnz; rp == NULL only sizes). */
void orc_uniform(uint64_t seed, int n, double lo, double hi, double* out);
int orc_partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed,
                        int* part);
int orc_varcoef3d(int nx, int ny, int nz, double sigma, double corr, uint64_t seed, int* rp,
                  int* ci, double* v);

#ifdef __cplusplus
}
#endif
#endif
