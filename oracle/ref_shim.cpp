// ref_shim.cpp -- C entry points over the reference's own, unmodified sources.
//
// TEST INFRASTRUCTURE ONLY.  Built by oracle/Makefile (target `ref`) from
// the reference tree where it lies, into oracle/_ref/libref.so; used to pin
// the oracle restatement (oracle.c) and to generate tests/golden fixtures.
// It includes the reference headers and links src/core/gmres.cpp and
// src/core/fgmres.cpp; nothing here re-implements reference numerics.
#include "core/sparse_matrix.h"
#include "core/gmres.h"
#include "core/fgmres.h"
#include "core/vector.h"
#include "mesh/poisson.h"
#include "precond/jacobi.h"
#include "precond/ilu0.h"
#include "precond/asm.h"
#include "precond/ras.h"
#include "precond/two_level_schwarz.h"
#include "decomp/domain_decomp.h"
#include "core/bicgstab.h"
#include "io/matrix_market.h"
#include "analysis/convergence_analysis.h"
#include "analysis/condition_estimator.h"
#include "analysis/spectral_analysis.h"

#include <cstring>
#include <exception>
#include <memory>
#include <vector>

using namespace schwarz;

namespace {
std::vector<int> g_partition;  // injected partition for the METIS seam
int g_nparts = 0;

CSRMatrix make_csr(int n, const int* rp, const int* ci, const double* v) {
    CSRMatrix A;
    A.nrows = n;
    A.ncols = n;
    A.row_ptr.assign(rp, rp + n + 1);
    A.col_idx.assign(ci, ci + rp[n]);
    A.vals.assign(v, v + rp[n]);
    return A;
}

// RASPrecond keeps the owned-local map protected; a derived class reads it.
struct RASView : RASPrecond {
    RASView(int p, int o) : RASPrecond(p, o) {}
    const std::vector<std::vector<int>>& ownloc() const { return owned_local_indices_; }
};

struct RefPC {
    int kind = 0;
    std::unique_ptr<Preconditioner> pc;
    CSRMatrix A;
};
}  // namespace

extern "C" {

int METIS_PartGraphKway(idx_t* nvtxs, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*, idx_t*,
                        idx_t* nparts, real_t*, real_t*, idx_t*, idx_t* objval,
                        idx_t* part) {
    if (static_cast<int>(g_partition.size()) != *nvtxs || g_nparts != *nparts)
        return METIS_ERROR_INPUT;
    for (int i = 0; i < *nvtxs; ++i) part[i] = g_partition[i];
    *objval = 0;
    return METIS_OK;
}

void ref_set_partition(const int* part, int n, int nparts) {
    g_partition.assign(part, part + n);
    g_nparts = nparts;
}

void ref_spmv(int n, const int* rp, const int* ci, const double* v, const double* x,
              double* y) {
    CSRMatrix A = make_csr(n, rp, ci, v);
    A.spmv(x, y);
}

int ref_poisson2d(int nx, int ny, int* rp, int* ci, double* v) {
    CSRMatrix A = make_poisson_2d(nx, ny);
    if (rp) {
        std::memcpy(rp, A.row_ptr.data(), sizeof(int) * A.row_ptr.size());
        std::memcpy(ci, A.col_idx.data(), sizeof(int) * A.col_idx.size());
        std::memcpy(v, A.vals.data(), sizeof(double) * A.vals.size());
    }
    return A.nnz();
}

int ref_poisson3d(int nx, int ny, int nz, int* rp, int* ci, double* v) {
    CSRMatrix A = make_poisson_3d(nx, ny, nz);
    if (rp) {
        std::memcpy(rp, A.row_ptr.data(), sizeof(int) * A.row_ptr.size());
        std::memcpy(ci, A.col_idx.data(), sizeof(int) * A.col_idx.size());
        std::memcpy(v, A.vals.data(), sizeof(double) * A.vals.size());
    }
    return A.nnz();
}

// ILU(0) factors: lu_out[nnz], diag_out[n]
void ref_ilu0(int n, const int* rp, const int* ci, const double* v, double* lu_out,
              int* diag_out) {
    CSRMatrix A = make_csr(n, rp, ci, v);
    ILU0Precond ilu;
    ilu.setup(A);
    std::memcpy(lu_out, ilu.lu_vals().data(), sizeof(double) * ilu.lu_vals().size());
    std::memcpy(diag_out, ilu.diag_ptr().data(), sizeof(int) * ilu.diag_ptr().size());
}

// Decomposition of RASPrecond::setup (uses the injected partition).
// Sizes first (sub_total, ownloc_total) when the array pointers are null.
int ref_decompose(int n, const int* rp, const int* ci, const double* v, int nparts,
                  int overlap, int* sub_ptr, int* sub, int* ownloc_ptr, int* ownloc,
                  int* owned_ptr, int* owned) {
    try {
        CSRMatrix A = make_csr(n, rp, ci, v);
        RASView ras(nparts, overlap);
        ras.setup(A);
        const DomainDecomposition& dd = ras.decomposition();
        int total = 0, ototal = 0, wtotal = 0;
        for (int s = 0; s < nparts; ++s) {
            if (sub_ptr) sub_ptr[s] = total;
            if (ownloc_ptr) ownloc_ptr[s] = ototal;
            if (owned_ptr) owned_ptr[s] = wtotal;
            for (int d : dd.subdomain_dofs[s]) { if (sub) sub[total] = d; ++total; }
            for (int d : ras.ownloc()[s]) { if (ownloc) ownloc[ototal] = d; ++ototal; }
            for (int d : dd.owned_dofs[s]) { if (owned) owned[wtotal] = d; ++wtotal; }
        }
        if (sub_ptr) sub_ptr[nparts] = total;
        if (ownloc_ptr) ownloc_ptr[nparts] = ototal;
        if (owned_ptr) owned_ptr[nparts] = wtotal;
        return total;
    } catch (const std::exception&) {
        return -1;
    }
}

// Coarse operator A0 of TwoLevelSchwarzPrecond (dense, as the reference builds it).
int ref_coarse_a0(int n, const int* rp, const int* ci, const double* v, int nparts,
                  int overlap, double* a0_out) {
    try {
        CSRMatrix A = make_csr(n, rp, ci, v);
        RASView ras(nparts, overlap);
        ras.setup(A);
        CoarseSpace cs;
        cs.build_piecewise_constant(A, ras.decomposition());
        std::memcpy(a0_out, cs.A0.data(), sizeof(double) * cs.A0.size());
        return cs.n_coarse;
    } catch (const std::exception&) {
        return -1;
    }
}

// kinds: 0 none, 1 jacobi, 2 ilu0, 3 asm, 4 ras, 5 twolevel_asm, 6 twolevel_ras
void* ref_pc_create(int kind, int n, const int* rp, const int* ci, const double* v,
                    int nparts, int overlap) {
    try {
        auto* h = new RefPC();
        h->kind = kind;
        h->A = make_csr(n, rp, ci, v);
        switch (kind) {
        case 1: h->pc = std::make_unique<JacobiPrecond>(); break;
        case 2: h->pc = std::make_unique<ILU0Precond>(); break;
        case 3: h->pc = std::make_unique<ASMPrecond>(nparts, overlap); break;
        case 4: h->pc = std::make_unique<RASPrecond>(nparts, overlap); break;
        case 5:
            h->pc = std::make_unique<TwoLevelSchwarzPrecond>(nparts, overlap, FineLevelType::ASM);
            break;
        case 6:
            h->pc = std::make_unique<TwoLevelSchwarzPrecond>(nparts, overlap, FineLevelType::RAS);
            break;
        default: break;
        }
        if (h->pc) h->pc->setup(h->A);
        return h;
    } catch (const std::exception&) {
        return nullptr;
    }
}

void ref_pc_apply(void* hp, const double* x, double* y, int n) {
    auto* h = static_cast<RefPC*>(hp);
    if (h->pc) h->pc->apply(x, y, n);
    else std::memcpy(y, x, sizeof(double) * n);
}

void ref_pc_destroy(void* hp) { delete static_cast<RefPC*>(hp); }

static int run_solver(bool flexible, void* hp, const double* b, double* x, int restart,
                      int max_iter, double tol, int* iters, double* res, double* hist,
                      int hist_cap, int* hist_len) {
    auto* h = static_cast<RefPC*>(hp);
    int n = h->A.nrows;
    std::vector<double> bb(b, b + n), xx(x, x + n);
    GMRESParams p;
    p.restart = restart;
    p.max_iter = max_iter;
    p.tol = tol;
    GMRESResult r = flexible ? fgmres(h->A, bb, xx, h->pc.get(), p)
                             : gmres(h->A, bb, xx, h->pc.get(), p);
    std::memcpy(x, xx.data(), sizeof(double) * n);
    *iters = r.iterations;
    *res = r.residual_norm;
    int nh = static_cast<int>(r.residual_history.size());
    if (hist)
        for (int i = 0; i < nh && i < hist_cap; ++i) hist[i] = r.residual_history[i];
    if (hist_len) *hist_len = nh;
    return r.converged ? 1 : 0;
}

int ref_gmres(void* hp, const double* b, double* x, int restart, int max_iter, double tol,
              int* iters, double* res, double* hist, int hist_cap, int* hist_len) {
    return run_solver(false, hp, b, x, restart, max_iter, tol, iters, res, hist, hist_cap,
                      hist_len);
}

int ref_fgmres(void* hp, const double* b, double* x, int restart, int max_iter, double tol,
               int* iters, double* res, double* hist, int hist_cap, int* hist_len) {
    return run_solver(true, hp, b, x, restart, max_iter, tol, iters, res, hist, hist_cap,
                      hist_len);
}

// ---- I/O, the adjacent solver and the analysis tools on the same boundary
int ref_read_mm(const char* path, int* nrows, int* ncols, int* nnz, int* rp, int* ci, double* v,
                int cap) {
    try {
        CSRMatrix A = read_matrix_market(path);
        *nrows = A.nrows;
        *ncols = A.ncols;
        *nnz = A.nnz();
        if (rp) {
            if (cap < A.nnz()) return -2;
            std::memcpy(rp, A.row_ptr.data(), sizeof(int) * (A.nrows + 1));
            std::memcpy(ci, A.col_idx.data(), sizeof(int) * A.nnz());
            std::memcpy(v, A.vals.data(), sizeof(double) * A.nnz());
        }
        return 0;
    } catch (const std::exception&) {
        return -1;
    }
}

// dout: initial, final, asymptotic rate; iout: iterations, stagnation start
void ref_conv_metrics(const double* hist, int len, int conv, double* dout, int* iout,
                      double* rates) {
    std::vector<double> h(hist, hist + len);
    ConvergenceMetrics m = analyze_convergence(h, conv != 0);
    dout[0] = m.initial_residual;
    dout[1] = m.final_residual;
    dout[2] = m.asymptotic_rate;
    iout[0] = m.iterations;
    iout[1] = m.stagnation_start;
    if (rates)
        for (int i = 0; i < (int)m.rates.size(); ++i) rates[i] = m.rates[i];
}

void ref_conv_write(const char* path, const char* matrix, const char* precond, int nparts,
                    int overlap, const double* hist, int len, int conv) {
    std::vector<double> h(hist, hist + len);
    analyze_convergence(h, conv != 0).write_jsonl(path, matrix, precond, nparts, overlap);
}

int ref_bicgstab(void* hp, const double* b, double* x, int max_iter, double tol, int* iters,
                 double* res, double* hist, int hist_cap, int* hist_len) {
    auto* h = static_cast<RefPC*>(hp);
    int n = h->A.nrows;
    std::vector<double> bb(b, b + n), xx(x, x + n);
    GMRESParams p;
    p.max_iter = max_iter;
    p.tol = tol;
    GMRESResult r = bicgstab(h->A, bb, xx, h->pc.get(), p);
    std::memcpy(x, xx.data(), sizeof(double) * n);
    *iters = r.iterations;
    *res = r.residual_norm;
    int nh = static_cast<int>(r.residual_history.size());
    if (hist)
        for (int i = 0; i < nh && i < hist_cap; ++i) hist[i] = r.residual_history[i];
    if (hist_len) *hist_len = nh;
    return r.converged ? 1 : 0;
}

// out: lambda_min, lambda_max, kappa; iout: Lanczos steps, valid
void ref_condition(void* hp, int k, unsigned seed, double* out, int* iout) {
    auto* h = static_cast<RefPC*>(hp);
    ConditionEstimate e = estimate_condition(h->A, h->pc.get(), k, seed);
    out[0] = e.lambda_min;
    out[1] = e.lambda_max;
    out[2] = e.kappa;
    iout[0] = e.lanczos_steps;
    iout[1] = e.valid ? 1 : 0;
}

// out: spectral radius; iout: power iterations, convergence_ok
void ref_spectral(void* hp, int max_iter, double tol, unsigned seed, double* out, int* iout) {
    auto* h = static_cast<RefPC*>(hp);
    SpectralResult r = estimate_spectral_radius(h->A, h->pc.get(), max_iter, tol, seed);
    out[0] = r.spectral_radius;
    iout[0] = r.power_iters;
    iout[1] = r.convergence_ok ? 1 : 0;
}

}  // extern "C"
