// schwarz_gmres.hpp -- header-only C++17 facade over libsgmres.so with the
// reference's names and signatures, so code written against the reference's
// src/core/*.h and src/precond/*.h compiles unchanged and runs on the GPU:
//
//   CSRMatrix                 src/core/sparse_matrix.h:13-96
//   Preconditioner            src/precond/preconditioner.h:7-20
//   JacobiPrecond             src/precond/jacobi.h:10-27
//   ILU0Precond               src/precond/ilu0.h:11-93
//   ASMPrecond / RASPrecond   src/precond/asm.h:13-71, src/precond/ras.h:16-82
//   TwoLevelSchwarzPrecond    src/precond/two_level_schwarz.h:21-75
//   GMRESParams/GMRESResult   src/core/gmres.h:12-24
//   gmres / fgmres            src/core/gmres.h:28-33, src/core/fgmres.h:42-47
//   FlexApply / fgmres_flex   src/core/fgmres.h:37, :50-55
//   bicgstab                  src/core/bicgstab.h:57-204
//   make_poisson_2d/3d        src/mesh/poisson.h:10-74
//   read_matrix_market        src/io/matrix_market.h:14-92
//   ConvergenceMetrics /      src/analysis/convergence_analysis.h:15-123
//     analyze_convergence
//   ConditionEstimate /       src/analysis/condition_estimator.h:32-191
//     estimate_condition
//   SpectralResult /          src/analysis/spectral_analysis.h:21-97
//     estimate_spectral_radius
//
// Errors surface as std::runtime_error, as in the reference.  Extra knobs
// (partition vector, factor/sweep dtypes, precision, stopping rule) are
// optional members with the reference's behaviour as default.  The GPU
// preconditioners of this header run on the device; any other
// Preconditioner subclass (and fgmres_flex's FlexApply) is called on the
// host through sg_precond_create_host, in stream order inside the solve --
// its apply must not call CUDA.
#pragma once

#include <cstdio>
#include <functional>
#include <iostream>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

#include "sgmres.h"

namespace schwarz {

namespace detail {
inline void check(sg_status st) {
    if (st != SG_OK)
        throw std::runtime_error(std::string("libsgmres: ") + sg_status_string(st) + ": " +
                                 sg_last_error());
}
// one context (device 0, own stream) per process
inline sg_ctx* context() {
    static std::shared_ptr<sg_ctx> ctx = [] {
        sg_ctx* c = nullptr;
        check(sg_ctx_create(0, &c));
        return std::shared_ptr<sg_ctx>(c, [](sg_ctx* p) { sg_ctx_destroy(p); });
    }();
    return ctx.get();
}
struct CsrHandle {
    sg_csr* h = nullptr;
    ~CsrHandle() {
        if (h) sg_csr_destroy(h);
    }
};
}  // namespace detail

struct CSRMatrix {
    int nrows = 0;
    int ncols = 0;
    std::vector<int> row_ptr;
    std::vector<int> col_idx;
    std::vector<double> vals;

    int nnz() const { return static_cast<int>(vals.size()); }

    void resize(int nr, int nc, int nz) {
        nrows = nr;
        ncols = nc;
        row_ptr.resize(nr + 1);
        col_idx.resize(nz);
        vals.resize(nz);
    }

    // device copy of the current arrays
    std::shared_ptr<detail::CsrHandle> device() const {
        auto d = std::make_shared<detail::CsrHandle>();
        detail::check(sg_csr_create(detail::context(), nrows, ncols, nnz(), row_ptr.data(),
                                    col_idx.data(), vals.data(), SG_MEM_HOST, &d->h));
        return d;
    }

    // y = A x on the GPU, bit-identical to the reference's serial row loop
    void spmv(const double* x, double* y) const {
        auto d = device();
        detail::check(sg_csr_spmv(d->h, x, y, SG_MEM_HOST));
    }
    void spmv(const std::vector<double>& x, std::vector<double>& y) const {
        if (static_cast<int>(x.size()) < ncols) throw std::runtime_error("spmv: x too short");
        y.resize(nrows);
        spmv(x.data(), y.data());
    }

    double diagonal(int i) const {
        for (int j = row_ptr[i]; j < row_ptr[i + 1]; ++j)
            if (col_idx[j] == i) return vals[j];
        return 0.0;
    }

    CSRMatrix extract_submatrix(const std::vector<int>& indices) const {
        const int n = static_cast<int>(indices.size());
        std::vector<int> inv(static_cast<size_t>(nrows > ncols ? nrows : ncols), -1);
        for (int i = 0; i < n; ++i) inv[indices[i]] = i;
        CSRMatrix s;
        s.nrows = s.ncols = n;
        s.row_ptr.assign(n + 1, 0);
        for (int li = 0; li < n; ++li) {
            const int gi = indices[li];
            s.row_ptr[li] = static_cast<int>(s.col_idx.size());
            for (int j = row_ptr[gi]; j < row_ptr[gi + 1]; ++j) {
                const int lj = inv[col_idx[j]];
                if (lj >= 0) {
                    s.col_idx.push_back(lj);
                    s.vals.push_back(vals[j]);
                }
            }
        }
        s.row_ptr[n] = static_cast<int>(s.col_idx.size());
        return s;
    }
};

inline CSRMatrix make_identity(int n) {
    CSRMatrix I;
    I.nrows = I.ncols = n;
    I.row_ptr.resize(n + 1);
    I.col_idx.resize(n);
    I.vals.assign(n, 1.0);
    for (int i = 0; i <= n; ++i) I.row_ptr[i] = i;
    for (int i = 0; i < n; ++i) I.col_idx[i] = i;
    return I;
}

namespace detail {
inline CSRMatrix gen(int nx, int ny, int nz, bool three_d) {
    int nnz = 0;
    const int n = nx * ny * (three_d ? nz : 1);
    if (three_d) check(sg_gen_poisson3d(nx, ny, nz, nullptr, nullptr, nullptr, &nnz));
    else check(sg_gen_poisson2d(nx, ny, nullptr, nullptr, nullptr, &nnz));
    CSRMatrix A;
    A.resize(n, n, nnz);
    if (three_d)
        check(sg_gen_poisson3d(nx, ny, nz, A.row_ptr.data(), A.col_idx.data(), A.vals.data(), &nnz));
    else
        check(sg_gen_poisson2d(nx, ny, A.row_ptr.data(), A.col_idx.data(), A.vals.data(), &nnz));
    return A;
}
}  // namespace detail

inline CSRMatrix make_poisson_2d(int nx, int ny) { return detail::gen(nx, ny, 1, false); }
inline CSRMatrix make_poisson_3d(int nx, int ny, int nz) { return detail::gen(nx, ny, nz, true); }

// ------------------------------------------------------------------ preconditioners
class Preconditioner {
public:
    virtual ~Preconditioner() = default;
    virtual void setup(const CSRMatrix& A) = 0;
    // y = M^{-1} x
    virtual void apply(const double* x, double* y, int n) const = 0;
    void apply(const std::vector<double>& x, std::vector<double>& y) const {
        y.resize(x.size());
        apply(x.data(), y.data(), static_cast<int>(x.size()));
    }
};

// A preconditioner that lives on the GPU (every class below).
class DevicePreconditioner : public Preconditioner {
public:
    explicit DevicePreconditioner(sg_precond_kind kind, int nparts = 1, int overlap = 0)
        : kind_(kind) {
        opts_.nparts = nparts;
        opts_.overlap = overlap;
        opts_.factor_dtype = SG_FP64;
        opts_.sweep_dtype = SG_FP64;
        opts_.partition = nullptr;
    }
    ~DevicePreconditioner() override {
        if (pc_) sg_precond_destroy(pc_);
    }
    DevicePreconditioner(const DevicePreconditioner&) = delete;
    DevicePreconditioner& operator=(const DevicePreconditioner&) = delete;

    // optional: partition vector (replaces METIS), factor and sweep dtypes
    void set_partition(std::vector<int> part) { partition_ = std::move(part); }
    void set_precision(sg_dtype factor, sg_dtype sweep) {
        opts_.factor_dtype = factor;
        opts_.sweep_dtype = sweep;
    }

    void setup(const CSRMatrix& A) override {
        if (pc_) sg_precond_destroy(pc_);
        pc_ = nullptr;
        A_ = A.device();
        opts_.partition = partition_.empty() ? nullptr : partition_.data();
        detail::check(sg_precond_create(detail::context(), kind_, &opts_, &pc_));
        detail::check(sg_precond_setup(pc_, A_->h));
        n_ = A.nrows;
    }
    void apply(const double* x, double* y, int n) const override {
        if (!pc_) throw std::runtime_error("preconditioner used before setup");
        detail::check(sg_precond_apply(pc_, x, y, n, SG_MEM_HOST));
    }
    sg_precond* handle() const { return pc_; }
    const sg_csr* matrix() const { return A_ ? A_->h : nullptr; }

protected:
    sg_precond_kind kind_;
    sg_precond_opts opts_{};
    std::vector<int> partition_;
    sg_precond* pc_ = nullptr;
    std::shared_ptr<detail::CsrHandle> A_;
    int n_ = 0;
};

class JacobiPrecond : public DevicePreconditioner {
public:
    JacobiPrecond() : DevicePreconditioner(SG_PC_JACOBI) {}
};

class ILU0Precond : public DevicePreconditioner {
public:
    ILU0Precond() : DevicePreconditioner(SG_PC_ILU0) {}
};

class ASMPrecond : public DevicePreconditioner {
public:
    ASMPrecond(int nparts, int overlap) : DevicePreconditioner(SG_PC_ASM, nparts, overlap) {}
};

class RASPrecond : public DevicePreconditioner {
public:
    RASPrecond(int nparts, int overlap) : DevicePreconditioner(SG_PC_RAS, nparts, overlap) {}
};

enum class FineLevelType { ASM, RAS };

class TwoLevelSchwarzPrecond : public DevicePreconditioner {
public:
    TwoLevelSchwarzPrecond(int nparts, int overlap, FineLevelType fine_type = FineLevelType::RAS)
        : DevicePreconditioner(fine_type == FineLevelType::ASM ? SG_PC_TWOLEVEL_ASM
                                                               : SG_PC_TWOLEVEL_RAS,
                               nparts, overlap) {}
};

// ------------------------------------------------------------------ solvers
struct GMRESResult {
    int iterations = 0;
    double residual_norm = 0.0;
    bool converged = false;
    double time_solve_s = 0.0;
    std::vector<double> residual_history;
    // GPU extras
    double true_rel_residual = 0.0;
    int cycles = 0;
};

struct GMRESParams {
    int restart = 30;
    int max_iter = 1000;
    double tol = 1e-10;
    // GPU extras (defaults = the reference's behaviour)
    sg_tol_kind tol_kind = SG_TOL_REF_ABS;
    sg_dtype precision = SG_FP64;
    bool use_graph = true;
};

namespace detail {
// Any host-side apply (a foreign Preconditioner, a FlexApply) as a host
// preconditioner of the library.  The C callback catches exceptions and
// reports them through the status; solve() rethrows the message.
struct HostApply {
    std::function<void(const double*, double*, int)> fn;
    std::string error;
    static int call(void* user, const double* x, double* y, int n) {
        auto* h = static_cast<HostApply*>(user);
        try {
            h->fn(x, y, n);
            return 0;
        } catch (const std::exception& e) {
            h->error = e.what();
        } catch (...) {
            h->error = "unknown exception";
        }
        return 1;
    }
};
struct PrecondHandle {
    sg_precond* h = nullptr;
    ~PrecondHandle() {
        if (h) sg_precond_destroy(h);
    }
};

inline GMRESResult solve_with(sg_solver solver, const CSRMatrix& A, const std::vector<double>& b,
                              std::vector<double>& x, const DevicePreconditioner* dm,
                              HostApply* host, const GMRESParams& p) {
    if (static_cast<int>(b.size()) != A.nrows) throw std::runtime_error("b has the wrong size");
    x.resize(A.nrows, 0.0);
    std::shared_ptr<CsrHandle> dA;
    const sg_csr* hA = dm ? dm->matrix() : nullptr;
    if (!hA) {
        dA = A.device();
        hA = dA->h;
    }
    PrecondHandle hp;
    sg_precond* pc = dm ? dm->handle() : nullptr;
    if (host) {
        check(sg_precond_create_host(context(), &HostApply::call, host, A.nrows, &hp.h));
        pc = hp.h;
    }
    std::vector<double> hist(static_cast<size_t>(p.max_iter) + p.restart + 1);
    sg_solve_params prm{};
    prm.restart = p.restart;
    prm.max_iter = p.max_iter;
    prm.tol = p.tol;
    prm.tol_kind = p.tol_kind;
    prm.precision = p.precision;
    prm.use_graph = p.use_graph ? 1 : 0;
    prm.history = hist.data();
    prm.history_cap = static_cast<int>(hist.size());
    sg_solve_result r{};
    const sg_status st = sg_solve(context(), solver, hA, pc, b.data(), x.data(), A.nrows,
                                  SG_MEM_HOST, &prm, &r);
    if (st == SG_ERR_CALLBACK && host && !host->error.empty())
        throw std::runtime_error(host->error);  // what the apply threw
    check(st);
    GMRESResult out;
    out.iterations = r.iterations;
    out.residual_norm = r.residual_norm;
    out.converged = r.converged != 0;
    out.time_solve_s = r.time_solve_s;
    out.true_rel_residual = r.true_rel_residual;
    out.cycles = r.cycles;
    const int h = r.history_len < prm.history_cap ? r.history_len : prm.history_cap;
    out.residual_history.assign(hist.begin(), hist.begin() + h);
    return out;
}

inline GMRESResult solve(sg_solver solver, const CSRMatrix& A, const std::vector<double>& b,
                         std::vector<double>& x, const Preconditioner* M, const GMRESParams& p) {
    const auto* dm = dynamic_cast<const DevicePreconditioner*>(M);
    if (M && !dm) {
        // a Preconditioner plugin of the caller's own: applied on the host
        HostApply host{[M](const double* in, double* out, int n) { M->apply(in, out, n); }, {}};
        return solve_with(solver, A, b, x, nullptr, &host, p);
    }
    return solve_with(solver, A, b, x, dm, nullptr, p);
}
}  // namespace detail

inline GMRESResult gmres(const CSRMatrix& A, const std::vector<double>& b, std::vector<double>& x,
                         const Preconditioner* M, const GMRESParams& params = {}) {
    return detail::solve(SG_GMRES, A, b, x, M, params);
}

inline GMRESResult fgmres(const CSRMatrix& A, const std::vector<double>& b,
                          std::vector<double>& x, const Preconditioner* M,
                          const GMRESParams& params = {}) {
    return detail::solve(SG_FGMRES, A, b, x, M, params);
}

// FGMRES with an arbitrary (possibly nonlinear) apply z = M(v), as
// fgmres_flex (src/core/fgmres.h:37, :50-55); an empty FlexApply is the
// identity.  The apply runs on the host, on the normalised basis vector.
using FlexApply = std::function<void(const double* x, double* y, int n)>;
inline GMRESResult fgmres_flex(const CSRMatrix& A, const std::vector<double>& b,
                               std::vector<double>& x, FlexApply apply,
                               const GMRESParams& params = {}) {
    if (!apply) return detail::solve(SG_FGMRES, A, b, x, nullptr, params);
    detail::HostApply host{std::move(apply), {}};
    return detail::solve_with(SG_FGMRES, A, b, x, nullptr, &host, params);
}

// BiCGSTAB, right preconditioned (src/core/bicgstab.h:57-204), FP64.
inline GMRESResult bicgstab(const CSRMatrix& A, const std::vector<double>& b,
                            std::vector<double>& x, const Preconditioner* M,
                            const GMRESParams& params = {}) {
    return detail::solve(SG_BICGSTAB, A, b, x, M, params);
}

// ------------------------------------------------------------------ analysis
struct ConditionEstimate {
    double lambda_min = 0.0;
    double lambda_max = 0.0;
    double kappa = 0.0;
    int lanczos_steps = 0;
    bool valid = false;
};

struct SpectralResult {
    double spectral_radius = 0.0;
    bool convergence_ok = false;
    int power_iters = 0;
    std::vector<double> eigenvector;
};

namespace detail {
// runs f(ctx, device matrix, device-or-host preconditioner)
template <class F>
void with_operator(const CSRMatrix& A, const Preconditioner* M, F&& f) {
    const auto* dm = dynamic_cast<const DevicePreconditioner*>(M);
    std::shared_ptr<CsrHandle> dA;
    const sg_csr* hA = dm ? dm->matrix() : nullptr;
    if (!hA) {
        dA = A.device();
        hA = dA->h;
    }
    PrecondHandle hp;
    HostApply host{[M](const double* in, double* out, int n) { M->apply(in, out, n); }, {}};
    sg_precond* pc = dm ? dm->handle() : nullptr;
    if (M && !dm) {
        check(sg_precond_create_host(context(), &HostApply::call, &host, A.nrows, &hp.h));
        pc = hp.h;
    }
    const sg_status st = f(context(), hA, pc);
    if (st == SG_ERR_CALLBACK && !host.error.empty()) throw std::runtime_error(host.error);
    check(st);
}
}  // namespace detail

// estimate_condition (src/analysis/condition_estimator.h:94-191): k Lanczos
// steps on M^{-1}A (A when M is null) on the GPU.
inline ConditionEstimate estimate_condition(const CSRMatrix& A, const Preconditioner* M,
                                            int k = 80, unsigned int seed = 42) {
    sg_condition_estimate e{};
    detail::with_operator(A, M, [&](sg_ctx* c, const sg_csr* hA, sg_precond* pc) {
        return sg_estimate_condition(c, hA, pc, k, seed, &e);
    });
    ConditionEstimate out;
    out.lambda_min = e.lambda_min;
    out.lambda_max = e.lambda_max;
    out.kappa = e.kappa;
    out.lanczos_steps = e.lanczos_steps;
    out.valid = e.valid != 0;
    return out;
}

// estimate_spectral_radius (src/analysis/spectral_analysis.h:30-97).
inline SpectralResult estimate_spectral_radius(const CSRMatrix& A, const Preconditioner* M,
                                               int max_iter = 200, double tol = 1e-6,
                                               unsigned int seed = 123) {
    sg_spectral_result r{};
    SpectralResult out;
    out.eigenvector.resize(A.nrows);
    detail::with_operator(A, M, [&](sg_ctx* c, const sg_csr* hA, sg_precond* pc) {
        return sg_estimate_spectral_radius(c, hA, pc, max_iter, tol, seed, out.eigenvector.data(),
                                           &r);
    });
    out.spectral_radius = r.spectral_radius;
    out.convergence_ok = r.convergence_ok != 0;
    out.power_iters = r.power_iters;
    return out;
}

inline void print_condition_estimate(const ConditionEstimate& e, const std::string& label = "") {
    std::cout << "  Condition estimate" << (label.empty() ? "" : " (" + label + ")")
              << " [Lanczos " << e.lanczos_steps << " steps]:\n";
    if (!e.valid || e.lambda_min <= 0.0)
        std::cout << "    Ritz(min) = " << e.lambda_min << "\n    Ritz(max) = " << e.lambda_max
                  << "\n    kappa_est = " << e.kappa
                  << "\n    (Note: M^{-1}A is non-symmetric; bounds are approximate)\n";
    else
        std::cout << "    lambda_min = " << e.lambda_min << "\n    lambda_max = " << e.lambda_max
                  << "\n    kappa      = " << e.kappa << "\n";
}

inline void print_spectral_result(const SpectralResult& r, const std::string& label = "") {
    std::cout << "  Spectral radius" << (label.empty() ? "" : " (" + label + ")")
              << " [power iter " << r.power_iters << " steps]:\n"
              << "    rho(I - M^{-1}A) = " << r.spectral_radius << "\n"
              << "    Convergence cond : "
              << (r.convergence_ok ? "SATISFIED (rho < 1)" : "VIOLATED (rho >= 1)") << "\n";
}

// ConvergenceMetrics / analyze_convergence (src/analysis/
// convergence_analysis.h:15-123), computed by the library.
struct ConvergenceMetrics {
    std::vector<double> residuals;
    std::vector<double> rates;
    double initial_residual = 0.0;
    double final_residual = 0.0;
    double asymptotic_rate = 0.0;
    int stagnation_start = -1;
    bool converged = false;
    int iterations = 0;

    void compute(const std::vector<double>& history, bool conv) {
        residuals = history;
        rates.assign(history.size(), 0.0);
        sg_convergence m{};
        detail::check(sg_convergence_metrics(history.data(), static_cast<int>(history.size()),
                                             conv ? 1 : 0, &m, rates.data()));
        initial_residual = m.initial_residual;
        final_residual = m.final_residual;
        asymptotic_rate = m.asymptotic_rate;
        stagnation_start = m.stagnation_start;
        converged = m.converged != 0;
        iterations = m.iterations;
    }
    // appends the <output>.conv.jsonl record
    void write_jsonl(const std::string& path, const std::string& matrix,
                     const std::string& precond, int nparts, int overlap) const {
        detail::check(sg_write_convergence_jsonl(path.c_str(), matrix.c_str(), precond.c_str(),
                                                 nparts, overlap, residuals.data(),
                                                 static_cast<int>(residuals.size()),
                                                 converged ? 1 : 0));
    }
    void print_summary() const {
        std::cout << "  Convergence analysis:\n"
                  << "    Initial residual : " << initial_residual << "\n"
                  << "    Final residual   : " << final_residual << "\n"
                  << "    Asymptotic rate  : " << asymptotic_rate << "\n";
        if (stagnation_start >= 0)
            std::cout << "    *** Stagnation detected at iter " << stagnation_start << " ***\n";
        else
            std::cout << "    No stagnation detected\n";
    }
};

inline ConvergenceMetrics analyze_convergence(const std::vector<double>& history, bool converged) {
    ConvergenceMetrics m;
    m.compute(history, converged);
    return m;
}

// read_matrix_market (src/io/matrix_market.h:14-92), the library's reader
inline CSRMatrix read_matrix_market(const std::string& filename) {
    int nr = 0, nc = 0, nz = 0;
    detail::check(sg_read_matrix_market(filename.c_str(), &nr, &nc, &nz, nullptr, nullptr,
                                        nullptr, 0));
    CSRMatrix A;
    A.resize(nr, nc, nz);
    detail::check(sg_read_matrix_market(filename.c_str(), &nr, &nc, &nz, A.row_ptr.data(),
                                        A.col_idx.data(), A.vals.data(), nz));
    return A;
}

}  // namespace schwarz
