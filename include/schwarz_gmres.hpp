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
//   make_poisson_2d/3d        src/mesh/poisson.h:10-74
//
// Errors surface as std::runtime_error, as in the reference.  Extra knobs
// (partition vector, factor/sweep dtypes, precision, stopping rule) are
// optional members with the reference's behaviour as default.  Only the GPU
// preconditioners of this header can be passed to gmres()/fgmres().
#pragma once

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
inline GMRESResult solve(sg_solver solver, const CSRMatrix& A, const std::vector<double>& b,
                         std::vector<double>& x, const Preconditioner* M, const GMRESParams& p) {
    const auto* dm = dynamic_cast<const DevicePreconditioner*>(M);
    if (M && !dm)
        throw std::runtime_error("only the GPU preconditioners of schwarz_gmres.hpp can be used");
    if (static_cast<int>(b.size()) != A.nrows) throw std::runtime_error("b has the wrong size");
    x.resize(A.nrows, 0.0);
    std::shared_ptr<CsrHandle> dA;
    const sg_csr* hA = dm ? dm->matrix() : nullptr;
    if (!hA) {
        dA = A.device();
        hA = dA->h;
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
    check(sg_solve(context(), solver, hA, dm ? dm->handle() : nullptr, b.data(), x.data(),
                   A.nrows, SG_MEM_HOST, &prm, &r));
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

}  // namespace schwarz
