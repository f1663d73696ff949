// Drop-in check of include/schwarz_gmres.hpp with caller-side plug-ins:
// a Preconditioner subclass of the caller's own (applied on the host inside
// the GPU solve), fgmres_flex with a FlexApply, bicgstab, the analysis calls
// and read_matrix_market -- code written against the reference's headers.
// Prints one "key value" line per result; the test reads them.
#include <cmath>
#include <cstdio>
#include <vector>

#include "schwarz_gmres.hpp"

using namespace schwarz;

// Jacobi written as a caller would write a Preconditioner plug-in
// (src/precond/preconditioner.h:7-20): host arrays, overwrites all of y.
class HostJacobi : public Preconditioner {
public:
    void setup(const CSRMatrix& A) override {
        inv_.assign(A.nrows, 1.0);
        for (int i = 0; i < A.nrows; ++i)
            for (int e = A.row_ptr[i]; e < A.row_ptr[i + 1]; ++e)
                if (A.col_idx[e] == i && std::fabs(A.vals[e]) > 1e-15) inv_[i] = 1.0 / A.vals[e];
    }
    void apply(const double* x, double* y, int n) const override {
        ++calls;
        for (int i = 0; i < n; ++i) y[i] = inv_[i] * x[i];
    }
    mutable long calls = 0;

private:
    std::vector<double> inv_;
};

class Throwing : public Preconditioner {
public:
    void setup(const CSRMatrix&) override {}
    void apply(const double*, double*, int) const override {
        throw std::runtime_error("plug-in failure 42");
    }
};

int main(int argc, char** argv) {
    const CSRMatrix A = make_poisson_2d(24, 24);
    const int n = A.nrows;
    std::vector<double> ones(n, 1.0), b(n);
    A.spmv(ones, b);
    GMRESParams p;
    p.restart = 30;
    p.max_iter = 1000;
    p.tol = 1e-10;

    auto err = [&](const std::vector<double>& x) {
        double e = 0.0;
        for (int i = 0; i < n; ++i) e = std::fmax(e, std::fabs(x[i] - 1.0));
        return e;
    };
    // the caller's plug-in through gmres(), against the GPU Jacobi
    HostJacobi hj;
    hj.setup(A);
    std::vector<double> x(n, 0.0);
    GMRESResult r = gmres(A, b, x, &hj, p);
    std::printf("plugin_gmres %d %d %.3e %ld\n", r.converged ? 1 : 0, r.iterations, err(x), hj.calls);
    JacobiPrecond gj;
    gj.setup(A);
    std::vector<double> xg(n, 0.0);
    GMRESResult rg = gmres(A, b, xg, &gj, p);
    std::printf("device_gmres %d %d %.3e\n", rg.converged ? 1 : 0, rg.iterations, err(xg));
    // fgmres_flex with a lambda (the same Jacobi), and with a nonlinear apply
    std::vector<double> xf(n, 0.0);
    GMRESResult rf = fgmres_flex(A, b, xf, [&](const double* v, double* z, int m) {
        hj.apply(v, z, m);
    }, p);
    std::printf("flex_fgmres %d %d %.3e\n", rf.converged ? 1 : 0, rf.iterations, err(xf));
    std::vector<double> xdf(n, 0.0);
    GMRESResult rdf = fgmres(A, b, xdf, &gj, p);
    std::printf("device_fgmres %d %d %.3e\n", rdf.converged ? 1 : 0, rdf.iterations, err(xdf));
    std::vector<double> xn(n, 0.0);
    int sweeps = 0;
    GMRESResult rn = fgmres_flex(A, b, xn, [&](const double* v, double* z, int m) {
        // a few Jacobi sweeps on A z = v: nonlinear in the iteration count
        // (host arithmetic only: the apply runs on a CUDA host-function
        // thread and must not call CUDA)
        ++sweeps;
        std::vector<double> t(m, 0.0), az(m);
        for (int it = 0; it < 1 + sweeps % 3; ++it) {
            for (int i = 0; i < m; ++i) {
                double acc = 0.0;
                for (int e = A.row_ptr[i]; e < A.row_ptr[i + 1]; ++e)
                    acc += A.vals[e] * t[A.col_idx[e]];
                az[i] = acc;
            }
            for (int i = 0; i < m; ++i) t[i] += 0.25 * (v[i] - az[i]);
        }
        for (int i = 0; i < m; ++i) z[i] = t[i];
    }, p);
    std::printf("flex_nonlinear %d %d %.3e\n", rn.converged ? 1 : 0, rn.iterations, err(xn));
    // BiCGSTAB with the plug-in and with the GPU ILU(0)
    std::vector<double> xb(n, 0.0);
    GMRESResult rb = bicgstab(A, b, xb, &hj, p);
    std::printf("plugin_bicgstab %d %d %.3e\n", rb.converged ? 1 : 0, rb.iterations, err(xb));
    ILU0Precond ilu;
    ilu.setup(A);
    std::vector<double> xi(n, 0.0);
    GMRESResult ri = bicgstab(A, b, xi, &ilu, p);
    std::printf("device_bicgstab %d %d %.3e\n", ri.converged ? 1 : 0, ri.iterations, err(xi));
    // analysis on the plug-in and on the device preconditioner
    ConditionEstimate c1 = estimate_condition(A, &hj, 80);
    ConditionEstimate c2 = estimate_condition(A, &gj, 80);
    std::printf("condition %.12e %.12e %.12e %.12e %d\n", c1.lambda_min, c1.lambda_max,
                c2.lambda_min, c2.lambda_max, c1.lanczos_steps);
    SpectralResult s1 = estimate_spectral_radius(A, &ilu, 200);
    std::printf("spectral %.12e %d %d\n", s1.spectral_radius, s1.power_iters,
                s1.convergence_ok ? 1 : 0);
    ConvergenceMetrics cm = analyze_convergence(r.residual_history, r.converged);
    std::printf("convergence %d %.6e\n", cm.iterations, cm.asymptotic_rate);
    // a plug-in that throws: the message comes back as std::runtime_error
    Throwing bad;
    std::vector<double> xt(n, 0.0);
    try {
        gmres(A, b, xt, &bad, p);
        std::printf("throw none\n");
    } catch (const std::runtime_error& e) {
        std::printf("throw %s\n", e.what());
    }
    if (argc > 1) {
        CSRMatrix M = read_matrix_market(argv[1]);
        std::printf("mtx %d %d %d\n", M.nrows, M.ncols, M.nnz());
    }
    return 0;
}
