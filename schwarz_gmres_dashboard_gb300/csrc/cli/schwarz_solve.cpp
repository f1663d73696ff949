// schwarz_solve -- drop-in for the reference CLI's single-rank solve path
// (src/main.cpp:37-275) on one GPU: same flags, same stdout lines
// (:245-249), same JSONL metrics record (src/io/metrics_logger.h:28-51),
// exit code 0 iff converged (:274).  No MPI: a single process drives one GPU.
//
// Reference flags kept: --matrix --poisson --precond --restart --tol
// --maxiter --fgmres --bicgstab --analyze --nparts --overlap --gpu (implied)
// --output.  Flags of the reference's ILUT preconditioner (--precond ilut,
// --drop-tol, --fill-factor), outside this solve path, are rejected with a
// message.  Added: --poisson3d N, --varcoef N, --precision fp64|mixed,
// --factor fp64|fp32|bf16, --stop ref|true_rel, --partition boxes|graph,
// --learned FILE (learned coarse stage, FGMRES), --nrhs R and --aniso-batch S
// (the batched solver), --autotune (accepted: formats are always tuned).
#include <chrono>
#include <cstdint>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iostream>
#include <sstream>
#include <string>
#include <vector>
#include <algorithm>

#include "schwarz_gmres.hpp"

using namespace schwarz;

static void usage() {
    std::cerr << "Usage: schwarz_solve [options]\n"
                 "\nMatrix source (one required):\n"
                 "  --matrix <file.mtx>      Matrix Market file\n"
                 "  --poisson <N>            N x N Poisson 2D (n = N^2)\n"
                 "  --poisson3d <N>          N^3 Poisson 3D (7-point)\n"
                 "  --varcoef <N>            N^3 -div(k grad u), k = exp(GRF), sigma 1, corr 8\n"
                 "\nPreconditioner:\n"
                 "  --precond <type>         none|jacobi|ilu0|asm|ras|twolevel_asm|twolevel_ras\n"
                 "  --factor <t>             ILU factor storage fp64|fp32|bf16 (default fp64)\n"
                 "\nSolver:\n"
                 "  --restart <m>            GMRES restart length (default 30)\n"
                 "  --tol <val>              Convergence tolerance (default 1e-10)\n"
                 "  --maxiter <n>            Max iterations (default 1000)\n"
                 "  --fgmres                 Use Flexible GMRES (right-preconditioned)\n"
                 "  --bicgstab               Use BiCGSTAB (Van der Vorst 1992), FP64\n"
                 "  --precision <p>          fp64 | mixed (FP32 inner Krylov, FP64 outer)\n"
                 "  --stop <rule>            ref (|g| < tol, the reference rule) | true_rel\n"
                 "\nDomain decomposition:\n"
                 "  --nparts <n>             Subdomains (default 4)\n"
                 "  --overlap <n>            Overlap size (default 1)\n"
                 "  --partition <p>          graph (default) | boxes (3D grids, uneven cuts)\n"
                 "\nGPU extensions:\n"
                 "  --learned <file>         learned coarse stage after the Schwarz\n"
                 "                           preconditioner (raw float32 weights,\n"
                 "                           sg_learned_num_params() of them; cubic\n"
                 "                           --varcoef/--poisson3d grids); implies --fgmres\n"
                 "  --stagnation <r>         learned stage fallback ratio (default 0.5)\n"
                 "  --nrhs <R>               solve R right-hand sides at once (b_0 = A*ones,\n"
                 "                           the rest U[-1,1]) with the batched solver\n"
                 "  --aniso-batch <S>        S anisotropic 2D systems (9-point, n in 32..256,\n"
                 "                           4-16 box subdomains each) x --nrhs (default 4)\n"
                 "                           right-hand sides, batched GMRES + RAS\n"
                 "  --autotune               accepted; SpMV format and sweep block size are\n"
                 "                           always timed at set-up\n"
                 "\nHardware:\n"
                 "  --gpu                    accepted; every solve runs on the GPU\n"
                 "\nOutput:\n"
                 "  --output <file.jsonl>    Append metrics to JSONL file\n"
                 "  --analyze                Run convergence / condition / spectral analysis\n";
}

// The batch of make_aniso_batch (schwarz_gmres_dashboard_gb300/batched.py):
// sizes n ~ U{32..256}, eps ~ LogUniform[1e-3, 1], theta ~ U[0, pi) from
// SplitMix64(seed), parts clamp(rint(n^2/4096), 4, 16), seeded boxes.
struct AnisoBatch {
    CSRMatrix A;
    std::vector<int> sys_row_ptr, part;
    int nparts = 0;
};
static AnisoBatch make_aniso_batch(int nsys, uint64_t seed) {
    std::vector<double> u(3 * (size_t)nsys);
    detail::check(sg_gen_uniform(seed, 3 * nsys, 0.0, 1.0, u.data()));
    AnisoBatch B;
    B.sys_row_ptr.push_back(0);
    std::vector<int> rp{0}, ci;
    std::vector<double> v;
    for (int s = 0; s < nsys; ++s) {
        const int n = 32 + std::min((int)(u[3 * s] * 225.0), 224);
        const double eps = std::pow(10.0, -3.0 + 3.0 * u[3 * s + 1]);
        const double theta = M_PI * u[3 * s + 2];
        const int parts = (int)std::min(16.0, std::max(4.0, std::nearbyint(n * (double)n / 4096.0)));
        int nnz = 0;
        detail::check(sg_gen_aniso2d(n, n, eps, theta, nullptr, nullptr, nullptr, &nnz));
        std::vector<int> srp(n * n + 1), sci(nnz);
        std::vector<double> sv(nnz);
        detail::check(sg_gen_aniso2d(n, n, eps, theta, srp.data(), sci.data(), sv.data(), &nnz));
        std::vector<int> sp(n * n);
        detail::check(sg_partition_boxes(n, n, 1, parts, 0.08, seed * 1000003ull + s, sp.data()));
        const int r0 = B.sys_row_ptr.back(), z0 = rp.back();
        for (int i = 1; i <= n * n; ++i) rp.push_back(z0 + srp[i]);
        for (int c : sci) ci.push_back(c + r0);
        v.insert(v.end(), sv.begin(), sv.end());
        for (int p : sp) B.part.push_back(p + B.nparts);
        B.nparts += parts;
        B.sys_row_ptr.push_back(r0 + n * n);
    }
    B.A.nrows = B.A.ncols = B.sys_row_ptr.back();
    B.A.row_ptr = std::move(rp);
    B.A.col_idx = std::move(ci);
    B.A.vals = std::move(v);
    return B;
}

static CSRMatrix make_varcoef(int N) {
    int nnz = 0;
    detail::check(sg_gen_varcoef3d(N, N, N, 1.0, 8.0, 0, nullptr, nullptr, nullptr, &nnz));
    CSRMatrix A;
    A.resize(N * N * N, N * N * N, nnz);
    detail::check(sg_gen_varcoef3d(N, N, N, 1.0, 8.0, 0, A.row_ptr.data(), A.col_idx.data(),
                                   A.vals.data(), &nnz));
    return A;
}

static void solve_batch(const CSRMatrix& A, sg_precond* pc, const std::vector<int>& sys_row_ptr,
                        int nrhs, const std::vector<double>& B, std::vector<double>& X,
                        const GMRESParams& params, std::vector<sg_batch_result>& res,
                        double& seconds) {
    auto dA = A.device();
    sg_solve_params prm{};
    prm.restart = std::min(params.restart, 32);
    prm.max_iter = params.max_iter;
    prm.tol = params.tol;
    prm.tol_kind = params.tol_kind;
    prm.precision = params.precision;
    prm.use_graph = 1;
    res.assign((size_t)(sys_row_ptr.size() - 1) * nrhs, sg_batch_result{});
    detail::check(sg_solve_batched(detail::context(), dA->h, pc, (int)sys_row_ptr.size() - 1,
                                   sys_row_ptr.data(), nrhs, B.data(), X.data(), SG_MEM_HOST, &prm,
                                   res.data(), &seconds));
}

static int report_batch(const std::vector<sg_batch_result>& res, double seconds, double t_setup,
                        const std::string& label, const std::string& matrix, int n, int nnz,
                        int nrhs, const GMRESParams& params, const std::string& output_file) {
    int conv = 0, max_it = 0;
    double sum_it = 0.0, max_rel = 0.0;
    for (const auto& r : res) {
        conv += r.converged ? 1 : 0;
        max_it = std::max(max_it, r.iterations);
        sum_it += r.iterations;
        max_rel = std::max(max_rel, r.true_rel_residual);
    }
    const bool all = conv == (int)res.size();
    std::cout << "  Converged: " << (all ? "yes" : "no") << " (" << conv << "/" << res.size()
              << ")\n"
              << "  Iterations: max " << max_it << ", mean " << sum_it / res.size() << "\n"
              << "  Setup time: " << t_setup << " s\n"
              << "  Solve time: " << seconds << " s\n"
              << "  Max true relative residual: " << max_rel << "\n";
    if (!output_file.empty()) {
        std::ofstream out(output_file, std::ios::app);
        out << std::setprecision(6) << "{\"matrix\":\"" << matrix << "\",\"method\":\"GPU_BATCHED_"
            << label << "\",\"n\":" << n << ",\"nnz\":" << nnz << ",\"nrhs\":" << nrhs
            << ",\"solves\":" << res.size() << ",\"ranks\":1,\"gpus\":1,\"restart\":"
            << std::min(params.restart, 32) << ",\"iterations\":" << max_it << ",\"tol\":"
            << params.tol << ",\"time_setup_s\":" << t_setup << ",\"time_solve_s\":" << seconds
            << std::scientific << ",\"true_rel_residual\":" << max_rel << "}\n";
    }
    return all ? 0 : 1;
}

// R right-hand sides of one system through the batched solver
static int run_multi_rhs(const CSRMatrix& A, DevicePreconditioner* M, int nrhs,
                         const GMRESParams& params, const std::string& precond,
                         const std::string& matrix, const std::string& output_file, double t_setup) {
    const int n = A.nrows;
    std::vector<double> B((size_t)nrhs * n), X((size_t)nrhs * n, 0.0), ones(n, 1.0), b0(n);
    A.spmv(ones, b0);
    std::copy(b0.begin(), b0.end(), B.begin());
    if (nrhs > 1) detail::check(sg_gen_uniform(1000, (nrhs - 1) * n, -1.0, 1.0, B.data() + n));
    std::cout << "Solving " << nrhs << " right-hand sides with batched GMRES("
              << std::min(params.restart, 32) << ") + " << precond << "\n";
    std::vector<sg_batch_result> res;
    double seconds = 0.0;
    const std::vector<int> rows{0, n};
    solve_batch(A, M ? M->handle() : nullptr, rows, nrhs, B, X, params, res, seconds);
    return report_batch(res, seconds, t_setup, precond, matrix, n, A.nnz(), nrhs, params,
                        output_file);
}

// the anisotropic batch: RAS with FP32 factors and sweeps, FP32 Krylov,
// FP64 true relative residual <= tol (default 1e-8)
static int run_aniso_batch(int nsys, int nrhs, GMRESParams params, const std::string& output_file) {
    std::cout << "Generating " << nsys << " anisotropic 2D systems\n";
    AnisoBatch P = make_aniso_batch(nsys, 0);
    std::cout << "  n=" << P.A.nrows << "  nnz=" << P.A.nnz() << "  subdomains=" << P.nparts
              << "\n";
    auto t0 = std::chrono::high_resolution_clock::now();
    RASPrecond M(P.nparts, 1);
    M.set_precision(SG_FP32, SG_FP32);
    M.set_partition(P.part);
    M.setup(P.A);
    const double t_setup =
        std::chrono::duration<double>(std::chrono::high_resolution_clock::now() - t0).count();
    if (params.tol == 1e-10) params.tol = 1e-8;
    params.tol_kind = SG_TOL_TRUE_REL;
    params.precision = SG_FP32;
    const int n = P.A.nrows;
    std::vector<double> B((size_t)nrhs * n), X((size_t)nrhs * n, 0.0);
    detail::check(sg_gen_uniform(1000, nrhs * n, -1.0, 1.0, B.data()));
    std::cout << "Solving " << nsys << " x " << nrhs << " systems with batched GMRES("
              << std::min(params.restart, 32) << ") + ras\n";
    std::vector<sg_batch_result> res;
    double seconds = 0.0;
    solve_batch(P.A, M.handle(), P.sys_row_ptr, nrhs, B, X, params, res, seconds);
    return report_batch(res, seconds, t_setup, "ras", "aniso_batch_" + std::to_string(nsys), n,
                        P.A.nnz(), nrhs, params, output_file);
}

int main(int argc, char** argv) {
    std::string matrix_file, precond_type = "ilu0", output_file, precision = "fp64",
                factor = "fp64", stop = "ref", partition = "graph";
    GMRESParams params;
    int overlap = 1, nparts = 4, poisson_n = 0, poisson3d_n = 0, varcoef_n = 0;
    int nrhs = 1, aniso_batch = 0;
    double stagnation = 0.5;
    std::string learned_file;
    bool use_fgmres = false;
    bool use_bicgstab = false;
    bool run_analysis = false;
    for (int i = 1; i < argc; ++i) {
        auto is = [&](const char* f) { return !std::strcmp(argv[i], f); };
        auto more = [&] { return i + 1 < argc; };
        if (is("--matrix") && more()) matrix_file = argv[++i];
        else if (is("--precond") && more()) precond_type = argv[++i];
        else if (is("--restart") && more()) params.restart = std::atoi(argv[++i]);
        else if (is("--tol") && more()) params.tol = std::atof(argv[++i]);
        else if (is("--maxiter") && more()) params.max_iter = std::atoi(argv[++i]);
        else if (is("--overlap") && more()) overlap = std::atoi(argv[++i]);
        else if (is("--nparts") && more()) nparts = std::atoi(argv[++i]);
        else if (is("--output") && more()) output_file = argv[++i];
        else if (is("--gpu")) {
        } else if (is("--fgmres")) use_fgmres = true;
        else if (is("--bicgstab")) use_bicgstab = true;
        else if (is("--analyze")) run_analysis = true;
        else if (is("--poisson") && more()) poisson_n = std::atoi(argv[++i]);
        else if (is("--poisson3d") && more()) poisson3d_n = std::atoi(argv[++i]);
        else if (is("--varcoef") && more()) varcoef_n = std::atoi(argv[++i]);
        else if (is("--precision") && more()) precision = argv[++i];
        else if (is("--factor") && more()) factor = argv[++i];
        else if (is("--stop") && more()) stop = argv[++i];
        else if (is("--partition") && more()) partition = argv[++i];
        else if (is("--learned") && more()) learned_file = argv[++i];
        else if (is("--stagnation") && more()) stagnation = std::atof(argv[++i]);
        else if (is("--nrhs") && more()) nrhs = std::atoi(argv[++i]);
        else if (is("--aniso-batch") && more()) aniso_batch = std::atoi(argv[++i]);
        else if (is("--autotune")) {
        }
        else if (is("--drop-tol") || is("--fill-factor")) {
            std::cerr << "schwarz_solve: " << argv[i]
                      << " belongs to a reference feature outside the GPU solve path\n";
            return 1;
        } else {
            usage();
            return 1;
        }
    }
    if (matrix_file.empty() && poisson_n <= 0 && poisson3d_n <= 0 && varcoef_n <= 0 &&
        aniso_batch <= 0) {
        usage();
        return 1;
    }
    if (nrhs < 1) {
        std::cerr << "schwarz_solve: --nrhs must be >= 1\n";
        return 1;
    }
    try {
        if (aniso_batch > 0)
            return run_aniso_batch(aniso_batch, nrhs == 1 ? 4 : nrhs, params, output_file);
        CSRMatrix A;
        int gx = 0;  // grid edge for --partition boxes
        if (poisson_n > 0) {
            std::cout << "Generating Poisson2D " << poisson_n << "x" << poisson_n << "\n";
            A = make_poisson_2d(poisson_n, poisson_n);
            if (matrix_file.empty()) matrix_file = "poisson2d_" + std::to_string(poisson_n);
        } else if (poisson3d_n > 0) {
            std::cout << "Generating Poisson3D " << poisson3d_n << "^3\n";
            A = make_poisson_3d(poisson3d_n, poisson3d_n, poisson3d_n);
            gx = poisson3d_n;
            matrix_file = "poisson3d_" + std::to_string(poisson3d_n);
        } else if (varcoef_n > 0) {
            std::cout << "Generating variable-coefficient 3D " << varcoef_n << "^3\n";
            A = make_varcoef(varcoef_n);
            gx = varcoef_n;
            matrix_file = "varcoef3d_" + std::to_string(varcoef_n);
        } else {
            std::cout << "Loading matrix: " << matrix_file << "\n";
            A = read_matrix_market(matrix_file);
        }
        std::cout << "  n=" << A.nrows << "  nnz=" << A.nnz() << "\n";
        const int n = A.nrows;
        // b = A * ones, x0 = 0 (src/main.cpp:153-155, :228)
        std::vector<double> x_exact(n, 1.0), b(n);
        A.spmv(x_exact, b);

        const sg_dtype fdt = factor == "bf16" ? SG_BF16 : factor == "fp32" ? SG_FP32 : SG_FP64;
        const bool mixed = precision == "mixed";
        std::unique_ptr<DevicePreconditioner> M;
        auto t0 = std::chrono::high_resolution_clock::now();
        if (precond_type == "jacobi") M.reset(new JacobiPrecond());
        else if (precond_type == "ilu0") M.reset(new ILU0Precond());
        else if (precond_type == "asm") M.reset(new ASMPrecond(nparts, overlap));
        else if (precond_type == "ras") M.reset(new RASPrecond(nparts, overlap));
        else if (precond_type == "twolevel_asm")
            M.reset(new TwoLevelSchwarzPrecond(nparts, overlap, FineLevelType::ASM));
        else if (precond_type == "twolevel_ras")
            M.reset(new TwoLevelSchwarzPrecond(nparts, overlap, FineLevelType::RAS));
        else if (precond_type == "ilut") {
            std::cerr << "schwarz_solve: ilut is outside the GPU solve path\n";
            return 1;
        }
        // an unknown --precond leaves M empty, as in src/main.cpp:190-208
        if (M) {
            if (fdt != SG_FP64 || mixed)
                M->set_precision(fdt == SG_FP64 ? SG_FP32 : fdt, SG_FP32);
            if (partition == "boxes" && gx > 0) {
                std::vector<int> part(n);
                detail::check(sg_partition_boxes(gx, gx, gx, nparts, 0.08, 1, part.data()));
                M->set_partition(part);
            }
            M->setup(A);
        }
        auto t1 = std::chrono::high_resolution_clock::now();
        const double t_setup = std::chrono::duration<double>(t1 - t0).count();

        params.precision = mixed ? SG_FP32 : SG_FP64;
        params.tol_kind = stop == "true_rel" ? SG_TOL_TRUE_REL : SG_TOL_REF_ABS;
        if (nrhs > 1) return run_multi_rhs(A, M.get(), nrhs, params, precond_type, matrix_file,
                                           output_file, t_setup);
        // learned coarse stage: weights from a raw float32 file
        sg_learned* L = nullptr;
        struct LearnedGuard {
            sg_learned*& L;
            ~LearnedGuard() {
                if (L) sg_learned_destroy(L);
            }
        } lguard{L};
        if (!learned_file.empty()) {
            if (gx <= 0 || !M)
                throw std::runtime_error("--learned needs --varcoef/--poisson3d and a Schwarz --precond");
            std::vector<float> w(sg_learned_num_params());
            std::ifstream in(learned_file, std::ios::binary);
            if (!in.read(reinterpret_cast<char*>(w.data()), (std::streamsize)(w.size() * sizeof(float))))
                throw std::runtime_error("cannot read " + std::to_string(w.size()) +
                                         " float32 weights from " + learned_file);
            detail::check(sg_learned_create(detail::context(), gx, gx, gx, &L));
            detail::check(sg_learned_set_weights(L, w.data(), (int)w.size()));
            detail::check(sg_learned_set_matrix(L, M->matrix()));
            detail::check(sg_precond_set_learned(M->handle(), L, stagnation));
            use_fgmres = true;
            std::cout << "Learned stage: " << learned_file << "\n";
        }
        // pre-solve analysis (src/main.cpp:213-224): Lanczos condition
        // estimates of A and M^{-1}A, power-iteration spectral radius of
        // I - M^{-1}A, all on the GPU
        if (run_analysis && M) {
            std::cout << "\n--- Pre-solve analysis ---\n";
            print_condition_estimate(estimate_condition(A, nullptr, 80), "A (unpreconditioned)");
            print_condition_estimate(estimate_condition(A, M.get(), 80),
                                     "M^{-1}A (preconditioned)");
            print_spectral_result(estimate_spectral_radius(A, M.get(), 300), precond_type);
            std::cout << "\n";
        }
        std::vector<double> x(n, 0.0);
        if (use_bicgstab && L)
            throw std::runtime_error("--bicgstab takes no learned stage (it needs FGMRES)");
        const std::string label = use_bicgstab ? std::string("BiCGSTAB")
                                               : (use_fgmres ? "FGMRES(" : "GMRES(") +
                                                     std::to_string(params.restart) + ")";
        std::cout << "Solving with " << label << " + " << precond_type << "\n";
        if (use_bicgstab) params.precision = SG_FP64;
        GMRESResult res = use_bicgstab ? bicgstab(A, b, x, M.get(), params)
                          : use_fgmres ? fgmres(A, b, x, M.get(), params)
                                       : gmres(A, b, x, M.get(), params);
        std::cout << "  Converged: " << (res.converged ? "yes" : "no") << "\n"
                  << "  Iterations: " << res.iterations << "\n"
                  << "  Residual: " << res.residual_norm << "\n"
                  << "  Setup time: " << t_setup << " s\n"
                  << "  Solve time: " << res.time_solve_s << " s\n"
                  << "  True relative residual: " << res.true_rel_residual << "\n";
        if (L) {
            int on = 0, fb = -1;
            long long applies = 0;
            detail::check(sg_learned_get_state(L, &on, &fb, &applies));
            std::cout << "  Learned stage: "
                      << (fb >= 0 ? "fell back after cycle " + std::to_string(fb) : std::string("on"))
                      << " (" << applies << " applies)\n";
        }
        // post-solve convergence analysis and its .conv.jsonl record
        // (src/main.cpp:251-258)
        if (run_analysis) {
            const ConvergenceMetrics ca = analyze_convergence(res.residual_history, res.converged);
            ca.print_summary();
            if (!output_file.empty())
                ca.write_jsonl(output_file + ".conv.jsonl", matrix_file, precond_type, nparts,
                               overlap);
        }
        if (!output_file.empty()) {
            // the Metrics record of src/io/metrics_logger.h:28-51, plus extras
            std::ofstream out(output_file, std::ios::app);
            out << std::setprecision(6) << "{\"matrix\":\"" << matrix_file << "\","
                << "\"method\":\""
                << (use_bicgstab ? "GPU_BiCGSTAB+" : use_fgmres ? "GPU_FGMRES+" : "GPU_GMRES+")
                << precond_type
                << "\",\"n\":" << n << ",\"nnz\":" << A.nnz() << ",\"ranks\":1,\"threads\":1,"
                << "\"gpus\":1,\"overlap\":" << overlap << ",\"restart\":" << params.restart
                << ",\"iterations\":" << res.iterations << ",\"tol\":" << params.tol
                << ",\"residual_norm\":" << std::scientific << res.residual_norm << std::fixed
                << ",\"time_setup_s\":" << t_setup << ",\"time_solve_s\":" << res.time_solve_s
                << ",\"speedup\":" << 1.0 << ",\"efficiency\":" << 1.0 << std::scientific
                << ",\"true_rel_residual\":" << res.true_rel_residual << ",\"precision\":\""
                << precision << "\"}\n";
        }
        return res.converged ? 0 : 1;
    } catch (const std::exception& e) {
        std::cerr << "schwarz_solve: " << e.what() << "\n";
        return 2;
    }
}
