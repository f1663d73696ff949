// schwarz_solve -- drop-in for the reference CLI's single-rank solve path
// (src/main.cpp:37-275) on one GPU: same flags, same stdout lines
// (:245-249), same JSONL metrics record (src/io/metrics_logger.h:28-51),
// exit code 0 iff converged (:274).  No MPI: a single process drives one GPU.
//
// Reference flags kept: --matrix --poisson --precond --restart --tol
// --maxiter --fgmres --nparts --overlap --gpu (implied) --output.
// Flags of reference features outside this solve path (--precond ilut,
// --drop-tol, --fill-factor, --bicgstab, --analyze) are rejected with a
// message.  Added: --poisson3d N, --varcoef N, --precision fp64|mixed,
// --factor fp64|fp32|bf16, --stop ref|true_rel, --partition boxes|graph.
#include <chrono>
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
                 "  --precision <p>          fp64 | mixed (FP32 inner Krylov, FP64 outer)\n"
                 "  --stop <rule>            ref (|g| < tol, the reference rule) | true_rel\n"
                 "\nDomain decomposition:\n"
                 "  --nparts <n>             Subdomains (default 4)\n"
                 "  --overlap <n>            Overlap size (default 1)\n"
                 "  --partition <p>          graph (default) | boxes (3D grids, uneven cuts)\n"
                 "\nHardware:\n"
                 "  --gpu                    accepted; every solve runs on the GPU\n"
                 "\nOutput:\n"
                 "  --output <file.jsonl>    Append metrics to JSONL file\n";
}

// Matrix Market reader with the semantics of src/io/matrix_market.h:14-92
// (symmetric entries mirrored, pattern files read as 1.0, entries sorted by
// row then column, duplicates kept).
static CSRMatrix read_matrix_market(const std::string& filename) {
    std::ifstream in(filename);
    if (!in.is_open()) throw std::runtime_error("Cannot open file: " + filename);
    std::string line;
    bool symmetric = false, pattern = false;
    while (std::getline(in, line)) {
        if (!line.empty() && line[0] == '%') {
            if (line.find("symmetric") != std::string::npos) symmetric = true;
            if (line.find("pattern") != std::string::npos) pattern = true;
            continue;
        }
        break;
    }
    int nrows = 0, ncols = 0, nnz = 0;
    {
        std::istringstream iss(line);
        iss >> nrows >> ncols >> nnz;
    }
    struct T {
        int r, c;
        double v;
    };
    std::vector<T> e;
    e.reserve(symmetric ? 2 * (size_t)nnz : (size_t)nnz);
    for (int k = 0; k < nnz; ++k) {
        if (!std::getline(in, line)) throw std::runtime_error("Premature end of file");
        std::istringstream iss(line);
        int r, c;
        double v = 1.0;
        iss >> r >> c;
        if (!pattern) iss >> v;
        --r;
        --c;
        e.push_back({r, c, v});
        if (symmetric && r != c) e.push_back({c, r, v});
    }
    std::sort(e.begin(), e.end(), [](const T& a, const T& b) {
        return a.r < b.r || (a.r == b.r && a.c < b.c);
    });
    CSRMatrix A;
    A.nrows = nrows;
    A.ncols = ncols;
    A.row_ptr.assign(nrows + 1, 0);
    A.col_idx.resize(e.size());
    A.vals.resize(e.size());
    for (auto& t : e) A.row_ptr[t.r + 1]++;
    for (int i = 0; i < nrows; ++i) A.row_ptr[i + 1] += A.row_ptr[i];
    std::vector<int> pos(A.row_ptr.begin(), A.row_ptr.end());
    for (auto& t : e) {
        const int p = pos[t.r]++;
        A.col_idx[p] = t.c;
        A.vals[p] = t.v;
    }
    return A;
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

int main(int argc, char** argv) {
    std::string matrix_file, precond_type = "ilu0", output_file, precision = "fp64",
                factor = "fp64", stop = "ref", partition = "graph";
    GMRESParams params;
    int overlap = 1, nparts = 4, poisson_n = 0, poisson3d_n = 0, varcoef_n = 0;
    bool use_fgmres = false;
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
        else if (is("--poisson") && more()) poisson_n = std::atoi(argv[++i]);
        else if (is("--poisson3d") && more()) poisson3d_n = std::atoi(argv[++i]);
        else if (is("--varcoef") && more()) varcoef_n = std::atoi(argv[++i]);
        else if (is("--precision") && more()) precision = argv[++i];
        else if (is("--factor") && more()) factor = argv[++i];
        else if (is("--stop") && more()) stop = argv[++i];
        else if (is("--partition") && more()) partition = argv[++i];
        else if (is("--bicgstab") || is("--analyze") || is("--drop-tol") || is("--fill-factor")) {
            std::cerr << "schwarz_solve: " << argv[i]
                      << " belongs to a reference feature outside the GPU solve path\n";
            return 1;
        } else {
            usage();
            return 1;
        }
    }
    if (matrix_file.empty() && poisson_n <= 0 && poisson3d_n <= 0 && varcoef_n <= 0) {
        usage();
        return 1;
    }
    try {
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
        std::vector<double> x(n, 0.0);
        const std::string label = (use_fgmres ? "FGMRES(" : "GMRES(") +
                                  std::to_string(params.restart) + ")";
        std::cout << "Solving with " << label << " + " << precond_type << "\n";
        GMRESResult res = use_fgmres ? fgmres(A, b, x, M.get(), params)
                                     : gmres(A, b, x, M.get(), params);
        std::cout << "  Converged: " << (res.converged ? "yes" : "no") << "\n"
                  << "  Iterations: " << res.iterations << "\n"
                  << "  Residual: " << res.residual_norm << "\n"
                  << "  Setup time: " << t_setup << " s\n"
                  << "  Solve time: " << res.time_solve_s << " s\n"
                  << "  True relative residual: " << res.true_rel_residual << "\n";
        if (!output_file.empty()) {
            // the Metrics record of src/io/metrics_logger.h:28-51, plus extras
            std::ofstream out(output_file, std::ios::app);
            out << std::setprecision(6) << "{\"matrix\":\"" << matrix_file << "\","
                << "\"method\":\"" << (use_fgmres ? "GPU_FGMRES+" : "GPU_GMRES+") << precond_type
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
