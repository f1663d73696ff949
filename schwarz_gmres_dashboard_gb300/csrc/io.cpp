// io.cpp -- host-side file formats of the solve path: Matrix Market input
// (src/io/matrix_market.h:14-92) and the convergence record that the
// reference CLI appends to <output>.conv.jsonl for its dashboard
// (src/analysis/convergence_analysis.h:15-93, src/main.cpp:251-258).
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <string>
#include <utility>
#include <vector>

#include "sg_internal.h"

namespace sg {

namespace {

// ---------------------------------------------------------------- Matrix Market
// Reading rules of the reference reader, so that the same file gives the
// same matrix:
//  * lines opening with '%' are comments; one that mentions "symmetric" makes
//    every off-diagonal entry stand for itself and its mirror image, one that
//    mentions "pattern" means entries carry no value (read as 1.0);
//  * the first other line holds rows, columns and the number of entries,
//    then one entry per line, 1-based;
//  * duplicates are kept (not summed); rows and columns end up ascending.
// Built by bucketing: a first pass counts entries per row (mirror images
// included), a second drops each into its row's range in file order, and each
// row is then ordered by column (stable: duplicates keep file order).  Unlike
// the reference, blank lines are skipped and an index outside the declared
// size is an error rather than undefined behaviour.
struct MMEntry {
    int row, col;
    double val;
};

// the next line that is neither blank nor a comment (comments set the flags)
bool mm_content_line(std::istream& in, std::string& line, bool* sym, bool* pat) {
    while (std::getline(in, line)) {
        const size_t first = line.find_first_not_of(" \t\r");
        if (first == std::string::npos) continue;
        if (line[first] == '%') {
            if (sym && line.find("symmetric") != std::string::npos) *sym = true;
            if (pat && line.find("pattern") != std::string::npos) *pat = true;
            continue;
        }
        return true;
    }
    return false;
}

struct MMMatrix {
    int nrows = 0, ncols = 0;
    std::vector<int> rp, ci;
    std::vector<double> v;
};

MMMatrix mm_read(const char* path) {
    std::ifstream in(path);
    if (!in) fail(SG_ERR_INVALID_ARG, "cannot open Matrix Market file '%s'", path);
    bool sym = false, pat = false;
    std::string line;
    if (!mm_content_line(in, line, &sym, &pat))
        fail(SG_ERR_INVALID_ARG, "Matrix Market file '%s' has no size line", path);
    long long dims[3] = {0, 0, 0};
    {
        const char* p = line.c_str();
        for (long long& d : dims) {
            char* end = nullptr;
            d = std::strtoll(p, &end, 10);
            if (end == p) fail(SG_ERR_INVALID_ARG, "bad size line in '%s': %s", path, line.c_str());
            p = end;
        }
    }
    if (dims[0] < 0 || dims[1] < 0 || dims[2] < 0 || dims[0] > INT32_MAX || dims[1] > INT32_MAX)
        fail(SG_ERR_INVALID_ARG, "bad sizes in '%s': %s", path, line.c_str());
    MMMatrix A;
    A.nrows = (int)dims[0];
    A.ncols = (int)dims[1];
    const long long declared = dims[2];
    std::vector<MMEntry> ent;
    ent.reserve((size_t)declared);
    for (long long k = 0; k < declared; ++k) {
        if (!mm_content_line(in, line, nullptr, nullptr))
            fail(SG_ERR_INVALID_ARG, "Matrix Market file '%s' ends after %lld of %lld entries",
                 path, k, declared);
        const char* p = line.c_str();
        char* end = nullptr;
        const long r = std::strtol(p, &end, 10);
        p = end;
        const long c = std::strtol(p, &end, 10);
        p = end;
        double val = 1.0;
        if (!pat) val = std::strtod(p, &end);
        if (r < 1 || r > A.nrows || c < 1 || c > A.ncols)
            fail(SG_ERR_INVALID_ARG, "entry %lld of '%s' lies outside the declared size: %s",
                 k + 1, path, line.c_str());
        ent.push_back({(int)r - 1, (int)c - 1, val});
    }
    // row buckets: counts (mirror images included), offsets, placement
    A.rp.assign((size_t)A.nrows + 1, 0);
    for (const auto& e : ent) {
        A.rp[(size_t)e.row + 1]++;
        if (sym && e.row != e.col) A.rp[(size_t)e.col + 1]++;
    }
    for (int i = 0; i < A.nrows; ++i) A.rp[i + 1] += A.rp[i];
    const size_t total = (size_t)A.rp[A.nrows];
    if (total > (size_t)INT32_MAX) fail(SG_ERR_INVALID_ARG, "'%s' has too many entries", path);
    std::vector<int> fill(A.rp.begin(), A.rp.end() - 1);
    std::vector<std::pair<int, double>> slot(total);
    for (const auto& e : ent) {
        slot[(size_t)fill[e.row]++] = {e.col, e.val};
        if (sym && e.row != e.col) slot[(size_t)fill[e.col]++] = {e.row, e.val};
    }
    A.ci.resize(total);
    A.v.resize(total);
    for (int i = 0; i < A.nrows; ++i) {
        auto b = slot.begin() + A.rp[i], en = slot.begin() + A.rp[i + 1];
        std::stable_sort(b, en, [](const std::pair<int, double>& x,
                                   const std::pair<int, double>& y) { return x.first < y.first; });
        for (auto it = b; it != en; ++it) {
            const size_t q = (size_t)(it - slot.begin());
            A.ci[q] = it->first;
            A.v[q] = it->second;
        }
    }
    return A;
}

// ---------------------------------------------------------------- convergence
// The metrics of ConvergenceMetrics::compute (convergence_analysis.h:29-65):
// per-iteration rate (r_k / r_0)^(1/k), the mean of the last (up to) 20
// rates, and the first 20-iteration window whose relative reduction is
// below 1e-3 (stagnation).
constexpr int STAG_WINDOW = 20;
constexpr double STAG_TOL = 1e-3;

void conv_metrics(const double* h, int len, int converged, sg_convergence* m, double* rates) {
    std::memset(m, 0, sizeof(*m));
    m->converged = converged ? 1 : 0;
    m->iterations = len;
    m->stagnation_start = -1;
    if (len <= 0) return;
    m->initial_residual = h[0];
    m->final_residual = h[len - 1];
    std::vector<double> rho((size_t)len);
    for (int k = 1; k <= len; ++k) {
        const double q = h[k - 1] / (h[0] + 1e-300);
        rho[k - 1] = q > 0.0 ? std::pow(q, 1.0 / k) : 0.0;
    }
    const int tail = std::min(STAG_WINDOW, len);
    if (tail >= 2) {
        double acc = 0.0;
        for (int k = len - tail; k < len; ++k) acc += rho[k];
        m->asymptotic_rate = acc / tail;
    } else {
        m->asymptotic_rate = rho[len - 1];
    }
    for (int i = STAG_WINDOW; i < len; ++i) {
        const double a = h[i - STAG_WINDOW], b = h[i];
        if ((a - b) / (a + 1e-300) < STAG_TOL) {
            m->stagnation_start = i - STAG_WINDOW + 1;
            break;
        }
    }
    if (rates) std::copy(rho.begin(), rho.end(), rates);
}

// %.6g: the reference stream's setprecision(6) in its default float format
std::string g6(double x) {
    char buf[64];
    std::snprintf(buf, sizeof(buf), "%.6g", x);
    return buf;
}

}  // namespace

}  // namespace sg

using namespace sg;

extern "C" sg_status sg_read_matrix_market(const char* path, int* nrows, int* ncols, int* nnz,
                                           int* row_ptr, int* col_idx, double* vals, int cap) {
    try {
        SG_CHECK_ARG(path && nrows && ncols && nnz, "NULL argument");
        MMMatrix A = mm_read(path);
        *nrows = A.nrows;
        *ncols = A.ncols;
        *nnz = (int)A.ci.size();
        if (row_ptr) {
            SG_CHECK_ARG(col_idx && vals, "row_ptr given without col_idx / vals");
            SG_CHECK_ARG(cap >= *nnz, "capacity %d below the %d entries", cap, *nnz);
            std::copy(A.rp.begin(), A.rp.end(), row_ptr);
            std::copy(A.ci.begin(), A.ci.end(), col_idx);
            std::copy(A.v.begin(), A.v.end(), vals);
        }
        set_last_error("");
        return SG_OK;
    } catch (const Error& e) {
        set_last_error(e.msg.c_str());
        return e.status;
    } catch (const std::exception& e) {
        set_last_error(e.what());
        return SG_ERR_INTERNAL;
    }
}

extern "C" sg_status sg_convergence_metrics(const double* history, int len, int converged,
                                            sg_convergence* out, double* rates) {
    try {
        SG_CHECK_ARG(out && (len == 0 || history), "NULL argument");
        SG_CHECK_ARG(len >= 0, "len must be >= 0");
        conv_metrics(history, len, converged, out, rates);
        set_last_error("");
        return SG_OK;
    } catch (const Error& e) {
        set_last_error(e.msg.c_str());
        return e.status;
    }
}

extern "C" sg_status sg_write_convergence_jsonl(const char* path, const char* matrix,
                                                const char* precond, int nparts, int overlap,
                                                const double* history, int len, int converged) {
    try {
        SG_CHECK_ARG(path && matrix && precond && (len == 0 || history), "NULL argument");
        sg_convergence m;
        conv_metrics(history, len, converged, &m, nullptr);
        // one record per line, the keys and order of ConvergenceMetrics::
        // write_jsonl (convergence_analysis.h:69-93), which the dashboard reads
        std::string rec = std::string("{\"type\":\"convergence\",\"matrix\":\"") + matrix +
                          "\",\"precond\":\"" + precond + "\",\"nparts\":" +
                          std::to_string(nparts) + ",\"overlap\":" + std::to_string(overlap) +
                          ",\"iterations\":" + std::to_string(m.iterations) +
                          ",\"converged\":" + (m.converged ? "true" : "false") +
                          ",\"initial_residual\":" + g6(m.initial_residual) +
                          ",\"final_residual\":" + g6(m.final_residual) +
                          ",\"asymptotic_rate\":" + g6(m.asymptotic_rate) +
                          ",\"stagnation_start\":" + std::to_string(m.stagnation_start) +
                          ",\"residual_history\":[";
        for (int i = 0; i < len; ++i) {
            if (i) rec += ",";
            rec += g6(history[i]);
        }
        rec += "]}\n";
        std::FILE* f = std::fopen(path, "a");
        if (!f) fail(SG_ERR_INVALID_ARG, "cannot open '%s' for appending", path);
        const size_t w = std::fwrite(rec.data(), 1, rec.size(), f);
        std::fclose(f);
        if (w != rec.size()) fail(SG_ERR_INTERNAL, "short write to '%s'", path);
        set_last_error("");
        return SG_OK;
    } catch (const Error& e) {
        set_last_error(e.msg.c_str());
        return e.status;
    }
}
