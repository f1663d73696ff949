// api.cpp -- the C ABI of libsgmres (declared in include/sgmres.h).  Every
// entry point validates its arguments, runs on the context's device and
// stream, and turns internal failures into an sg_status plus a thread-local
// message.
#include <atomic>
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstring>
#include <exception>
#include <new>
#include <string>

#include "kernels.h"
#include "sg_internal.h"

namespace sg {
uint64_t next_object_gen() {
    static std::atomic<uint64_t> g{0};
    return ++g;
}
}  // namespace sg

namespace sg {

// The last error message of this thread.  A fixed buffer rather than a
// std::string: thread_local objects with destructors are destroyed before
// static ones at exit, and a caller that releases its objects from a static
// destructor (a context kept in a static smart pointer, say) would otherwise
// write into the freed string.
struct LastError {
    char msg[1024];
    void set(const char* m) {
        size_t k = 0;
        if (m)
            for (; m[k] && k + 1 < sizeof(msg); ++k) msg[k] = m[k];
        msg[k] = '\0';
    }
    void clear() { msg[0] = '\0'; }
};
static thread_local LastError g_last_error{};

void set_last_error(const char* msg) { g_last_error.set(msg); }

void fail(sg_status st, const char* fmt, ...) {
    char buf[1024];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    throw Error{st, buf};
}

// defined in setup.cpp / solver.cu
void build_schwarz_host(sg_precond* pc, const sg_csr* A, const int* part, int nparts, int overlap);
bool build_schwarz_device(sg_precond* pc, const sg_csr* A, const int* part, int nparts,
                          int overlap);
void partition_graph(int n, const int* rp, const int* ci, int nparts, int* part);
void partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed, int* part);
int gen_poisson2d(int nx, int ny, int* rp, int* ci, double* v);
int gen_poisson3d(int nx, int ny, int nz, int* rp, int* ci, double* v);
int gen_varcoef3d(int nx, int ny, int nz, double sigma, double corr, uint64_t seed, int* rp, int* ci,
                  double* v);
void gen_uniform(uint64_t seed, int n, double lo, double hi, double* out);
int gen_aniso2d(int nx, int ny, double eps, double theta, int* rp, int* ci, double* v);
int sell_variant_count();
int sell_variant_info(int variant, int what);
void solve_device(sg_ctx* ctx, int solver, const sg_csr* A, sg_precond* pc, const double* b,
                  double* x, const sg_solve_params& prm, sg_solve_result* res);

template <class F>
static sg_status guard(F&& f) {
    try {
        f();
        g_last_error.clear();
        return SG_OK;
    } catch (const Error& e) {
        g_last_error.set(e.msg.c_str());
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error.set("host allocation failed");
        return SG_ERR_OOM;
    } catch (const std::exception& e) {
        g_last_error.set(e.what());
        return SG_ERR_INTERNAL;
    } catch (...) {
        g_last_error.set("unknown internal error");
        return SG_ERR_INTERNAL;
    }
}

static void use_device(const sg_ctx* ctx) { SG_CUDA(cudaSetDevice(ctx->device)); }

}  // namespace sg

using namespace sg;

void sg_csr::ensure_fp32() {
    if (val32.p) return;
    std::vector<float> v32(h_val.size() + 16, 0.0f);
    for (size_t i = 0; i < h_val.size(); ++i) v32[i] = (float)h_val[i];
    val32.upload(v32, ctx->stream);
    if (sell_ok) {
        // FP32 copy of the SELL values (same slice layout)
        std::vector<double> sv(sell_entries);
        SG_CUDA(cudaMemcpyAsync(sv.data(), sl_val.p, sizeof(double) * sell_entries,
                                cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        std::vector<float> s32(sell_entries);
        for (long long i = 0; i < sell_entries; ++i) s32[i] = (float)sv[i];
        sl_val32.upload(s32, ctx->stream);
    }
    SG_CUDA(cudaStreamSynchronize(ctx->stream));
}

// SELL-32 copy (slices of 32 rows, slice-major, padded per slice).  Kept only
// when the padding stays under 25% of the nonzeros.
void sg_csr::build_sell() {
    sell_ok = false;
    if (nrows <= 0 || nrows != ncols) return;
    nslices = (nrows + 31) / 32;
    std::vector<long long> ptr(nslices + 1, 0);
    std::vector<int> w(nslices, 0);
    for (int s = 0; s < nslices; ++s) {
        int mw = 0;
        for (int r = s * 32; r < std::min(nrows, s * 32 + 32); ++r)
            mw = std::max(mw, h_rp[r + 1] - h_rp[r]);
        w[s] = mw;
        ptr[s + 1] = ptr[s] + 32ll * mw;
    }
    sell_entries = ptr[nslices];
    sell_maxw = 0;
    for (int s = 0; s < nslices; ++s) sell_maxw = std::max(sell_maxw, w[s]);
    if (sell_entries > (long long)nnz + nnz / 4 + 64 || sell_entries >= (1ll << 31)) return;
    std::vector<int> col(sell_entries > 0 ? sell_entries : 1, 0);
    std::vector<double> val(sell_entries > 0 ? sell_entries : 1, 0.0);
    for (int s = 0; s < nslices; ++s)
        for (int lane = 0; lane < 32; ++lane) {
            const int r = s * 32 + lane;
            int k = 0;
            if (r < nrows)
                for (int e = h_rp[r]; e < h_rp[r + 1]; ++e, ++k) {
                    col[ptr[s] + 32ll * k + lane] = h_ci[e];
                    val[ptr[s] + 32ll * k + lane] = h_val[e];
                }
            for (; k < w[s]; ++k) {
                col[ptr[s] + 32ll * k + lane] = r < nrows ? r : 0;
                val[ptr[s] + 32ll * k + lane] = 0.0;
            }
        }
    sl_ptr.upload(ptr, ctx->stream);
    sl_w.upload(w, ctx->stream);
    sl_col.upload(col, ctx->stream);
    sl_val.upload(val, ctx->stream);
    // 16-bit column offsets when every |column - row| fits (banded matrices)
    sl_dcol.release();
    {
        bool fits = true;
        std::vector<int16_t> dcol(col.size());
        for (int s = 0; s < nslices && fits; ++s)
            for (long long e = ptr[s]; e < ptr[s + 1]; ++e) {
                const int r = s * 32 + (int)((e - ptr[s]) % 32);
                const long long d = (long long)col[e] - (r < nrows ? r : 0);
                if (r >= nrows) {
                    // lanes past the last row: result never stored; point the
                    // load at row n-1 (offset >= -31)
                    dcol[e] = (int16_t)((nrows - 1) - r);
                    continue;
                }
                if (d < -32768 || d > 32767) {
                    fits = false;
                    break;
                }
                dcol[e] = (int16_t)d;
            }
        if (fits) sl_dcol.upload(dcol, ctx->stream);
    }
    sell_ok = true;
}

extern "C" {

int sg_abi_version(void) { return SG_ABI_VERSION; }

const char* sg_last_error(void) { return g_last_error.msg; }

const char* sg_status_string(sg_status st) {
    switch (st) {
    case SG_OK: return "ok";
    case SG_ERR_INVALID_ARG: return "invalid argument";
    case SG_ERR_CUDA: return "CUDA error";
    case SG_ERR_OOM: return "out of memory";
    case SG_ERR_SINGULAR: return "singular";
    case SG_ERR_NOT_SETUP: return "not set up";
    case SG_ERR_NONFINITE: return "non-finite value";
    case SG_ERR_DEVICE_TIMEOUT: return "device wait timed out";
    case SG_ERR_UNSUPPORTED: return "unsupported";
    case SG_ERR_INTERNAL: return "internal error";
    case SG_ERR_CALLBACK: return "host callback error";
    }
    return "unknown status";
}

sg_status sg_ctx_create(int device, sg_ctx** out) {
    return guard([&] {
        SG_CHECK_ARG(out, "out is NULL");
        *out = nullptr;
        int count = 0;
        cudaError_t e = cudaGetDeviceCount(&count);
        if (e != cudaSuccess || count == 0)
            fail(SG_ERR_CUDA, "no CUDA device available (%s)",
                 e != cudaSuccess ? cudaGetErrorString(e) : "0 devices");
        SG_CHECK_ARG(device >= 0 && device < count, "device %d out of range [0,%d)", device, count);
        auto* ctx = new sg_ctx();
        try {
            ctx->device = device;
            SG_CUDA(cudaSetDevice(device));
            SG_CUDA(cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, device));
            SG_CUDA(cudaStreamCreateWithFlags(&ctx->own_stream, cudaStreamNonBlocking));
            ctx->stream = ctx->own_stream;
            ctx->partials.alloc((size_t)ctx->num_sms * 8 * 40);
            ctx->counter.alloc(4);
            ctx->counter.zero(ctx->stream);
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            delete ctx;
            throw;
        }
        *out = ctx;
    });
}

sg_status sg_ctx_destroy(sg_ctx* ctx) {
    return guard([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        if (ctx->stream) cudaStreamSynchronize(ctx->stream);
        delete ctx->work;
        ctx->work = nullptr;
        destroy_batch_work(ctx->batch);
        ctx->batch = nullptr;
        collect_timers(ctx);
        for (cudaEvent_t e : ctx->ev_pool) cudaEventDestroy(e);
        ctx->ev_pool.clear();
        ctx->partials.release();
        ctx->counter.release();
        ctx->hist.release();
        if (ctx->own_stream) cudaStreamDestroy(ctx->own_stream);
        delete ctx;
    });
}

sg_status sg_ctx_set_stream(sg_ctx* ctx, void* stream) {
    return guard([&] {
        SG_CHECK_ARG(ctx, "ctx is NULL");
        use_device(ctx);
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->stream = stream ? static_cast<cudaStream_t>(stream) : ctx->own_stream;
    });
}

sg_status sg_ctx_get_stream(sg_ctx* ctx, void** stream) {
    return guard([&] {
        SG_CHECK_ARG(ctx && stream, "NULL argument");
        *stream = ctx->stream;
    });
}

sg_status sg_ctx_get_launch_count(sg_ctx* ctx, long long* count) {
    return guard([&] {
        SG_CHECK_ARG(ctx && count, "NULL argument");
        *count = ctx->launches;
    });
}

sg_status sg_ctx_get_capture_count(sg_ctx* ctx, long long* count) {
    return guard([&] {
        SG_CHECK_ARG(ctx && count, "NULL argument");
        *count = ctx->captures;
    });
}

sg_status sg_ctx_set_timing(sg_ctx* ctx, int on) {
    return guard([&] {
        SG_CHECK_ARG(ctx, "ctx is NULL");
        ctx->timing = on != 0;
        for (int k = 0; k < 8; ++k) {
            ctx->class_ms[k] = 0.0;
            ctx->class_count[k] = 0;
        }
    });
}

sg_status sg_ctx_get_timing(sg_ctx* ctx, int kind, double* ms, long long* count) {
    return guard([&] {
        SG_CHECK_ARG(ctx && ms && count, "NULL argument");
        SG_CHECK_ARG(kind >= 0 && kind < 8, "kind must be in [0,8)");
        use_device(ctx);
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        collect_timers(ctx);
        *ms = ctx->class_ms[kind];
        *count = ctx->class_count[kind];
    });
}

sg_status sg_ctx_synchronize(sg_ctx* ctx) {
    return guard([&] {
        SG_CHECK_ARG(ctx, "ctx is NULL");
        use_device(ctx);
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

// ------------------------------------------------------------------ matrix
sg_status sg_csr_create(sg_ctx* ctx, int nrows, int ncols, int nnz, const int* row_ptr,
                        const int* col_idx, const double* vals, sg_mem mem, sg_csr** out) {
    return guard([&] {
        sg::TraceRange trace("sg_csr_create");
        SG_CHECK_ARG(ctx && out, "NULL argument");
        *out = nullptr;
        SG_CHECK_ARG(nrows >= 0 && ncols >= 0 && nnz >= 0, "negative size");
        SG_CHECK_ARG(row_ptr, "row_ptr is NULL");
        SG_CHECK_ARG(nnz == 0 || (col_idx && vals), "col_idx/vals are NULL");
        use_device(ctx);
        auto* A = new sg_csr();
        A->gen = next_object_gen();
        try {
            A->ctx = ctx;
            A->nrows = nrows;
            A->ncols = ncols;
            A->nnz = nnz;
            A->h_rp.resize((size_t)nrows + 1);
            A->h_ci.resize((size_t)nnz + 16, 0);
            A->h_val.resize((size_t)nnz);
            if (mem == SG_MEM_DEVICE) {
                SG_CUDA(cudaMemcpy(A->h_rp.data(), row_ptr, sizeof(int) * (nrows + 1),
                                   cudaMemcpyDeviceToHost));
                if (nnz) {
                    SG_CUDA(cudaMemcpy(A->h_ci.data(), col_idx, sizeof(int) * nnz,
                                       cudaMemcpyDeviceToHost));
                    SG_CUDA(cudaMemcpy(A->h_val.data(), vals, sizeof(double) * nnz,
                                       cudaMemcpyDeviceToHost));
                }
            } else {
                std::memcpy(A->h_rp.data(), row_ptr, sizeof(int) * (nrows + 1));
                if (nnz) {
                    std::memcpy(A->h_ci.data(), col_idx, sizeof(int) * nnz);
                    std::memcpy(A->h_val.data(), vals, sizeof(double) * nnz);
                }
            }
            SG_CHECK_ARG(A->h_rp[0] == 0, "row_ptr[0] must be 0");
            SG_CHECK_ARG(A->h_rp[nrows] == nnz, "row_ptr[nrows] (%d) != nnz (%d)", A->h_rp[nrows],
                         nnz);
            for (int i = 0; i < nrows; ++i) {
                SG_CHECK_ARG(A->h_rp[i + 1] >= A->h_rp[i], "row_ptr decreases at row %d", i);
                for (int e = A->h_rp[i]; e < A->h_rp[i + 1]; ++e) {
                    const int c = A->h_ci[e];
                    SG_CHECK_ARG(c >= 0 && c < ncols, "col_idx[%d] = %d outside [0,%d)", e, c, ncols);
                    if (e > A->h_rp[i] && c < A->h_ci[e - 1]) A->sorted = false;
                }
            }
            std::vector<double> vpad(A->h_val);
            vpad.resize((size_t)nnz + 16, 0.0);
            A->rp.upload(A->h_rp, ctx->stream);
            A->ci.upload(A->h_ci, ctx->stream);
            A->val.upload(vpad, ctx->stream);
            A->h_ci.resize(nnz);
            if (A->sorted) A->build_sell();
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            delete A;
            throw;
        }
        *out = A;
    });
}

sg_status sg_csr_set_format(sg_csr* A, int format) {
    return guard([&] {
        SG_CHECK_ARG(A, "NULL argument");
        SG_CHECK_ARG(format >= 0 && format <= 3,
                     "format must be 0 (auto), 1 (CSR), 2 (SELL) or 3 (SELL, 16-bit columns)");
        if (format >= 2 && !A->sell_ok)
            fail(SG_ERR_UNSUPPORTED, "no SELL copy of this matrix (unsorted rows or padding > 25%%)");
        if (format == 3 && !A->sl_dcol.p)
            fail(SG_ERR_UNSUPPORTED, "a column lies more than 32767 away from its row");
        A->format = format;
        A->format32 = format;
        A->format_user = format != 0;
    });
}

sg_status sg_csr_set_spmv_variant(sg_csr* A, int variant) {
    return guard([&] {
        SG_CHECK_ARG(A, "NULL argument");
        const int nv = sell_variant_count();
        SG_CHECK_ARG(variant >= 0 && variant < nv, "variant must be in [0,%d)", nv);
        if (!A->sell_ok) fail(SG_ERR_UNSUPPORTED, "no SELL copy of this matrix");
        const int dcol = sell_variant_info(variant, 0), pipe = sell_variant_info(variant, 1);
        if (dcol && !A->sl_dcol.p)
            fail(SG_ERR_UNSUPPORTED, "a column lies more than 32767 away from its row");
        if (pipe && A->sell_maxw > 8)
            fail(SG_ERR_UNSUPPORTED, "a row holds more than 8 entries");
        A->format = A->format32 = dcol ? 3 : 2;
        A->sell_cfg = A->sell_cfg32 = variant;
        A->format_user = true;
    });
}

sg_status sg_csr_get_spmv_choice(sg_csr* A, int* format, int* variant, int* format32,
                                 int* variant32) {
    return guard([&] {
        SG_CHECK_ARG(A, "NULL argument");
        if (format) *format = A->format;
        if (variant) *variant = A->sell_cfg;
        if (format32) *format32 = A->format32 ? A->format32 : A->format;
        if (variant32) *variant32 = A->sell_cfg32;
    });
}

sg_status sg_csr_get_format(sg_csr* A, int* format) {
    return guard([&] {
        SG_CHECK_ARG(A && format, "NULL argument");
        *format = A->format;
    });
}

sg_status sg_csr_destroy(sg_csr* A) {
    return guard([&] {
        if (!A) return;
        cudaSetDevice(A->ctx->device);
        delete A;
    });
}

sg_status sg_csr_spmv(sg_csr* A, const double* x, double* y, sg_mem mem) {
    return guard([&] {
        SG_CHECK_ARG(A && x && y, "NULL argument");
        sg_ctx* ctx = A->ctx;
        use_device(ctx);
        if (!ctx->work) ctx->work = new SolveWork();
        const double* dx = x;
        double* dy = y;
        if (mem == SG_MEM_HOST) {
            SolveWork* w = ctx->work;
            w->x64.upload(x, A->ncols, ctx->stream);
            if (w->b64.n < (size_t)std::max(A->nrows, 1)) w->b64.alloc(std::max(A->nrows, 1));
            dx = w->x64.p;
            dy = w->b64.p;
        }
        spmv_autotune(ctx, A);
        launch_spmv_a<double, double, double>(ctx, A, dx, dy, nullptr, nullptr);
        if (mem == SG_MEM_HOST)
            SG_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * A->nrows, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

// ------------------------------------------------------------------ preconditioner
sg_status sg_precond_create(sg_ctx* ctx, sg_precond_kind kind, const sg_precond_opts* opts,
                            sg_precond** out) {
    return guard([&] {
        SG_CHECK_ARG(ctx && out, "NULL argument");
        *out = nullptr;
        SG_CHECK_ARG(kind >= SG_PC_NONE && kind <= SG_PC_TWOLEVEL_RAS, "unknown kind %d", (int)kind);
        auto* pc = new sg_precond();
        pc->gen = next_object_gen();
        pc->ctx = ctx;
        pc->kind = kind;
        if (opts) pc->opts = *opts;
        else {
            pc->opts.nparts = 4;
            pc->opts.overlap = 1;
            pc->opts.factor_dtype = SG_FP64;
            pc->opts.sweep_dtype = SG_FP64;
        }
        const int swt = pc->opts.reserved[1];
        if (!(swt == 0 || swt == 32 || swt == 64 || swt == 128 || swt == 256 || swt == 384 ||
              swt == 512)) {
            delete pc;
            fail(SG_ERR_INVALID_ARG,
                 "sweep threads (reserved[1]) must be 0, 32, 64, 128, 256, 384 or 512");
        }
        if (pc->opts.reserved[4] < 0) {
            delete pc;
            fail(SG_ERR_INVALID_ARG, "sweep launch shape (reserved[4]) must be >= 0");
        }
        if (pc->opts.reserved[5] != 0 && pc->opts.reserved[5] != 1) {
            delete pc;
            fail(SG_ERR_INVALID_ARG, "set-up path (reserved[5]) must be 0 or 1");
        }
        const int grb = pc->opts.reserved[3];
        if (!(grb == 0 || (grb >= 1024 && grb <= 65536 && grb % 16 == 0))) {
            delete pc;
            fail(SG_ERR_INVALID_ARG,
                 "record group bytes (reserved[3]) must be 0 or a multiple of 16 in [1024, 65536]");
        }
        if (pc->opts.reserved[2] != 0 && pc->opts.reserved[2] != 1) {
            delete pc;
            fail(SG_ERR_INVALID_ARG, "restriction placement (reserved[2]) must be 0 or 1");
        }
        const int sd = pc->opts.sweep_dtype, fd = pc->opts.factor_dtype;
        const bool ok = (sd == SG_FP64 && fd == SG_FP64) ||
                        (sd == SG_FP32 && (fd == SG_FP32 || fd == SG_BF16));
        if (!ok) {
            delete pc;
            fail(SG_ERR_INVALID_ARG,
                 "sweep/factor dtypes: FP64 sweeps need FP64 factors; FP32 sweeps take FP32 or "
                 "BF16 factors");
        }
        *out = pc;
    });
}

namespace {
// FNV-1a over everything the host set-up of a Schwarz preconditioner reads
uint64_t structure_key(const sg_precond* pc, const sg_csr* A, const int* part, int nparts,
                       int overlap) {
    // four independent 64-bit lanes (multiply, xor-shift) over 8-byte words,
    // so the hash runs at memory speed; each array is hashed with its length
    uint64_t h[4] = {0x243f6a8885a308d3ull, 0x13198a2e03707344ull, 0xa4093822299f31d0ull,
                     0x082efa98ec4e6c89ull};
    auto step = [](uint64_t x, uint64_t w) {
        x ^= w * 0x9e3779b97f4a7c15ull;
        x *= 0xbf58476d1ce4e5b9ull;
        return x ^ (x >> 31);
    };
    auto mix = [&](const void* p, size_t bytes) {
        const unsigned char* c = static_cast<const unsigned char*>(p);
        size_t i = 0;
        for (; i + 32 <= bytes; i += 32) {
            uint64_t w[4];
            std::memcpy(w, c + i, 32);
            for (int l = 0; l < 4; ++l) h[l] = step(h[l], w[l]);
        }
        uint64_t tail[4] = {0, 0, 0, 0};
        std::memcpy(tail, c + i, bytes - i);
        for (int l = 0; l < 4; ++l) h[l] = step(h[l], tail[l] ^ ((uint64_t)bytes << (8 * l)));
    };
    const int head[6] = {pc->kind, A->nrows, A->ncols, A->nnz, nparts, overlap};
    mix(head, sizeof(head));
    mix(pc->opts.reserved, sizeof(pc->opts.reserved));
    mix(A->h_rp.data(), sizeof(int) * A->h_rp.size());
    mix(A->h_ci.data(), sizeof(int) * A->h_ci.size());
    mix(part, sizeof(int) * (size_t)A->nrows);
    uint64_t r = 0;
    for (int l = 0; l < 4; ++l) r = step(r ^ (uint64_t)l, h[l]);
    return r;
}
}  // namespace

sg_status sg_precond_setup(sg_precond* pc, const sg_csr* A) {
    return guard([&] {
        sg::TraceRange trace("sg_precond_setup");
        SG_CHECK_ARG(pc && A, "NULL argument");
        SG_CHECK_ARG(A->ctx == pc->ctx, "matrix and preconditioner belong to different contexts");
        use_device(pc->ctx);
        if (pc->kind == SG_PC_HOST) {
            // a host function is set up by its owner; only the size must agree
            SG_CHECK_ARG(A->nrows == pc->n, "the host preconditioner has %d rows, A %d", pc->n,
                         A->nrows);
            return;
        }
        pc->is_setup = false;
        pc->gen = next_object_gen();
        pc->n = A->nrows;
        if (pc->kind == SG_PC_NONE) {
            pc->is_setup = true;
            return;
        }
        if (pc->kind == SG_PC_JACOBI) {
            SG_CHECK_ARG(A->nrows <= A->ncols, "Jacobi needs nrows <= ncols");
            precond_setup_device(pc, A);
            pc->is_setup = true;
            return;
        }
        std::vector<int> part(A->nrows, 0);
        int nparts = 1, overlap = 0;
        if (pc->kind != SG_PC_ILU0) {
            nparts = pc->opts.nparts;
            overlap = pc->opts.overlap;
            SG_CHECK_ARG(nparts >= 1, "nparts must be >= 1");
            SG_CHECK_ARG(nparts <= std::max(A->nrows, 1), "nparts exceeds rows");
            SG_CHECK_ARG(nparts <= 4096 || (pc->kind != SG_PC_TWOLEVEL_ASM &&
                                            pc->kind != SG_PC_TWOLEVEL_RAS),
                         "two-level preconditioners support at most 4096 parts");
            if (pc->opts.partition)
                std::memcpy(part.data(), pc->opts.partition, sizeof(int) * A->nrows);
            else if (nparts > 1)
                partition_graph(A->nrows, A->h_rp.data(), A->h_ci.data(), nparts, part.data());
        }
        pc->overlap = overlap;
        // The integer set-up depends only on the sparsity pattern, the
        // partition and the options: a matrix with the same structure as the
        // previous set-up (new values, e.g. another coefficient field) keeps
        // it and only redoes the device factorisation.
        const uint64_t key = structure_key(pc, A, part.data(), nparts, overlap);
        if (!(pc->has_structure && pc->structure_key == key)) {
            pc->has_structure = false;
            // the integer set-up on the device (opts.reserved[5] = 0), unless
            // its bitmaps would not fit; else, or when asked (1), on host threads
            pc->setup_on_device = pc->opts.reserved[5] == 0 &&
                                  build_schwarz_device(pc, A, part.data(), nparts, overlap);
            if (!pc->setup_on_device) build_schwarz_host(pc, A, part.data(), nparts, overlap);
            pc->structure_key = key;
            pc->has_structure = true;
        }
        precond_setup_device(pc, A);
        pc->is_setup = true;
    });
}

sg_status sg_precond_apply(sg_precond* pc, const double* x, double* y, int n, sg_mem mem) {
    return guard([&] {
        sg::TraceRange trace("sg_precond_apply");
        SG_CHECK_ARG(pc && x && y, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(n == pc->n, "n (%d) does not match the set-up size (%d)", n, pc->n);
        sg_ctx* ctx = pc->ctx;
        if (pc->kind == SG_PC_HOST && mem == SG_MEM_HOST) {
            const int st = pc->host_fn(pc->host_user, x, y, n);
            if (st) fail(SG_ERR_CALLBACK, "the host preconditioner function returned %d", st);
            return;
        }
        use_device(ctx);
        const double* dx = x;
        double* dy = y;
        if (mem == SG_MEM_HOST) {
            pc->io_x.upload(x, n, ctx->stream);
            if (pc->io_y.n < (size_t)std::max(n, 1)) pc->io_y.alloc(std::max(n, 1));
            dx = pc->io_x.p;
            dy = pc->io_y.p;
        }
        precond_apply_device<double, double>(pc, dx, dy, nullptr, true);
        if (pc->learned) learned_apply<double, double>(pc->learned, dx, dy, n, nullptr);
        if (mem == SG_MEM_HOST)
            SG_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (sweep_error(pc))
            fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
        if (pc->learned && learned_error(pc->learned))
            fail(SG_ERR_DEVICE_TIMEOUT, "a learned-stage convolution gave up waiting for its tile");
        if (const int hst = host_precond_status(pc))
            fail(SG_ERR_CALLBACK, "the host preconditioner function returned %d", hst);
    });
}

sg_status sg_precond_create_host(sg_ctx* ctx, sg_host_apply_fn fn, void* user, int n,
                                 sg_precond** out) {
    return guard([&] {
        SG_CHECK_ARG(ctx && fn && out, "NULL argument");
        SG_CHECK_ARG(n >= 1, "n must be >= 1");
        *out = nullptr;
        use_device(ctx);
        auto* pc = new sg_precond();
        try {
            pc->gen = next_object_gen();
            pc->ctx = ctx;
            host_precond_init(pc, fn, user, n);
        } catch (...) {
            delete pc;
            throw;
        }
        *out = pc;
    });
}

sg_status sg_precond_set_wait_test(sg_precond* pc, int mode) {
    return guard([&] {
        SG_CHECK_ARG(pc, "NULL argument");
        SG_CHECK_ARG(mode >= 0 && mode <= 2, "wait test mode must be 0, 1 or 2 (got %d)", mode);
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        if (!sweep_wait_test_supported(pc, mode))
            fail(SG_ERR_UNSUPPORTED, mode == 2 ? "the sweep of this set-up does not compute the "
                                                 "coarse restriction itself"
                                               : "this set-up has no TMA-fed sweep");
        if (pc->wait_test != mode) {
            pc->wait_test = mode;
            pc->gen = next_object_gen();  // a captured cycle holds the old launch arguments
        }
    });
}

sg_status sg_precond_destroy(sg_precond* pc) {
    return guard([&] {
        if (!pc) return;
        cudaSetDevice(pc->ctx->device);
        learned_detach(pc->learned);
        delete pc;
    });
}

sg_status sg_precond_get_decomposition(sg_precond* pc, int which, int* out, int cap, int* len) {
    return guard([&] {
        SG_CHECK_ARG(pc && len, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        const std::vector<int>* v = nullptr;
        switch (which) {
        case 0: v = &pc->part; break;
        case 1: v = &pc->owned_ptr; break;
        case 2: v = &pc->owned; break;
        case 3: v = &pc->sub_ptr; break;
        case 4: v = &pc->sub; break;
        case 5: v = &pc->ownloc_ptr; break;
        case 6: v = &pc->ownloc; break;
        default: fail(SG_ERR_INVALID_ARG, "unknown decomposition array %d", which);
        }
        *len = (int)v->size();
        if (out) {
            SG_CHECK_ARG(cap >= (int)v->size(), "cap %d < length %d", cap, (int)v->size());
            std::copy(v->begin(), v->end(), out);
        }
    });
}

sg_status sg_precond_get_factors(sg_precond* pc, int s, int* n_s, int* nnz_s, int* row_ptr,
                                 int* col_idx, double* lu_vals, int* diag_ptr, int* level_lower,
                                 int* level_upper) {
    return guard([&] {
        SG_CHECK_ARG(pc, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(pc->kind >= SG_PC_ILU0, "no ILU factors for this preconditioner kind");
        SG_CHECK_ARG(s >= 0 && s < pc->nparts, "subdomain %d out of range", s);
        const SubInfo& inf = pc->h_info[s];
        const int* rp = pc->lrp.data() + inf.csr_row_off;
        const int nnz = rp[inf.n];
        if (n_s) *n_s = inf.n;
        if (nnz_s) *nnz_s = nnz;
        if (row_ptr) std::copy(rp, rp + inf.n + 1, row_ptr);
        if (col_idx) std::copy(pc->lci.begin() + inf.csr_nz_off,
                               pc->lci.begin() + inf.csr_nz_off + nnz, col_idx);
        if (diag_ptr) std::copy(pc->ldiag.begin() + inf.row_off,
                                pc->ldiag.begin() + inf.row_off + inf.n, diag_ptr);
        if (level_lower) std::copy(pc->lev_lo.begin() + inf.row_off,
                                   pc->lev_lo.begin() + inf.row_off + inf.n, level_lower);
        if (level_upper) std::copy(pc->lev_up.begin() + inf.row_off,
                                   pc->lev_up.begin() + inf.row_off + inf.n, level_upper);
        if (lu_vals) {
            use_device(pc->ctx);
            precond_read_factors(pc, s, lu_vals);
        }
    });
}

sg_status sg_precond_get_coarse(sg_precond* pc, double* a0, int cap, int* nc) {
    return guard([&] {
        SG_CHECK_ARG(pc && nc, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS,
                     "not a two-level preconditioner");
        *nc = pc->nc;
        if (a0) {
            SG_CHECK_ARG(cap >= pc->nc * pc->nc, "cap too small");
            use_device(pc->ctx);
            precond_read_coarse(pc, a0);
        }
    });
}

sg_status sg_precond_get_sweep_ring(sg_precond* pc, int* ring_bytes, int* group_bytes) {
    return guard([&] {
        SG_CHECK_ARG(pc, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        const bool tma = pc->use_rec && pc->rec_depth > 0;
        if (ring_bytes) *ring_bytes = tma ? (int)pc->ring1.ring_bytes : 0;
        if (group_bytes) *group_bytes = tma ? (int)pc->ring1.gmax : 0;
    });
}

sg_status sg_precond_check(sg_precond* pc, int plant, long long* violations) {
    return guard([&] {
        SG_CHECK_ARG(pc && violations, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        use_device(pc->ctx);
        *violations = sg::sweep_check(pc, plant);
    });
}

sg_status sg_precond_get_setup_path(sg_precond* pc, int* on_device) {
    return guard([&] {
        SG_CHECK_ARG(pc && on_device, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        *on_device = pc->setup_on_device ? 1 : 0;
    });
}

sg_status sg_precond_get_schedule(sg_precond* pc, int which, int* out, long long cap,
                                  long long* len) {
    return guard([&] {
        SG_CHECK_ARG(pc && len, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(pc->kind >= SG_PC_ILU0 && pc->kind != SG_PC_HOST,
                     "no subdomain schedule for this preconditioner kind");
        std::vector<int> tmp;
        const std::vector<int>* v = &tmp;
        switch (which) {
        case 0: v = &pc->h_lev_ptr_f; break;
        case 1: v = &pc->h_lev_ptr_b; break;
        case 2:
            if (pc->wide_cols) v = &pc->h_perm_f32;
            else tmp.assign(pc->h_perm_f16.begin(), pc->h_perm_f16.end());
            break;
        case 3:
            if (pc->wide_cols) v = &pc->h_perm_b32;
            else tmp.assign(pc->h_perm_b16.begin(), pc->h_perm_b16.end());
            break;
        case 4:
            for (const auto& inf : pc->h_info) tmp.push_back(inf.tshift);
            break;
        case 5: v = &pc->lmap; break;
        case 6: v = &pc->lrp; break;
        case 7: v = &pc->ldiag; break;
        case 8: v = &pc->lci; break;
        case 9: v = &pc->lev_lo; break;
        case 10: v = &pc->lev_up; break;
        case 11:
            for (const auto& inf : pc->h_info) {
                tmp.push_back(inf.wl);
                tmp.push_back(inf.wu);
                tmp.push_back(inf.nlev_f);
                tmp.push_back(inf.nlev_b);
            }
            break;
        case 12: tmp.assign(pc->h_order.begin(), pc->h_order.end()); break;
        default: fail(SG_ERR_INVALID_ARG, "unknown schedule array %d", which);
        }
        *len = (long long)v->size();
        if (out) {
            SG_CHECK_ARG(cap >= (long long)v->size(), "cap %lld < length %lld", cap,
                         (long long)v->size());
            std::copy(v->begin(), v->end(), out);
        }
    });
}

sg_status sg_precond_get_sweep(sg_precond* pc, int* sweep, int* threads) {
    return guard([&] {
        SG_CHECK_ARG(pc, "NULL argument");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        const bool ilu = pc->kind != SG_PC_NONE && pc->kind != SG_PC_JACOBI;
        const bool tma = ilu && pc->use_rec && pc->rec_depth > 0;
        if (sweep) *sweep = !ilu ? -1 : (tma ? 0 : (pc->use_sf ? 2 : 1));
        if (threads) *threads = tma ? (pc->sweep_threads > 0 ? pc->sweep_threads : 512) : 0;
    });
}

// ------------------------------------------------------------------ solve
sg_status sg_solve(sg_ctx* ctx, sg_solver solver, const sg_csr* A, sg_precond* pc,
                   const double* b, double* x, int n, sg_mem mem, const sg_solve_params* params,
                   sg_solve_result* result) {
    return guard([&] {
        sg::TraceRange trace("sg_solve");
        SG_CHECK_ARG(ctx && A && b && x, "NULL argument");
        SG_CHECK_ARG(A->ctx == ctx, "matrix belongs to a different context");
        SG_CHECK_ARG(A->nrows == A->ncols, "the solvers need a square matrix");
        SG_CHECK_ARG(n == A->nrows, "n (%d) != matrix rows (%d)", n, A->nrows);
        SG_CHECK_ARG(solver == SG_GMRES || solver == SG_FGMRES || solver == SG_BICGSTAB,
                     "unknown solver %d", (int)solver);
        if (pc) {
            SG_CHECK_ARG(pc->ctx == ctx, "preconditioner belongs to a different context");
            if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
            SG_CHECK_ARG(pc->n == n, "preconditioner was set up for n=%d", pc->n);
            SG_CHECK_ARG(!pc->learned || solver == SG_FGMRES,
                         "a learned stage makes the preconditioner nonlinear: use SG_FGMRES");
        }
        sg_solve_params prm{};
        if (params) prm = *params;
        else {
            prm.restart = 30;
            prm.max_iter = 1000;
            prm.tol = 1e-10;
            prm.tol_kind = SG_TOL_REF_ABS;
            prm.precision = SG_FP64;
            prm.use_graph = 1;
        }
        use_device(ctx);
        if (!ctx->work) ctx->work = new SolveWork();
        SolveWork* w = ctx->work;
        const double* db = b;
        double* dx = x;
        if (mem == SG_MEM_HOST) {
            w->b64.upload(b, n, ctx->stream);
            w->x64.upload(x, n, ctx->stream);
            db = w->b64.p;
            dx = w->x64.p;
        }
        struct CopyBack {
            sg_ctx* ctx;
            double* host;
            const double* dev;
            int n;
            bool on;
            ~CopyBack() {
                if (on) {
                    cudaMemcpyAsync(host, dev, sizeof(double) * n, cudaMemcpyDeviceToHost, ctx->stream);
                    cudaStreamSynchronize(ctx->stream);
                }
            }
        } cb{ctx, x, dx, n, mem == SG_MEM_HOST};
        if (solver == SG_BICGSTAB) solve_bicgstab_device(ctx, A, pc, db, dx, prm, result);
        else solve_device(ctx, solver, A, pc, db, dx, prm, result);
    });
}

sg_status sg_solve_batched(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int nsys,
                           const int* sys_row_ptr, int nrhs, const double* b, double* x,
                           sg_mem mem, const sg_solve_params* params, sg_batch_result* results,
                           double* time_s) {
    return guard([&] {
        sg::TraceRange trace("sg_solve_batched");
        SG_CHECK_ARG(ctx && A && b && x && sys_row_ptr, "NULL argument");
        SG_CHECK_ARG(A->ctx == ctx, "matrix belongs to a different context");
        SG_CHECK_ARG(A->nrows == A->ncols, "the solvers need a square matrix");
        SG_CHECK_ARG(nsys >= 1 && nrhs >= 1, "nsys and nrhs must be >= 1");
        SG_CHECK_ARG(mem == SG_MEM_HOST || mem == SG_MEM_DEVICE, "bad memory kind");
        SG_CHECK_ARG(sys_row_ptr[0] == 0 && sys_row_ptr[nsys] == A->nrows,
                     "sys_row_ptr must run from 0 to the matrix rows");
        for (int s = 0; s < nsys; ++s)
            SG_CHECK_ARG(sys_row_ptr[s + 1] > sys_row_ptr[s], "system %d has no rows", s);
        if (pc) {
            SG_CHECK_ARG(pc->ctx == ctx, "preconditioner belongs to a different context");
            if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
            SG_CHECK_ARG(pc->n == A->nrows, "preconditioner was set up for n=%d", pc->n);
            SG_CHECK_ARG(!pc->learned, "the batched solver takes no learned stage");
            SG_CHECK_ARG(pc->kind != SG_PC_HOST, "the batched solver takes no host preconditioner");
        }
        // block-diagonal matrix and system-local subdomains: checked in
        // solve_batched_device (once per matrix / preconditioner set-up)
        sg_solve_params prm{};
        if (params) prm = *params;
        else {
            prm.restart = 30;
            prm.max_iter = 1000;
            prm.tol = 1e-8;
            prm.tol_kind = SG_TOL_TRUE_REL;
            prm.precision = SG_FP32;
            prm.use_graph = 1;
        }
        use_device(ctx);
        // b and x are copied inside (host or device pointers alike)
        solve_batched_device(ctx, A, pc, nsys, sys_row_ptr, nrhs, b, x, prm, results, time_s);
    });
}

// ------------------------------------------------------------------ BLAS-1
namespace {
// host or device vector -> device pointer (host data staged in ctx buffers)
struct Staged {
    sg::DBuf<double> buf;
    const double* ptr(sg_ctx* ctx, const double* v, int n, sg_mem mem) {
        if (mem == SG_MEM_DEVICE) return v;
        buf.upload(v, (size_t)n, ctx->stream);
        return buf.p;
    }
};
void check_vec_args(sg_ctx* ctx, int n, sg_mem mem) {
    SG_CHECK_ARG(ctx, "ctx is NULL");
    SG_CHECK_ARG(n >= 0, "n must be >= 0");
    SG_CHECK_ARG(mem == SG_MEM_HOST || mem == SG_MEM_DEVICE, "bad memory kind");
}
}  // namespace

// ------------------------------------------------------------------ analysis
namespace {
void check_analysis_args(sg_ctx* ctx, const sg_csr* A, sg_precond* pc) {
    SG_CHECK_ARG(ctx && A, "NULL argument");
    SG_CHECK_ARG(A->ctx == ctx, "matrix belongs to a different context");
    SG_CHECK_ARG(A->nrows == A->ncols, "the analysis needs a square matrix");
    if (pc) {
        SG_CHECK_ARG(pc->ctx == ctx, "preconditioner belongs to a different context");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(pc->n == A->nrows, "preconditioner was set up for n=%d", pc->n);
    }
}
}  // namespace

sg_status sg_estimate_condition(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int k,
                                unsigned seed, sg_condition_estimate* out) {
    return guard([&] {
        sg::TraceRange trace("sg_estimate_condition");
        check_analysis_args(ctx, A, pc);
        SG_CHECK_ARG(out, "NULL argument");
        use_device(ctx);
        estimate_condition_device(ctx, A, pc, k, seed, out);
    });
}

sg_status sg_estimate_spectral_radius(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int max_iter,
                                      double tol, unsigned seed, double* eigenvector,
                                      sg_spectral_result* out) {
    return guard([&] {
        sg::TraceRange trace("sg_estimate_spectral_radius");
        check_analysis_args(ctx, A, pc);
        SG_CHECK_ARG(out, "NULL argument");
        use_device(ctx);
        estimate_spectral_device(ctx, A, pc, max_iter, tol, seed, eigenvector, out);
    });
}

sg_status sg_dot(sg_ctx* ctx, const double* x, const double* y, int n, sg_mem mem,
                 double* result) {
    return guard([&] {
        check_vec_args(ctx, n, mem);
        SG_CHECK_ARG(result && (n == 0 || (x && y)), "NULL argument");
        use_device(ctx);
        Staged sx, sy;
        const double* dx = sx.ptr(ctx, x, n, mem);
        const double* dy = x == y ? dx : sy.ptr(ctx, y, n, mem);
        DBuf<double> out;
        out.alloc(1);
        out.zero(ctx->stream);
        if (n > 0) launch_dot(ctx, dx, dy, n, out.p);
        SG_CUDA(cudaMemcpyAsync(result, out.p, sizeof(double), cudaMemcpyDeviceToHost,
                                ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

sg_status sg_norm2(sg_ctx* ctx, const double* x, int n, sg_mem mem, double* result) {
    sg_status st = sg_dot(ctx, x, x, n, mem, result);
    if (st == SG_OK) *result = std::sqrt(*result);
    return st;
}

sg_status sg_axpy(sg_ctx* ctx, double alpha, const double* x, double* y, int n, sg_mem mem) {
    return guard([&] {
        check_vec_args(ctx, n, mem);
        SG_CHECK_ARG(n == 0 || (x && y), "NULL argument");
        use_device(ctx);
        if (n == 0) return;
        Staged sx, sy;
        const double* dx = sx.ptr(ctx, x, n, mem);
        double* dy = const_cast<double*>(sy.ptr(ctx, y, n, mem));
        launch_axpy(ctx, alpha, dx, dy, n);
        if (mem == SG_MEM_HOST)
            SG_CUDA(cudaMemcpyAsync(y, dy, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

sg_status sg_scale(sg_ctx* ctx, double alpha, double* x, int n, sg_mem mem) {
    return guard([&] {
        check_vec_args(ctx, n, mem);
        SG_CHECK_ARG(n == 0 || x, "NULL argument");
        use_device(ctx);
        if (n == 0) return;
        Staged sx;
        double* dx = const_cast<double*>(sx.ptr(ctx, x, n, mem));
        launch_scale(ctx, alpha, dx, n);
        if (mem == SG_MEM_HOST)
            SG_CUDA(cudaMemcpyAsync(x, dx, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

// ------------------------------------------------------------------ generators
sg_status sg_gen_poisson2d(int nx, int ny, int* row_ptr, int* col_idx, double* vals, int* nnz) {
    return guard([&] {
        SG_CHECK_ARG(nx > 0 && ny > 0 && nnz, "bad arguments");
        SG_CHECK_ARG((long long)nx * ny * 5 < (1ll << 31), "grid too large for int32 CSR");
        *nnz = gen_poisson2d(nx, ny, row_ptr, row_ptr ? col_idx : nullptr, vals);
    });
}

sg_status sg_gen_poisson3d(int nx, int ny, int nz, int* row_ptr, int* col_idx, double* vals,
                           int* nnz) {
    return guard([&] {
        SG_CHECK_ARG(nx > 0 && ny > 0 && nz > 0 && nnz, "bad arguments");
        SG_CHECK_ARG((long long)nx * ny * nz * 7 < (1ll << 31), "grid too large for int32 CSR");
        *nnz = gen_poisson3d(nx, ny, nz, row_ptr, row_ptr ? col_idx : nullptr, vals);
    });
}

sg_status sg_gen_varcoef3d(int nx, int ny, int nz, double sigma, double corr_len, uint64_t seed,
                           int* row_ptr, int* col_idx, double* vals, int* nnz) {
    return guard([&] {
        SG_CHECK_ARG(nx > 0 && ny > 0 && nz > 0 && nnz, "bad arguments");
        SG_CHECK_ARG(corr_len > 0.0 && sigma >= 0.0, "bad field parameters");
        SG_CHECK_ARG((long long)nx * ny * nz * 7 < (1ll << 31), "grid too large for int32 CSR");
        *nnz = gen_varcoef3d(nx, ny, nz, sigma, corr_len, seed, row_ptr, col_idx, vals);
    });
}

sg_status sg_gen_aniso2d(int nx, int ny, double eps, double theta, int* row_ptr, int* col_idx,
                         double* vals, int* nnz) {
    return guard([&] {
        SG_CHECK_ARG(nx > 0 && ny > 0 && nnz, "bad arguments");
        SG_CHECK_ARG(eps > 0.0 && std::isfinite(eps) && std::isfinite(theta),
                     "eps must be positive and theta finite");
        SG_CHECK_ARG((long long)nx * ny * 9 < (1ll << 31), "grid too large for int32 CSR");
        *nnz = gen_aniso2d(nx, ny, eps, theta, row_ptr, row_ptr ? col_idx : nullptr, vals);
    });
}

sg_status sg_gen_uniform(uint64_t seed, int n, double lo, double hi, double* out) {
    return guard([&] {
        SG_CHECK_ARG(n >= 0 && (n == 0 || out), "bad arguments");
        gen_uniform(seed, n, lo, hi, out);
    });
}

sg_status sg_partition_graph(int n, const int* row_ptr, const int* col_idx, int nparts,
                             int* part) {
    return guard([&] {
        SG_CHECK_ARG(row_ptr && part && (n == 0 || col_idx), "NULL argument");
        partition_graph(n, row_ptr, col_idx, nparts, part);
    });
}

sg_status sg_partition_boxes(int nx, int ny, int nz, int nparts, double spread, uint64_t seed,
                             int* part) {
    return guard([&] {
        SG_CHECK_ARG(part, "NULL argument");
        partition_boxes(nx, ny, nz, nparts, spread, seed, part);
    });
}

sg_status sg_schwarz_structure(int n, const int* row_ptr, const int* col_idx, const int* part,
                               int nparts, int overlap, int which, int* out, int cap, int* len) {
    return guard([&] {
        SG_CHECK_ARG(n >= 0 && row_ptr && part && len, "NULL argument");
        sg_csr A;
        A.nrows = A.ncols = n;
        A.nnz = row_ptr[n];
        A.h_rp.assign(row_ptr, row_ptr + n + 1);
        A.h_ci.assign(col_idx, col_idx + A.nnz);
        for (int i = 0; i < n; ++i) {
            SG_CHECK_ARG(row_ptr[i + 1] >= row_ptr[i], "row_ptr decreases at row %d", i);
            for (int e = row_ptr[i]; e < row_ptr[i + 1]; ++e) {
                SG_CHECK_ARG(col_idx[e] >= 0 && col_idx[e] < n, "col_idx out of range");
                if (e > row_ptr[i] && col_idx[e] < col_idx[e - 1]) A.sorted = false;
            }
        }
        sg_precond pc;
        pc.opts.sweep_dtype = SG_FP64;
        build_schwarz_host(&pc, &A, part, nparts, overlap);
        std::vector<int> lrp_abs;
        const std::vector<int>* v = nullptr;
        switch (which) {
        case 0: v = &pc.part; break;
        case 1: v = &pc.owned_ptr; break;
        case 2: v = &pc.owned; break;
        case 3: v = &pc.sub_ptr; break;
        case 4: v = &pc.sub; break;
        case 5: v = &pc.ownloc_ptr; break;
        case 6: v = &pc.ownloc; break;
        case 7: v = &pc.lrp; break;
        case 8: v = &pc.lci; break;
        case 9: v = &pc.ldiag; break;
        case 10: v = &pc.lev_lo; break;
        case 11: v = &pc.lev_up; break;
        default: fail(SG_ERR_INVALID_ARG, "unknown structure array %d", which);
        }
        *len = (int)v->size();
        if (out) {
            SG_CHECK_ARG(cap >= (int)v->size(), "cap %d < length %d", cap, (int)v->size());
            std::copy(v->begin(), v->end(), out);
        }
    });
}

}  // extern "C"
