// sg_internal.h -- shared declarations of libsgmres (host + device).
#pragma once

#include <cuda_runtime.h>

#include <cstdarg>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "sgmres.h"

#include <nvtx3/nvToolsExt.h>

namespace sg {

// --------------------------------------------------------------- errors
struct Error {
    sg_status status;
    std::string msg;
};

[[noreturn]] void fail(sg_status st, const char* fmt, ...);
void set_last_error(const char* msg);

#define SG_CUDA(call)                                                                  \
    do {                                                                               \
        cudaError_t e_ = (call);                                                       \
        if (e_ != cudaSuccess)                                                         \
            ::sg::fail(e_ == cudaErrorMemoryAllocation ? SG_ERR_OOM : SG_ERR_CUDA,     \
                       "%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, \
                       __LINE__);                                                      \
    } while (0)

#define SG_CHECK_ARG(cond, ...)                                                        \
    do {                                                                               \
        if (!(cond)) ::sg::fail(SG_ERR_INVALID_ARG, __VA_ARGS__);                      \
    } while (0)

// NVTX range for the life of a scope (entry points, restart cycles): a
// profiler or tracer attached to the process shows set-up, applies, solves
// and cycles by name; without one the calls return at once.
struct TraceRange {
    explicit TraceRange(const char* name) { nvtxRangePushA(name); }
    ~TraceRange() { nvtxRangePop(); }
    TraceRange(const TraceRange&) = delete;
    TraceRange& operator=(const TraceRange&) = delete;
};

// --------------------------------------------------------------- device buffers
template <class T>
struct DBuf {
    T* p = nullptr;
    size_t n = 0;
    DBuf() = default;
    DBuf(const DBuf&) = delete;
    DBuf& operator=(const DBuf&) = delete;
    ~DBuf() { release(); }
    void alloc(size_t count) {
        release();
        if (count == 0) count = 1;
        SG_CUDA(cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
    }
    void release() {
        if (p) cudaFree(p);
        p = nullptr;
        n = 0;
    }
    void upload(const T* h, size_t count, cudaStream_t s) {
        if (n < count || !p) alloc(count);
        if (count) SG_CUDA(cudaMemcpyAsync(p, h, count * sizeof(T), cudaMemcpyHostToDevice, s));
    }
    void upload(const std::vector<T>& v, cudaStream_t s) { upload(v.data(), v.size(), s); }
    void zero(cudaStream_t s) {
        if (p) SG_CUDA(cudaMemsetAsync(p, 0, n * sizeof(T), s));
    }
};

// pinned host buffer (freed with the owner)
template <class T>
struct PinnedBuf {
    T* p = nullptr;
    size_t n = 0;
    PinnedBuf() = default;
    PinnedBuf(const PinnedBuf&) = delete;
    PinnedBuf& operator=(const PinnedBuf&) = delete;
    ~PinnedBuf() {
        if (p) cudaFreeHost(p);
    }
    void alloc(size_t count) {
        if (p) cudaFreeHost(p);
        p = nullptr;
        n = 0;
        if (count == 0) count = 1;
        SG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&p), count * sizeof(T)));
        n = count;
    }
};

// --------------------------------------------------------------- solver state
// Restart lengths up to SG_MMAX are supported.
constexpr int SG_MMAX = 128;
// restart lengths below SG_LAGM use the lagged CGS2 in the GMRES cycle
constexpr int SG_LAGM = 32;

// Device-resident Arnoldi / Givens state of one solve (FP64 throughout).
struct SolveState {
    // control
    int j;            // current Arnoldi step within the cycle
    int kcount;       // basis vectors produced in this cycle (for the update)
    int cycle_active; // 1 while steps of this cycle still run
    int done;         // 1 once the solve has finished (converged or out of iterations)
    int converged;
    int total_iter;
    int max_iter;
    int tol_kind;
    int breakdown;
    int nonfinite;
    int hist_len;
    int cycles;
    int sweep_err;     // the preconditioner's sweep error word, copied after every cycle
    double tol;
    double bnorm;      // ||b||
    double rnorm;      // ||b - A x|| at the current cycle start (FP64)
    double beta;       // ||z|| of the cycle start (the Krylov start norm)
    double est_scale;  // rnorm / beta: turns |g_{j+1}| into a true-residual estimate
    double last_res;   // last |g_{j+1}|
    double ss;         // reduction scratch: sum of squares
    double g[SG_MMAX + 1];
    double cs[SG_MMAX];
    double sn[SG_MMAX];
    double H[(SG_MMAX + 1) * SG_MMAX];  // column-major, ld = m+1
    double h[SG_MMAX + 1];              // projection coefficients of the current pass
    double hsum[SG_MMAX + 1];           // h1 + h2 of the current column
    double vscale[SG_MMAX + 1];         // basis vector k is stored as raw_k; v_k = vscale[k]*raw_k
    double y[SG_MMAX];
    // lagged CGS2 (left-preconditioned GMRES, restart < SG_LAGM): the
    // stored basis vectors raw_l relate to the orthonormal ones through an
    // upper triangular T, v_i = sum_{l<=i} T(l,i) raw_l; the newest stored
    // vector still lacks its second projection, held in lagc
    int lagged;
    double lagT[SG_LAGM * SG_LAGM];  // T(l,i) at l + i*SG_LAGM
    double lagH[SG_LAGM * SG_LAGM];  // unrotated Hessenberg, H(i,k) at i + k*SG_LAGM
    double lagc[SG_LAGM];            // v_j = T(j,j) raw_j - sum_{k<j} lagc[k] v_k
    double cfu[SG_LAGM];             // update coefficients on the stored vectors
};

struct BatchWork;  // workspace of the batched solver (batched.cu)
void destroy_batch_work(BatchWork* w);

// Per-context solve workspace (grown on demand, reused across solves).
// Everything a captured restart cycle bakes in: object identities and
// generations (a generation changes whenever an object's device buffers or
// launch choices may have changed), buffer addresses and sizes.  Compared
// bytewise, so instances are zeroed before their fields are set.
struct GraphKey {
    const void* A;
    uint64_t agen;
    int afmt, afmt32, acfg, acfg32;
    const void* aval32;
    const void* pc;
    uint64_t pgen;
    const void* L;
    uint64_t lgen;
    const void *b, *x;
    int n, m, flexible, fp32, lagged;
    size_t ldv;
    const void *V, *Z, *t, *r64, *st, *hist;
    int hist_cap;
};

struct SolveWork {
    DBuf<SolveState> st;
    DBuf<double> r64, b64, x64;  // residual; staging of host b / x
    DBuf<double> V64, Z64, t64;  // Krylov basis, FGMRES directions, SpMV output
    DBuf<float> V32, Z32, t32;
    SolveState* h_st = nullptr;  // pinned mirror of the state
    cudaGraphExec_t graph = nullptr;  // the last captured restart cycle
    GraphKey gkey{};                  // what it was captured for
    long long graph_nodes = 0;        // its kernel launches
    ~SolveWork();
};

}  // namespace sg

struct sg_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    int num_sms = 0;
    // reduction scratch shared by the kernels of this context (one stream)
    sg::DBuf<double> partials;
    sg::DBuf<unsigned int> counter;
    // residual history of the running solve (device)
    sg::DBuf<double> hist;
    double* hist_d = nullptr;
    int hist_cap = 0;
    sg::SolveWork* work = nullptr;
    sg::BatchWork* batch = nullptr;
    // kernel-class timers (CUDA events on the context stream, eager solves)
    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;
    struct EvPair {
        int kind;
        cudaEvent_t a, b;
    };
    std::vector<EvPair> ev_pending;
    double class_ms[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    long long class_count[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    // kernels launched by this context (graph launches add their kernel nodes)
    long long launches = 0;
    long long captured = 0;
    long long captures = 0;  // restart cycles captured as CUDA graphs
    bool capturing = false;
};

namespace sg {
// kernel classes of the timers
// (TK_LEARNED runs inside TK_PRECOND: the preconditioner class includes it)
enum { TK_SPMV = 0, TK_RESIDUAL = 1, TK_PRECOND = 2, TK_ORTHO = 3, TK_UPDATE = 4, TK_LEARNED = 5 };
// Records a CUDA event pair around the launches made during its lifetime
// when the context's timers are on (not while a graph is being captured).
struct ClassTimer {
    sg_ctx* ctx;
    int kind;
    cudaEvent_t a = nullptr;
    ClassTimer(sg_ctx* c, int k);
    ~ClassTimer();
};
// adds the elapsed times of completed pairs (call after a stream sync)
void collect_timers(sg_ctx* ctx);
// process-wide increasing generation numbers of matrices, preconditioners and
// learned stages (a recycled address never repeats a generation)
uint64_t next_object_gen();
inline void count_launch(sg_ctx* ctx) {
    if (ctx->capturing) ctx->captured++;
    else ctx->launches++;
}
}  // namespace sg

struct sg_csr {
    sg_ctx* ctx = nullptr;
    uint64_t gen = 0;  // object generation (sg::next_object_gen)
    int nrows = 0, ncols = 0, nnz = 0;
    bool sorted = true;  // column indices nondecreasing within each row
    std::vector<int> h_rp, h_ci;
    std::vector<double> h_val;
    sg::DBuf<int> rp, ci;
    sg::DBuf<double> val;
    sg::DBuf<float> val32;  // FP32 copy for the FP32 inner Krylov (made on demand)
    // SELL-C-sigma copy (C = 32, sigma = 1): slice s holds rows 32s..32s+31,
    // entry k of its lane at sl_ptr[s] + 32k + lane, padded to the slice's
    // longest row with (0, own row)
    int nslices = 0;
    long long sell_entries = 0;
    bool sell_ok = false;  // padding small enough to keep the copy
    int format = 0;        // 0 undecided, 1 CSR, 2 SELL, 3 SELL with 16-bit column offsets
    int format32 = 0;      // same for the FP32 copy (0: follow `format`)
    int sell_maxw = 0;     // widest SELL slice (entries per row)
    int sell_cfg = -1;     // tuned SELL launch variant (FP64 values; -1 default)
    int sell_cfg32 = -1;   // same for the FP32 copy
    bool format_user = false;  // set by the caller: the autotuner keeps it
    sg::DBuf<long long> sl_ptr;
    sg::DBuf<int> sl_w, sl_col;
    sg::DBuf<int16_t> sl_dcol;  // column - row when every entry fits in 16 bits
    sg::DBuf<double> sl_val;
    sg::DBuf<float> sl_val32;
    void ensure_fp32();
    void build_sell();
};

namespace sg {

// Per-subdomain metadata of the batched ILU(0) (device array of these).
struct SubInfo {
    int n;        // rows of the subdomain (with overlap)
    int row_off;  // offset into per-row arrays (dofs, perm_f, perm_b, udiag)
    int nlev_f, lev_off_f;
    int nlev_b, lev_off_b;
    int wl, wu;             // ELL widths of L and U (without the diagonal)
    long long fl_off, fu_off;  // offsets into the factor arrays
    int own_off, n_own;     // owned-local list
    int csr_row_off;        // offset into the local CSR row_ptr array (n+1 per sub)
    long long csr_nz_off;   // offset into the local CSR entries
    double cscale;          // 1/sqrt(|owned|) (two-level)
    int tshift;             // TMA sweep: row r sits in shared slot r + (r >> tshift) (0: r)
};

// Shared-memory slot of subdomain row r in the TMA-fed sweep: one unused word
// every 2^p rows (p = 0: none), chosen per subdomain so that the rows of a
// level -- a fixed stride apart in a box subdomain -- fall in distinct banks.
__host__ __device__ __forceinline__ int tslot(int r, int p) { return p ? r + (r >> p) : r; }

// One way of streaming the level records through the TMA-fed sweep's
// shared-memory ring: its size, the largest group of records copied at once,
// the block size, whether CTAs loop over subdomains (persistent: grid CTAs
// take subdomains from a work counter, largest first) and the static
// schedule -- per subdomain (sub: RingSub records as bytes), per level (meta:
// int4 as four ints), per record group (grp: int2 as two ints).
struct RingPlan {
    int R = 1;                 // right-hand sides interleaved in the shared vector
    bool ready = false;
    long long ring_bytes = 0;
    long long gmax = 0;
    int threads = 0;
    int grid = 0;              // CTAs of a persistent launch (0: one CTA per subdomain)
    std::vector<unsigned char> sub;
    std::vector<int> meta, grp;
    DBuf<unsigned char> sub_d;
    DBuf<int> meta_d, grp_d;
    DBuf<unsigned> work;       // persistent launches: next subdomain, CTAs done
};

}  // namespace sg

struct sg_precond {
    sg_ctx* ctx = nullptr;
    uint64_t gen = 0;  // renewed by every set-up and learned-stage change
    int kind = SG_PC_NONE;
    sg_precond_opts opts{};
    bool is_setup = false;
    bool has_structure = false;   // integer set-up done for structure_key
    bool setup_on_device = false; // ... by the device kernels (false: host threads)
    uint64_t structure_key = 0;
    int n = 0;
    int nparts = 0;
    int overlap = 0;
    // ---- host integer set-up (kept for parity read-back)
    std::vector<int> part, owned_ptr, owned, sub_ptr, sub, ownloc_ptr, ownloc;
    std::vector<int> lrp, lci, ldiag, lmap, lev_lo, lev_up;  // local CSR, per-sub blocks
    std::vector<sg::SubInfo> h_info;
    std::vector<int> h_order, h_lev_ptr_f, h_lev_ptr_b;
    std::vector<uint16_t> h_perm_f16, h_perm_b16;
    std::vector<int> h_perm_f32, h_perm_b32;
    std::vector<double> h_cscale;
    bool wide_cols = false;  // subdomains above 65534 rows use 32-bit local indices
    long long fl_total = 0, fu_total = 0;
    int max_n = 0;
    int t_len = 0;       // TMA sweep: largest tslot(n_s, tshift_s) + 1
    int max_levels = 0;  // largest nlev_f + nlev_b of a subdomain
    long long total_rows = 0;
    bool use_smem = true;
    // level records for the TMA-fed sweep: per level one 16-byte-aligned
    // record [rows | columns | values (| diagonal)], rows padded to 8
    bool use_rec = false;
    bool use_sf = false;   // sync-free sweep (per-row ready flags)
    int rec_depth = 0;               // 1 when the TMA-fed sweep is set up (0: not used)
    // how the level records stream through the sweep's shared-memory ring,
    // for one right-hand side at a time (ring1) and for four interleaved ones
    // (ring4, planned when a batched solve first asks for it)
    sg::RingPlan ring1, ring4;
    int sweep_threads = 0;           // threads per CTA of the TMA-fed sweep
    bool fuse_restrict = false;      // two-level: restriction inside the sweep (all CTAs resident)
    sg::DBuf<unsigned> coarse_sync;  // its arrival / departure counters
    long long rec_stage_bytes = 0;   // largest record
    long long rec_total = 0;
    std::vector<long long> h_rec_off_f, h_rec_off_b;  // byte offset per level
    std::vector<int> h_rec_rows_f, h_rec_rows_b;      // padded rows per level
    // ---- device
    sg::DBuf<double> inv_diag;  // jacobi
    sg::DBuf<float> inv_diag32;
    sg::DBuf<sg::SubInfo> info;
    sg::DBuf<int> order;  // launch order of subdomains (largest first)
    sg::DBuf<int> dofs;   // global index of every local row
    sg::DBuf<uint16_t> perm_f, perm_b;  // level order (16-bit, or 32-bit stored in pairs)
    sg::DBuf<int> lev_ptr_f, lev_ptr_b;
    sg::DBuf<uint16_t> lcol, ucol;  // ELL local columns (level-major)
    sg::DBuf<double> lval64, uval64, udiag64;
    sg::DBuf<float> lval32, uval32, udiag32;
    sg::DBuf<uint16_t> lval16, uval16, udiag16;  // bf16 bit patterns
    sg::DBuf<int> ownloc_d;
    sg::DBuf<int> owned_d, owned_ptr_d, part_d;
    sg::DBuf<int> lrp_d, lci_d, ldiag_d, lmap_d;
    sg::DBuf<double> lu_d;  // FP64 factors in local CSR layout
    sg::DBuf<long long> rec_off_f_d, rec_off_b_d;
    sg::DBuf<int> rec_rows_f_d, rec_rows_b_d;
    sg::DBuf<unsigned char> rec_d;
    sg::DBuf<int> err_d;  // device error word of the sweeps (bounded waits)
    int wait_test = 0;     // sg_precond_set_wait_test mode (0: normal)
    sg::DBuf<double> gscratch64;
    sg::DBuf<float> gscratch32;
    // ---- coarse space
    int nc = 0;
    sg::DBuf<double> a0, a0inv, lu0, r0, cscale_d;
    sg::DBuf<int> piv0, status_d;
    // ---- host-API staging
    sg::DBuf<double> io_x, io_y;
    // ---- learned coarse-correction stage applied after M (not owned)
    sg_learned* learned = nullptr;
    // optional device array [nparts]: 0 skips that subdomain's sweep (set by
    // the batched solver around its applies; NULL = every subdomain)
    const int* sub_on = nullptr;
    // ---- host preconditioner (kind SG_PC_HOST, sg_precond_create_host): a
    // caller's function applied in stream order between pinned copies
    sg_host_apply_fn host_fn = nullptr;
    void* host_user = nullptr;
    struct HostCtl {
        int active;    // the launch's active flag, copied before the call
        int status;    // first nonzero return of the function (0: none)
        double scale;  // the input vector's scale (FGMRES directions)
        long long calls;
    };
    sg::PinnedBuf<double> h_in, h_out;  // n doubles each (FP32 data uses the front)
    sg::PinnedBuf<HostCtl> h_ctl;
};
