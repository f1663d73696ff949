// solver.cu -- restarted GMRES(m) and FGMRES drivers on the device
// (src/core/gmres.cpp:34-160, src/core/fgmres.cpp:28-144).  Replaces the
// host-driven loop of src/gpu/gmres_gpu.cu:10-138, which returned every dot
// product to the host: here one restart cycle is a fixed launch sequence
// (optionally captured once as a CUDA graph), all scalars stay in a device
// SolveState, and the host reads the state once per cycle.
//
// Precision modes
//   SG_FP64: basis, SpMV and preconditioner I/O in FP64 (the all-FP64 solver).
//   SG_FP32: the Krylov basis, the inner SpMV and the preconditioner I/O are
//            FP32; every cycle starts from the FP64 true residual b - A x and
//            ends with an FP64 update of x, and the Hessenberg / Givens least
//            squares stays FP64 -- iterative refinement with a GMRES(m)
//            cycle as the inner solver (GMRES-IR).
#include <chrono>
#include <cmath>
#include <cstring>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

SolveWork::~SolveWork() {
    if (graph) cudaGraphExecDestroy(graph);
    if (h_st) cudaFreeHost(h_st);
}

static cudaEvent_t take_event(sg_ctx* ctx) {
    if (!ctx->ev_pool.empty()) {
        cudaEvent_t e = ctx->ev_pool.back();
        ctx->ev_pool.pop_back();
        return e;
    }
    cudaEvent_t e;
    SG_CUDA(cudaEventCreate(&e));
    return e;
}

ClassTimer::ClassTimer(sg_ctx* c, int k) : ctx(c), kind(k) {
    if (!ctx->timing || ctx->capturing) return;
    a = take_event(ctx);
    SG_CUDA(cudaEventRecord(a, ctx->stream));
}

ClassTimer::~ClassTimer() {
    if (!a) return;
    cudaEvent_t b = take_event(ctx);
    cudaEventRecord(b, ctx->stream);
    ctx->ev_pending.push_back({kind, a, b});
}

void collect_timers(sg_ctx* ctx) {
    for (auto& p : ctx->ev_pending) {
        float ms = 0.f;
        if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess && p.kind >= 0 && p.kind < 8) {
            ctx->class_ms[p.kind] += ms;
            ctx->class_count[p.kind] += 1;
        }
        ctx->ev_pool.push_back(p.a);
        ctx->ev_pool.push_back(p.b);
    }
    ctx->ev_pending.clear();
}

namespace {

template <class TV>
struct Basis;
template <>
struct Basis<double> {
    static DBuf<double>& V(SolveWork* w) { return w->V64; }
    static DBuf<double>& Z(SolveWork* w) { return w->Z64; }
    static DBuf<double>& T(SolveWork* w) { return w->t64; }
    static const double* vals(const sg_csr* A) { return A->val.p; }
};
template <>
struct Basis<float> {
    static DBuf<float>& V(SolveWork* w) { return w->V32; }
    static DBuf<float>& Z(SolveWork* w) { return w->Z32; }
    static DBuf<float>& T(SolveWork* w) { return w->t32; }
    static const float* vals(const sg_csr* A) { return A->val32.p; }
};

// host_scale (FGMRES): the device scale of the stored input vector; a host
// preconditioner function is applied to the normalised vector, as the
// reference's FGMRES applies its FlexApply (src/core/fgmres.cpp:133-136)
template <class TI, class TO>
void apply_pc(sg_ctx* ctx, sg_precond* pc, const TI* x, TO* y, int n, const int* active,
              const double* host_scale = nullptr) {
    // inside the solver FP64 sweeps may fuse multiply-adds (exact = false)
    if (pc && pc->kind == SG_PC_HOST) host_precond_apply<TI, TO>(pc, x, y, active, host_scale);
    else if (pc && pc->kind != SG_PC_NONE) precond_apply_device<TI, TO>(pc, x, y, active, false);
    else launch_copy<TI, TO>(ctx, x, y, n, active);
    if (pc && pc->learned) {
        ClassTimer tm(ctx, TK_LEARNED);
        learned_apply<TI, TO>(pc->learned, x, y, n, active);
    }
}

// The lagged two-pass CGS2 serves the left-preconditioned cycle (FP32 or
// FP64 basis) with a restart below SG_LAGM unless the caller asks for the
// classic three passes: it relies on the operator being linear (B v_k =
// V H(:,k)), which FGMRES's possibly nonlinear preconditioner does not give.
bool use_lagged(bool flexible, int m, int ortho) { return ortho == 0 && !flexible && m < SG_LAGM; }

// One restart cycle as a launch sequence on ctx->stream.
template <class TV>
void enqueue_cycle(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, const double* b, double* x,
                   int m, bool flexible, bool lagged, size_t ldv) {
    SolveWork* w = ctx->work;
    SolveState* st = w->st.p;
    const int n = A->nrows;
    TV* V = Basis<TV>::V(w).p;
    TV* Z = flexible ? Basis<TV>::Z(w).p : nullptr;
    TV* t = Basis<TV>::T(w).p;
    const int* active = &st->cycle_active;
    // r = b - A x is already in w->r64 (computed at the end of the previous
    // cycle, or before the first one) together with the convergence test.
    // Krylov start vector raw_0
    {
        ClassTimer tm(ctx, TK_PRECOND);
        if (!flexible) apply_pc<double, TV>(ctx, pc, w->r64.p, V, n, active);
        else launch_copy<double, TV>(ctx, w->r64.p, V, n, active);
    }
    {
        ClassTimer tm(ctx, TK_ORTHO);
        launch_cycle_init<TV>(ctx, V, n, st, m, flexible);
    }
    for (int j = 0; j < m; ++j) {
        TV* vj = V + (size_t)j * ldv;
        TV* wj = V + (size_t)(j + 1) * ldv;
        if (!flexible) {
            // w = M^{-1} A v_j  (src/core/gmres.cpp:280-285)
            {
                ClassTimer tm(ctx, TK_SPMV);
                launch_spmv_a<TV, TV, TV>(ctx, A, vj, t, &st->vscale[j], active);
            }
            ClassTimer tm(ctx, TK_PRECOND);
            apply_pc<TV, TV>(ctx, pc, t, wj, n, active);
        } else {
            // z_j = M^{-1} v_j ; w = A z_j  (src/core/fgmres.cpp:133-140)
            TV* zj = Z + (size_t)j * ldv;
            {
                ClassTimer tm(ctx, TK_PRECOND);
                apply_pc<TV, TV>(ctx, pc, vj, zj, n, active, &st->vscale[j]);
            }
            ClassTimer tm(ctx, TK_SPMV);
            launch_spmv_a<TV, TV, TV>(ctx, A, zj, wj, &st->vscale[j], active);
        }
        ClassTimer tm(ctx, TK_ORTHO);
        launch_cgs2<TV>(ctx, V, ldv, n, j, m, st, lagged);
    }
    {
        ClassTimer tm(ctx, TK_UPDATE);
        launch_backsolve(ctx, st, m);
        launch_update_x<TV>(ctx, flexible ? Z : V, ldv, n, x, st);
    }
    // FP64 true residual of the updated x: convergence test and the next
    // cycle's right-hand side
    {
        ClassTimer tm(ctx, TK_RESIDUAL);
        launch_residual(ctx, A, b, x, w->r64.p, st);
    }
    launch_cycle_end(ctx, st);
    if (pc && pc->learned) learned_monitor(pc->learned, st);
}

template <class T>
void ensure(DBuf<T>& b, size_t count) {
    if (b.n < count) b.alloc(count);
}

}  // namespace

void solve_device(sg_ctx* ctx, int solver, const sg_csr* A, sg_precond* pc, const double* b,
                  double* x, const sg_solve_params& prm, sg_solve_result* res) {
    const int n = A->nrows;
    const int m = prm.restart;
    SG_CHECK_ARG(m >= 1 && m <= SG_MMAX, "restart must be in [1,%d] (got %d)", SG_MMAX, m);
    SG_CHECK_ARG(prm.max_iter >= 0, "max_iter must be >= 0");
    SG_CHECK_ARG(prm.precision == SG_FP64 || prm.precision == SG_FP32,
                 "solve precision must be SG_FP64 or SG_FP32");
    SG_CHECK_ARG(prm.tol_kind >= SG_TOL_REF_ABS && prm.tol_kind <= SG_TOL_TRUE_REL,
                 "unknown tol_kind %d", prm.tol_kind);
    SG_CHECK_ARG(prm.ortho == 0 || prm.ortho == 1, "ortho must be 0 or 1 (got %d)", prm.ortho);
    const bool flexible = solver == SG_FGMRES;
    const bool fp32 = prm.precision == SG_FP32;
    const bool lagged = use_lagged(flexible, m, prm.ortho);
    if (!ctx->work) ctx->work = new SolveWork();
    SolveWork* w = ctx->work;
    // basis stride: a multiple of 32 elements plus 32, so consecutive basis
    // vectors never sit a power of two apart (equal strides of 2^k bytes map
    // every vector's element i to the same HBM channel)
    const size_t ldv = (((size_t)n + 31) & ~(size_t)31) + 32;
    ensure(w->st, 1);
    ensure(w->r64, ldv);
    if (!w->h_st) SG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&w->h_st), sizeof(SolveState)));
    if (fp32) const_cast<sg_csr*>(A)->ensure_fp32();
    // SpMV format: the faster of CSR and SELL on this matrix (same results);
    // the FP32 copy gets its own choice once it exists
    spmv_autotune(ctx, const_cast<sg_csr*>(A));
    if (fp32) {
        ensure(w->V32, ldv * (m + 1));
        ensure(w->t32, ldv);
        if (flexible) ensure(w->Z32, ldv * m);
    } else {
        ensure(w->V64, ldv * (m + 1));
        ensure(w->t64, ldv);
        if (flexible) ensure(w->Z64, ldv * m);
    }
    // history
    const int hcap = prm.history && prm.history_cap > 0 ? prm.history_cap : 0;
    if (hcap > 0) {
        if (ctx->hist.n < (size_t)hcap) ctx->hist.alloc(hcap);
        ctx->hist_d = ctx->hist.p;
        ctx->hist_cap = hcap;
    } else {
        ctx->hist_d = nullptr;
        ctx->hist_cap = 0;
    }
    // state
    SolveState* hs = w->h_st;
    std::memset(hs, 0, sizeof(SolveState));
    hs->max_iter = prm.max_iter;
    hs->tol = prm.tol;
    hs->tol_kind = prm.tol_kind;
    hs->lagged = lagged ? 1 : 0;
    const auto t0 = std::chrono::high_resolution_clock::now();
    SG_CUDA(cudaMemcpyAsync(w->st.p, hs, sizeof(SolveState), cudaMemcpyHostToDevice, ctx->stream));
    launch_bnorm(ctx, b, n, w->st.p);
    launch_residual(ctx, A, b, x, w->r64.p, w->st.p);
    if (pc && pc->learned) learned_begin(pc->learned, w->st.p);
    const size_t ctl_bytes = offsetof(SolveState, g);
    SG_CUDA(cudaMemcpyAsync(hs, w->st.p, ctl_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(cudaStreamSynchronize(ctx->stream));
    const bool done_at_start = hs->done != 0;

    const bool use_graph = prm.use_graph != 0 && !done_at_start && prm.max_iter > 0;
    cudaGraphExec_t exec = nullptr;
    if (use_graph) {
        // the restart cycle is captured once and reused while nothing it
        // bakes in has changed (same operator, preconditioner, vectors, sizes)
        GraphKey key;
        std::memset(&key, 0, sizeof(key));
        key.A = A;
        key.agen = A->gen;
        key.afmt = A->format;
        key.afmt32 = A->format32;
        key.acfg = A->sell_cfg;
        key.acfg32 = A->sell_cfg32;
        key.aval32 = A->val32.p;
        key.pc = pc;
        key.pgen = pc ? pc->gen : 0;
        key.L = pc ? pc->learned : nullptr;
        key.lgen = pc && pc->learned ? learned_gen(pc->learned) : 0;
        key.b = b;
        key.x = x;
        key.n = n;
        key.m = m;
        key.flexible = flexible ? 1 : 0;
        key.fp32 = fp32 ? 1 : 0;
        key.lagged = lagged ? 1 : 0;
        key.ldv = ldv;
        key.V = fp32 ? (const void*)w->V32.p : (const void*)w->V64.p;
        key.Z = fp32 ? (const void*)w->Z32.p : (const void*)w->Z64.p;
        key.t = fp32 ? (const void*)w->t32.p : (const void*)w->t64.p;
        key.r64 = w->r64.p;
        key.st = w->st.p;
        key.hist = ctx->hist_d;
        key.hist_cap = ctx->hist_cap;
        if (!(w->graph && std::memcmp(&key, &w->gkey, sizeof(key)) == 0)) {
            if (w->graph) {
                cudaGraphExecDestroy(w->graph);
                w->graph = nullptr;
            }
            cudaGraph_t g = nullptr;
            SG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeRelaxed));
            ctx->capturing = true;
            ctx->captured = 0;
            try {
                if (fp32) enqueue_cycle<float>(ctx, A, pc, b, x, m, flexible, lagged, ldv);
                else enqueue_cycle<double>(ctx, A, pc, b, x, m, flexible, lagged, ldv);
            } catch (...) {
                ctx->capturing = false;
                cudaStreamEndCapture(ctx->stream, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            ctx->capturing = false;
            SG_CUDA(cudaStreamEndCapture(ctx->stream, &g));
            cudaGraphExec_t ge = nullptr;
            cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
            cudaGraphDestroy(g);
            SG_CUDA(e);
            w->graph = ge;
            w->gkey = key;
            ctx->captures++;
            w->graph_nodes = ctx->captured;
        }
        exec = w->graph;
    }
    int cycles = 0;
    try {
        while (!done_at_start && cycles < prm.max_iter) {
            TraceRange trace_cycle(use_graph ? "restart cycle (graph)" : "restart cycle");
            if (use_graph) {
                SG_CUDA(cudaGraphLaunch(exec, ctx->stream));
                ctx->launches += w->graph_nodes;
            }
            else if (fp32) enqueue_cycle<float>(ctx, A, pc, b, x, m, flexible, lagged, ldv);
            else enqueue_cycle<double>(ctx, A, pc, b, x, m, flexible, lagged, ldv);
            ++cycles;
            // a sweep that gave up on a bounded wait ends the solve (its
            // output was not written, so later cycles would be meaningless)
            if (pc && pc->err_d.p)
                SG_CUDA(cudaMemcpyAsync(&w->st.p->sweep_err, pc->err_d.p, sizeof(int),
                                        cudaMemcpyDeviceToDevice, ctx->stream));
            SG_CUDA(cudaMemcpyAsync(hs, w->st.p, ctl_bytes, cudaMemcpyDeviceToHost, ctx->stream));
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
            if (ctx->timing) collect_timers(ctx);
            if (hs->done || hs->sweep_err) break;
        }
    } catch (...) {
        // a failed solve drops the cached cycle
        if (w->graph) cudaGraphExecDestroy(w->graph);
        w->graph = nullptr;
        throw;
    }
    // the state now holds the FP64 true residual of the returned x
    SG_CUDA(cudaMemcpyAsync(hs, w->st.p, ctl_bytes, cudaMemcpyDeviceToHost, ctx->stream));
    SG_CUDA(cudaStreamSynchronize(ctx->stream));
    const auto t1 = std::chrono::high_resolution_clock::now();
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->iterations = hs->total_iter;
        res->cycles = hs->cycles;
        res->converged = hs->converged;
        res->history_len = hs->hist_len;
        res->residual_norm = hs->hist_len > 0 ? hs->last_res : 0.0;
        res->true_rel_residual = hs->bnorm > 0 ? hs->rnorm / hs->bnorm : hs->rnorm;
        res->time_solve_s = std::chrono::duration<double>(t1 - t0).count();
    }
    if (hcap > 0) {
        const int cnt = hs->hist_len < hcap ? hs->hist_len : hcap;
        if (cnt > 0)
            SG_CUDA(cudaMemcpy(prm.history, ctx->hist.p, sizeof(double) * cnt,
                               cudaMemcpyDeviceToHost));
    }
    if (pc && sweep_error(pc))
        fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
    if (pc && pc->learned && learned_error(pc->learned))
        fail(SG_ERR_DEVICE_TIMEOUT, "a learned-stage convolution gave up waiting for its tile");
    if (pc) {
        const int hst = host_precond_status(pc);
        if (hst) fail(SG_ERR_CALLBACK, "the host preconditioner function returned %d", hst);
    }
    if (hs->nonfinite) fail(SG_ERR_NONFINITE, "non-finite value in the right-hand side or iteration");
}

}  // namespace sg
