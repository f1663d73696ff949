// bicgstab.cu -- BiCGSTAB with right preconditioning on the device
// (src/core/bicgstab.h:57-204), on the same Preconditioner boundary as the
// GMRES solvers.
//
// All scalars (rho, alpha, omega, norms, the stopping state) live in a device
// BiState; the host enqueues iterations in chunks and reads the state once
// per chunk.  One iteration is
//   p   = r + beta (p - omega v)          k_bi_p     (checks the rho breakdown)
//   y   = M^{-1} p ;  v = A y             the preconditioner, the SpMV
//   alpha = rho / (r^ . v)                k_bi_alpha (one dot, last block)
//   s   = r - alpha v, ||s||              k_bi_s     (lucky exit test)
//   z   = M^{-1} s ;  t = A z             the preconditioner, the SpMV
//   omega = (t . s) / (t . t)             k_bi_omega (two dots in one pass)
//   x  += alpha y + omega z ; r = s - omega t ; ||r|| and the next rho = r^ . r
//                                         k_bi_upd   (stopping tests)
// Every dot reduces per block and the last block to arrive sums the block
// partials in block order (deterministic).  The exits of the reference --
// rho or r^.v below 1e-300, ||s|| < tol ||r0|| (x += alpha y), t.t below
// 1e-300 (x += alpha y), ||r|| < tol ||r0||, |omega| < 1e-300, max_iter --
// set a device flag that makes every later launch of the chunk return
// at once.
#include <chrono>
#include <cmath>
#include <cstring>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int BT = 256;  // threads of the vector kernels

struct BiState {
    int running;   // 1 while iterations go on (the `active` flag of the launches)
    int finish;    // 1: the last kernel of the iteration adds alpha y and stops
    int done;
    int converged;
    int iter;      // completed iterations
    int iterations;  // GMRESResult::iterations as the reference reports it
    int max_iter;
    int hist_len;
    int nonfinite;
    int pad;
    double tol, r0;
    double rho, rho_prev, alpha, omega;
    double rn;     // ||r|| of the current r
    double sn;     // ||s|| of the current iteration
    double res;    // GMRESResult::residual_norm
};

__device__ __forceinline__ void bi_stop(BiState* st, int converged, double res, int iterations) {
    st->converged = converged;
    st->res = res;
    st->iterations = iterations;
    st->running = 0;
    st->done = 1;
}

// r = b - t (t = A x), r^ = r, ||r||^2 and r^.r (the same sum: r^ = r)
__global__ void __launch_bounds__(BT)
k_bi_init(const double* __restrict__ b, const double* __restrict__ t, double* __restrict__ r,
          double* __restrict__ rh, int n, BiState* st, double* partials, unsigned* counter) {
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double v = b[i] - t[i];
        r[i] = v;
        rh[i] = v;
        ss = fma(v, v, ss);
    }
    __shared__ double red[BT / 32], bs[1], tot[1];
    double v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot) || threadIdx.x != 0) return;
    const double r0 = sqrt(tot[0]);
    st->r0 = r0;
    st->rn = r0;
    st->rho = tot[0];
    st->rho_prev = 1.0;
    st->alpha = 1.0;
    st->omega = 1.0;
    st->iter = 0;
    st->finish = 0;
    if (!isfinite(r0)) {
        st->nonfinite = 1;
        bi_stop(st, 0, r0, 0);
    } else if (r0 < 1e-14) {
        bi_stop(st, 1, r0, 0);  // already converged at x0 (bicgstab.h:83-88)
    } else {
        st->running = 1;
        st->done = 0;
    }
}

// p = r + beta (p - omega v), beta = (rho / rho_prev) (alpha / omega); the
// first iteration p = r.  Stops on a rho breakdown or at max_iter.
__global__ void __launch_bounds__(BT)
k_bi_p(const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ p, int n,
       BiState* st) {
    if (!st->running) return;
    const double rho = st->rho;
    if (st->iter >= st->max_iter || fabs(rho) < 1e-300) {
        if (blockIdx.x == 0 && threadIdx.x == 0) {
            if (st->iter >= st->max_iter) bi_stop(st, 0, st->rn, st->iter);
            else bi_stop(st, 0, st->rn, st->iter + 1);  // bicgstab.h:101-107
        }
        return;
    }
    const bool first = st->iter == 0;
    const double beta = (rho / st->rho_prev) * (st->alpha / st->omega);
    const double om = st->omega;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        p[i] = first ? r[i] : r[i] + beta * (p[i] - om * v[i]);
}

// alpha = rho / (r^ . v)
__global__ void __launch_bounds__(BT)
k_bi_alpha(const double* __restrict__ rh, const double* __restrict__ v, int n, BiState* st,
           double* partials, unsigned* counter) {
    if (!st->running) return;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc = fma(rh[i], v[i], acc);
    __shared__ double red[BT / 32], bs[1], tot[1];
    double v1[1] = {acc};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot) || threadIdx.x != 0) return;
    const double rhv = tot[0];
    if (!isfinite(rhv)) {
        st->nonfinite = 1;
        bi_stop(st, 0, st->rn, st->iter + 1);
    } else if (fabs(rhv) < 1e-300) {
        bi_stop(st, 0, st->rn, st->iter + 1);  // bicgstab.h:125-130
    } else {
        st->alpha = st->rho / rhv;
    }
}

// s = r - alpha v, ||s||; ||s|| < tol ||r0||: x += alpha y and stop (the
// half-step exit, bicgstab.h:140-148)
__global__ void __launch_bounds__(BT)
k_bi_s(const double* __restrict__ r, const double* __restrict__ v, double* __restrict__ s, int n,
       BiState* st, double* partials, unsigned* counter, double* hist, int hist_cap) {
    if (!st->running) return;
    const double alpha = st->alpha;
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double q = r[i] - alpha * v[i];
        s[i] = q;
        ss = fma(q, q, ss);
    }
    __shared__ double red[BT / 32], bs[1], tot[1];
    double v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot) || threadIdx.x != 0) return;
    const double sn = sqrt(tot[0]);
    st->sn = sn;
    if (sn < st->tol * st->r0) {
        if (hist && st->hist_len < hist_cap) hist[st->hist_len] = sn;
        st->hist_len++;
        st->converged = 1;
        st->res = sn;
        st->iterations = st->iter + 1;
        st->running = 0;
        st->finish = 1;
    }
}

// omega = (t . s) / (t . t); t.t below 1e-300: x += alpha y and stop
// (bicgstab.h:158-165)
__global__ void __launch_bounds__(BT)
k_bi_omega(const double* __restrict__ t, const double* __restrict__ s, int n, BiState* st,
           double* partials, unsigned* counter) {
    if (!st->running) return;
    double tt = 0.0, ts = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double ti = t[i];
        tt = fma(ti, ti, tt);
        ts = fma(ti, s[i], ts);
    }
    __shared__ double red[2 * BT / 32], bs[2], tot[2];
    double v2[2] = {tt, ts};
    block_sum_multi<2>(v2, 2, red, bs);
    if (!last_block_reduce(partials, counter, bs, 2, tot) || threadIdx.x != 0) return;
    if (!isfinite(tot[0]) || !isfinite(tot[1])) {
        st->nonfinite = 1;
        bi_stop(st, 0, st->sn, st->iter + 1);
    } else if (tot[0] < 1e-300) {
        st->converged = st->sn < st->tol * st->r0;
        st->res = st->sn;
        st->iterations = st->iter + 1;
        st->running = 0;
        st->finish = 1;
    } else {
        st->omega = tot[1] / tot[0];
    }
}

// x += alpha y + omega z ; r = s - omega t ; ||r||, next rho = r^ . r and the
// stopping tests.  With `finish` set by an earlier exit: x += alpha y only.
__global__ void __launch_bounds__(BT)
k_bi_upd(double* __restrict__ x, const double* __restrict__ y, const double* __restrict__ z,
         const double* __restrict__ s, const double* __restrict__ t, double* __restrict__ r,
         const double* __restrict__ rh, int n, BiState* st, double* partials,
         unsigned* counter, double* hist, int hist_cap) {
    const int finish = st->finish;
    if (!st->running && !finish) return;
    const double alpha = st->alpha, omega = st->omega;
    double rr = 0.0, hr = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (finish) {
            x[i] += alpha * y[i];
        } else {
            x[i] += alpha * y[i] + omega * z[i];
            const double q = s[i] - omega * t[i];
            r[i] = q;
            rr = fma(q, q, rr);
            hr = fma(rh[i], q, hr);
        }
    }
    __shared__ double red[2 * BT / 32], bs[2], tot[2];
    double v2[2] = {rr, hr};
    block_sum_multi<2>(v2, 2, red, bs);
    if (!last_block_reduce(partials, counter, bs, 2, tot) || threadIdx.x != 0) return;
    if (finish) {
        st->finish = 0;
        st->done = 1;
        return;
    }
    const double rn = sqrt(tot[0]);
    st->rn = rn;
    if (hist && st->hist_len < hist_cap) hist[st->hist_len] = rn;
    st->hist_len++;
    st->iter++;
    st->iterations = st->iter;
    st->res = rn;
    st->rho_prev = st->rho;
    st->rho = tot[1];
    if (!isfinite(rn)) {
        st->nonfinite = 1;
        bi_stop(st, 0, rn, st->iter);
    } else if (rn < st->tol * st->r0) {
        bi_stop(st, 1, rn, st->iter);  // bicgstab.h:181-186
    } else if (fabs(omega) < 1e-300) {
        bi_stop(st, 0, rn, st->iter);  // bicgstab.h:188-194
    }
}

// ||b - A x|| / ||b|| in FP64 (the reported true residual): t = A x given
__global__ void __launch_bounds__(BT)
k_bi_true(const double* __restrict__ b, const double* __restrict__ t, int n, double* out2,
          double* partials, unsigned* counter) {
    double rr = 0.0, bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double q = b[i] - t[i];
        rr = fma(q, q, rr);
        bb = fma(b[i], b[i], bb);
    }
    __shared__ double red[2 * BT / 32], bs[2], tot[2];
    double v2[2] = {rr, bb};
    block_sum_multi<2>(v2, 2, red, bs);
    if (!last_block_reduce(partials, counter, bs, 2, tot) || threadIdx.x != 0) return;
    out2[0] = sqrt(tot[0]);
    out2[1] = sqrt(tot[1]);
}

int bgrid(sg_ctx* ctx, int n) {
    long long need = ((long long)n + BT - 1) / BT;
    const long long cap = (long long)ctx->num_sms * 4;
    if (need > cap) need = cap;
    return need < 1 ? 1 : (int)need;
}

struct BiWork {
    DBuf<double> r, rh, p, v, y, z, s, t, tmp, true2;
    DBuf<BiState> st;
    BiState* h_st = nullptr;
    ~BiWork() {
        if (h_st) cudaFreeHost(h_st);
    }
};

template <class T>
void grow(DBuf<T>& b, size_t n) {
    if (b.n < n) b.alloc(n);
}

}  // namespace

// BiCGSTAB solve of A x = b (device vectors b, x), x holding x0.  The
// reference rule stops on ||r|| < tol ||r0|| (recursively updated r); with a
// true-residual tol_kind the solve restarts from the current x (fresh shadow
// residual) while ||b - A x|| / ||b|| > tol and iterations remain.
void solve_bicgstab_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, const double* b,
                           double* x, const sg_solve_params& prm, sg_solve_result* res) {
    const int n = A->nrows;
    SG_CHECK_ARG(prm.max_iter >= 0, "max_iter must be >= 0");
    SG_CHECK_ARG(prm.precision == SG_FP64, "BiCGSTAB runs in FP64 (precision must be SG_FP64)");
    SG_CHECK_ARG(prm.tol_kind >= SG_TOL_REF_ABS && prm.tol_kind <= SG_TOL_TRUE_REL,
                 "unknown tol_kind %d", prm.tol_kind);
    BiWork w;
    const size_t nn = (size_t)std::max(n, 1);
    for (DBuf<double>* d : {&w.r, &w.rh, &w.p, &w.v, &w.y, &w.z, &w.s, &w.t, &w.tmp}) grow(*d, nn);
    grow(w.true2, 2);
    grow(w.st, 1);
    SG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&w.h_st), sizeof(BiState)));
    spmv_autotune(ctx, const_cast<sg_csr*>(A));
    const int hcap = prm.history && prm.history_cap > 0 ? prm.history_cap : 0;
    DBuf<double> hist;
    if (hcap) hist.alloc((size_t)hcap);
    cudaStream_t stream = ctx->stream;
    const int g = bgrid(ctx, n);
    BiState* st = w.st.p;
    const int* active = &st->running;
    auto launched = [&] {
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    };
    auto apply_m = [&](const double* in, double* out) {
        ClassTimer tm(ctx, TK_PRECOND);
        if (pc && pc->kind != SG_PC_NONE) precond_apply_device<double, double>(pc, in, out, active, false);
        else launch_copy<double, double>(ctx, in, out, n, active);
    };
    auto spmv = [&](const double* in, double* out) {
        ClassTimer tm(ctx, TK_SPMV);
        launch_spmv_a<double, double, double>(ctx, A, in, out, nullptr, active);
    };
    const auto t0 = std::chrono::high_resolution_clock::now();
    int total_iter = 0, restarts = 0, hist_len = 0, converged = 0, nonfinite = 0;
    double res_norm = 0.0, true_rel = 0.0;
    for (;;) {
        BiState h{};
        h.max_iter = prm.max_iter - total_iter;
        h.tol = prm.tol;
        h.hist_len = hist_len;
        std::memcpy(w.h_st, &h, sizeof(h));
        SG_CUDA(cudaMemcpyAsync(st, w.h_st, sizeof(BiState), cudaMemcpyHostToDevice, stream));
        launch_spmv_a<double, double, double>(ctx, A, x, w.tmp.p, nullptr, nullptr);
        k_bi_init<<<g, BT, 0, stream>>>(b, w.tmp.p, w.r.p, w.rh.p, n, st, ctx->partials.p,
                                         ctx->counter.p);
        launched();
        // iterations in chunks of 8 between reads of the state
        for (;;) {
            for (int it = 0; it < 8; ++it) {
                k_bi_p<<<g, BT, 0, stream>>>(w.r.p, w.v.p, w.p.p, n, st);
                launched();
                apply_m(w.p.p, w.y.p);
                spmv(w.y.p, w.v.p);
                {
                    ClassTimer tm(ctx, TK_ORTHO);
                    k_bi_alpha<<<g, BT, 0, stream>>>(w.rh.p, w.v.p, n, st, ctx->partials.p,
                                                     ctx->counter.p);
                    launched();
                    k_bi_s<<<g, BT, 0, stream>>>(w.r.p, w.v.p, w.s.p, n, st, ctx->partials.p,
                                                 ctx->counter.p, hcap ? hist.p : nullptr, hcap);
                    launched();
                }
                apply_m(w.s.p, w.z.p);
                spmv(w.z.p, w.t.p);
                ClassTimer tm(ctx, TK_UPDATE);
                k_bi_omega<<<g, BT, 0, stream>>>(w.t.p, w.s.p, n, st, ctx->partials.p,
                                                 ctx->counter.p);
                launched();
                k_bi_upd<<<g, BT, 0, stream>>>(x, w.y.p, w.z.p, w.s.p, w.t.p, w.r.p, w.rh.p, n, st,
                                               ctx->partials.p, ctx->counter.p,
                                               hcap ? hist.p : nullptr, hcap);
                launched();
            }
            SG_CUDA(cudaMemcpyAsync(w.h_st, st, sizeof(BiState), cudaMemcpyDeviceToHost, stream));
            SG_CUDA(cudaStreamSynchronize(stream));
            if (ctx->timing) collect_timers(ctx);
            if (w.h_st->done && !w.h_st->finish) break;
        }
        const BiState& e = *w.h_st;
        total_iter += e.iterations;
        hist_len = e.hist_len;
        res_norm = e.res;
        converged = e.converged;
        nonfinite |= e.nonfinite;
        // FP64 true residual of the returned x
        launch_spmv_a<double, double, double>(ctx, A, x, w.tmp.p, nullptr, nullptr);
        k_bi_true<<<g, BT, 0, stream>>>(b, w.tmp.p, n, w.true2.p, ctx->partials.p, ctx->counter.p);
        launched();
        double tr[2] = {0.0, 0.0};
        SG_CUDA(cudaMemcpyAsync(tr, w.true2.p, sizeof(tr), cudaMemcpyDeviceToHost, stream));
        SG_CUDA(cudaStreamSynchronize(stream));
        true_rel = tr[1] > 0 ? tr[0] / tr[1] : tr[0];
        if (prm.tol_kind == SG_TOL_REF_ABS || nonfinite) break;
        converged = true_rel <= prm.tol;
        // restart from the current x while the true residual misses the
        // target, iterations remain and the last run made progress
        if (converged || total_iter >= prm.max_iter || e.iterations == 0) break;
        ++restarts;
    }
    const auto t1 = std::chrono::high_resolution_clock::now();
    if (res) {
        std::memset(res, 0, sizeof(*res));
        res->iterations = total_iter;
        res->cycles = restarts + 1;
        res->converged = converged;
        res->history_len = hist_len;
        res->residual_norm = res_norm;
        res->true_rel_residual = true_rel;
        res->time_solve_s = std::chrono::duration<double>(t1 - t0).count();
    }
    if (hcap) {
        const int cnt = std::min(hist_len, hcap);
        if (cnt > 0)
            SG_CUDA(cudaMemcpy(prm.history, hist.p, sizeof(double) * cnt, cudaMemcpyDeviceToHost));
    }
    if (pc && sweep_error(pc))
        fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
    if (pc) {
        const int hst = host_precond_status(pc);
        if (hst) fail(SG_ERR_CALLBACK, "the host preconditioner function returned %d", hst);
    }
    if (nonfinite) fail(SG_ERR_NONFINITE, "non-finite value in the right-hand side or iteration");
}

}  // namespace sg
