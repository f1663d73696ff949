// analysis.cu -- the reference CLI's pre-solve analysis on the solve path's
// kernels: a Lanczos estimate of the extreme eigenvalues (and condition
// number) of M^{-1}A (src/analysis/condition_estimator.h:94-191) and the
// power-iteration estimate of the spectral radius of I - M^{-1}A
// (src/analysis/spectral_analysis.h:30-97).
//
// Each step is one SpMV and one preconditioner apply (the Schwarz sweeps)
// plus a fused vector kernel whose last block updates a small device state
// (no host round trip per step); the host reads the state once per chunk of
// steps.  Lanczos rotates three device vectors without copies; the
// eigenvalues of the k x k tridiagonal come from Sturm-sequence bisection on
// the host (exact to the last bits of the interval, no iteration limit),
// where the reference runs implicit QL -- the extreme eigenvalues agree to
// rounding.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int AT = 256;
constexpr int LANCZOS_MAX = 1024;  // steps a single estimate may take

struct LanState {
    int running;  // 1 while steps go on
    int steps;    // alpha values produced
    int nbeta;    // beta values kept (off-diagonal of T)
    int nonfinite;
    double beta;      // the last kept beta (the coefficient of v_prev)
    double inv_beta;  // 1 / beta_new of the step in flight
    double alpha[LANCZOS_MAX];
    double betas[LANCZOS_MAX];
};

struct PowState {
    int running;
    int steps;
    int scale;  // 1: the next scale kernel normalises v (w / ||w||)
    int pad;
    double mu_prev;
    double inv_norm;
    double tol;
};

int agrid(sg_ctx* ctx, int n) {
    long long need = ((long long)n + AT - 1) / AT;
    const long long cap = (long long)ctx->num_sms * 4;
    if (need > cap) need = cap;
    return need < 1 ? 1 : (int)need;
}

// alpha_j = v . z
__global__ void __launch_bounds__(AT)
k_lan_alpha(const double* __restrict__ v, const double* __restrict__ z, int n, LanState* st,
            double* partials, unsigned* counter) {
    if (!st->running) return;
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc = fma(v[i], z[i], acc);
    __shared__ double red[AT / 32], bs[1], tot[1];
    double v1[1] = {acc};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot) || threadIdx.x != 0) return;
    st->alpha[st->steps] = tot[0];
    st->steps++;
    if (!isfinite(tot[0])) {
        st->nonfinite = 1;
        st->running = 0;
    }
}

// z -= alpha v + beta v_prev ; ||z||; stop at an invariant subspace
// (beta_new < 1e-10 (1 + |alpha|)), keep beta_new unless this is the last step
__global__ void __launch_bounds__(AT)
k_lan_orth(double* __restrict__ z, const double* __restrict__ v, const double* __restrict__ vp,
           int n, int last, LanState* st, double* partials, unsigned* counter) {
    if (!st->running) return;
    const double alpha = st->alpha[st->steps - 1], beta = st->beta;
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double q = z[i] - (alpha * v[i] + beta * vp[i]);
        z[i] = q;
        ss = fma(q, q, ss);
    }
    __shared__ double red[AT / 32], bs[1], tot[1];
    double v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot) || threadIdx.x != 0) return;
    const double bn = sqrt(tot[0]);
    if (!isfinite(bn)) {
        st->nonfinite = 1;
        st->running = 0;
    } else if (bn < 1e-10 * (1.0 + fabs(alpha)) || last) {
        st->running = 0;
    } else {
        st->betas[st->nbeta++] = bn;
        st->beta = bn;
        st->inv_beta = 1.0 / bn;
    }
}

// v_next = z / beta_new, written over v_prev's storage (then the host
// rotates the roles of the three vectors)
__global__ void __launch_bounds__(AT)
k_lan_next(const double* __restrict__ z, double* __restrict__ vnext, int n, const LanState* st) {
    if (!st->running) return;
    const double s = st->inv_beta;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        vnext[i] = z[i] * s;
}

// w = v - z (z = M^{-1} A v); mu = v . w; ||w||; stop on ||w|| < 1e-14 or
// |mu - mu_prev| < tol (1 + |mu|) (after normalising v)
__global__ void __launch_bounds__(AT)
k_pow_step(const double* __restrict__ v, const double* __restrict__ z, double* __restrict__ w,
           int n, PowState* st, double* partials, unsigned* counter) {
    if (!st->running) return;
    double mu = 0.0, ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double q = v[i] - z[i];
        w[i] = q;
        mu = fma(v[i], q, mu);
        ss = fma(q, q, ss);
    }
    __shared__ double red[2 * AT / 32], bs[2], tot[2];
    double v2[2] = {mu, ss};
    block_sum_multi<2>(v2, 2, red, bs);
    if (!last_block_reduce(partials, counter, bs, 2, tot) || threadIdx.x != 0) return;
    const double m = tot[0], en = sqrt(tot[1]);
    st->steps++;
    if (!(en >= 1e-14)) {  // also NaN
        st->running = 0;
        st->scale = 0;
        return;
    }
    st->inv_norm = 1.0 / en;
    st->scale = 1;
    if (fabs(m - st->mu_prev) < st->tol * (1.0 + fabs(m))) st->running = 0;
    else st->mu_prev = m;
}

__global__ void __launch_bounds__(AT)
k_pow_scale(const double* __restrict__ w, double* __restrict__ v, int n, PowState* st) {
    if (!st->scale) return;
    const double s = st->inv_norm;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        v[i] = w[i] * s;
}

__global__ void k_pow_clear_scale(PowState* st) { st->scale = 0; }

// The reference's start vector: x <- 1664525 x + 1013904223 (32 bits), each
// value read as a signed int / 2^31, then normalised; `guard` keeps a tiny
// norm at 1 (condition_estimator.h:107-117, spectral_analysis.h:40-49).
std::vector<double> lcg_unit(int n, unsigned seed, bool guard) {
    std::vector<double> v((size_t)n);
    unsigned st = seed;
    double nrm = 0.0;
    for (int i = 0; i < n; ++i) {
        st = st * 1664525u + 1013904223u;
        v[i] = (double)(int)st / 2147483648.0;
        nrm += v[i] * v[i];
    }
    nrm = std::sqrt(nrm);
    if (guard && nrm < 1e-14) nrm = 1.0;
    for (int i = 0; i < n; ++i) v[i] /= nrm;
    return v;
}

// Sturm count: eigenvalues of the symmetric tridiagonal (d, e) below x
int sturm_below(const std::vector<double>& d, const std::vector<double>& e, double x) {
    int cnt = 0;
    double q = 1.0;
    const int n = (int)d.size();
    for (int i = 0; i < n; ++i) {
        const double off = i > 0 ? e[i - 1] * e[i - 1] : 0.0;
        q = d[i] - x - (i > 0 ? off / q : 0.0);
        if (q == 0.0) q = -1e-300;  // a zero pivot counts as negative
        if (q < 0.0) ++cnt;
    }
    return cnt;
}

// k-th smallest eigenvalue (0-based) by bisection on the Gershgorin interval
double tridiag_eig(const std::vector<double>& d, const std::vector<double>& e, int k) {
    const int n = (int)d.size();
    double lo = d[0], hi = d[0];
    for (int i = 0; i < n; ++i) {
        const double r = (i > 0 ? std::fabs(e[i - 1]) : 0.0) + (i < n - 1 ? std::fabs(e[i]) : 0.0);
        lo = std::min(lo, d[i] - r);
        hi = std::max(hi, d[i] + r);
    }
    for (int it = 0; it < 200; ++it) {
        const double mid = 0.5 * (lo + hi);
        if (mid <= lo || mid >= hi) break;  // the interval is two adjacent doubles
        if (sturm_below(d, e, mid) > k) hi = mid;
        else lo = mid;
    }
    return 0.5 * (lo + hi);
}

}  // namespace

void estimate_condition_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int k, unsigned seed,
                               sg_condition_estimate* out) {
    std::memset(out, 0, sizeof(*out));
    const int n = A->nrows;
    SG_CHECK_ARG(k >= 0 && k <= LANCZOS_MAX, "Lanczos steps must be in [0,%d]", LANCZOS_MAX);
    k = std::min(k, n);
    if (k < 2) return;  // no estimate (condition_estimator.h:101-102)
    spmv_autotune(ctx, const_cast<sg_csr*>(A));
    cudaStream_t stream = ctx->stream;
    const size_t nn = (size_t)std::max(n, 1);
    DBuf<double> bufs[3], w, z;
    for (auto& b : bufs) b.alloc(nn);
    w.alloc(nn);
    DBuf<LanState> st;
    st.alloc(1);
    {
        const std::vector<double> v0 = lcg_unit(n, seed, true);
        bufs[0].upload(v0, stream);
        bufs[1].zero(stream);  // v_prev = 0
        LanState h{};
        h.running = 1;
        st.upload(&h, 1, stream);
    }
    const bool has_pc = pc && pc->kind != SG_PC_NONE;
    if (has_pc) z.alloc(nn);
    const int g = agrid(ctx, n);
    const int* active = &st.p->running;
    int cur = 0, prev = 1, spare = 2;
    for (int j = 0; j < k; ++j) {
        launch_spmv_a<double, double, double>(ctx, A, bufs[cur].p, w.p, nullptr, active);
        double* zz = w.p;
        if (has_pc) {
            precond_apply_device<double, double>(pc, w.p, z.p, active, false);
            zz = z.p;
        }
        k_lan_alpha<<<g, AT, 0, stream>>>(bufs[cur].p, zz, n, st.p, ctx->partials.p,
                                          ctx->counter.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        k_lan_orth<<<g, AT, 0, stream>>>(zz, bufs[cur].p, bufs[prev].p, n, j == k - 1 ? 1 : 0,
                                         st.p, ctx->partials.p, ctx->counter.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        // v_next into the spare buffer; then (cur, prev, spare) <- (spare, cur, prev)
        k_lan_next<<<g, AT, 0, stream>>>(zz, bufs[spare].p, n, st.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        const int c = cur;
        cur = spare;
        spare = prev;
        prev = c;
        if ((j & 15) == 15) {  // stop enqueueing once the device says so
            int running = 1;
            SG_CUDA(cudaMemcpyAsync(&running, active, sizeof(int), cudaMemcpyDeviceToHost, stream));
            SG_CUDA(cudaStreamSynchronize(stream));
            if (!running) break;
        }
    }
    LanState h;
    SG_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(h), cudaMemcpyDeviceToHost, stream));
    SG_CUDA(cudaStreamSynchronize(stream));
    if (pc && sweep_error(pc))
        fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
    if (pc && host_precond_status(pc))
        fail(SG_ERR_CALLBACK, "the host preconditioner function reported an error");
    const int m = h.steps;
    if (m < 2 || h.nonfinite) return;
    std::vector<double> d(h.alpha, h.alpha + m), e((size_t)m, 0.0);
    for (int i = 0; i < h.nbeta && i < m; ++i) e[i] = h.betas[i];
    const double lmin = tridiag_eig(d, e, 0), lmax = tridiag_eig(d, e, m - 1);
    out->lambda_min = lmin;
    out->lambda_max = lmax;
    out->kappa = std::fabs(lmin) > 1e-14 ? lmax / lmin : 1e30;
    out->lanczos_steps = m;
    out->valid = lmin > 0.0 ? 1 : 0;
}

void estimate_spectral_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int max_iter,
                              double tol, unsigned seed, double* eigvec_host,
                              sg_spectral_result* out) {
    std::memset(out, 0, sizeof(*out));
    const int n = A->nrows;
    SG_CHECK_ARG(max_iter >= 0, "max_iter must be >= 0");
    spmv_autotune(ctx, const_cast<sg_csr*>(A));
    cudaStream_t stream = ctx->stream;
    const size_t nn = (size_t)std::max(n, 1);
    DBuf<double> v, w, z;
    v.alloc(nn);
    w.alloc(nn);
    z.alloc(nn);
    DBuf<PowState> st;
    st.alloc(1);
    {
        const std::vector<double> v0 = lcg_unit(n, seed, false);
        v.upload(v0, stream);
        PowState h{};
        h.running = max_iter > 0 ? 1 : 0;
        h.tol = tol;
        st.upload(&h, 1, stream);
    }
    const bool has_pc = pc && pc->kind != SG_PC_NONE;
    const int g = agrid(ctx, n);
    const int* active = &st.p->running;
    for (int it = 0; it < max_iter; ++it) {
        launch_spmv_a<double, double, double>(ctx, A, v.p, w.p, nullptr, active);
        if (has_pc) precond_apply_device<double, double>(pc, w.p, z.p, active, false);
        else launch_copy<double, double>(ctx, w.p, z.p, n, active);
        k_pow_step<<<g, AT, 0, stream>>>(v.p, z.p, w.p, n, st.p, ctx->partials.p, ctx->counter.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        k_pow_scale<<<g, AT, 0, stream>>>(w.p, v.p, n, st.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        k_pow_clear_scale<<<1, 1, 0, stream>>>(st.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        if ((it & 15) == 15) {
            int running = 1;
            SG_CUDA(cudaMemcpyAsync(&running, active, sizeof(int), cudaMemcpyDeviceToHost, stream));
            SG_CUDA(cudaStreamSynchronize(stream));
            if (!running) break;
        }
    }
    PowState h;
    SG_CUDA(cudaMemcpyAsync(&h, st.p, sizeof(h), cudaMemcpyDeviceToHost, stream));
    if (eigvec_host)
        SG_CUDA(cudaMemcpyAsync(eigvec_host, v.p, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                stream));
    SG_CUDA(cudaStreamSynchronize(stream));
    if (pc && sweep_error(pc))
        fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
    if (pc && host_precond_status(pc))
        fail(SG_ERR_CALLBACK, "the host preconditioner function reported an error");
    out->spectral_radius = std::fabs(h.mu_prev);
    out->power_iters = h.steps;
    out->convergence_ok = out->spectral_radius < 1.0 ? 1 : 0;
}

}  // namespace sg
