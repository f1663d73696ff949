// spmv.cu -- CSR sparse matrix-vector products (CSRMatrix::spmv,
// src/core/sparse_matrix.h:30-37; replaces cusparseSpMV in
// src/gpu/cuda_sparse.h:53-74).
//
// Layout: one warp owns a tile of 32 consecutive rows.  The tile's nonzeros
// are one contiguous range of the CSR arrays; the warp streams it with
// 16-byte vector loads (2 FP64 or 4 FP32 values, 2 or 4 column indices per
// lane), forms the products into a per-warp shared-memory window and each
// lane then sums its own row from the window (a warp-segmented reduction
// whose per-row order is the entry order).  In FP64 the products and sums are
// rounded one by one, so y matches the reference's serial loop bit for bit.
#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int SPMV_WARPS = 8;
constexpr int SPMV_THREADS = SPMV_WARPS * 32;

template <class T>
struct VecT;
template <>
struct VecT<double> {
    using V = double2;
    using I = int2;
    static constexpr int N = 2;
};
template <>
struct VecT<float> {
    using V = float4;
    using I = int4;
    static constexpr int N = 4;
};

__device__ __forceinline__ double pmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double padd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float pmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ float padd(float a, float b) { return __fadd_rn(a, b); }

template <class T, class V>
__device__ __forceinline__ void unpack(const V& v, T (&o)[VecT<T>::N]);
template <>
__device__ __forceinline__ void unpack<double, double2>(const double2& v, double (&o)[2]) {
    o[0] = v.x; o[1] = v.y;
}
template <>
__device__ __forceinline__ void unpack<float, float4>(const float4& v, float (&o)[4]) {
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
__device__ __forceinline__ void unpacki(const int2& v, int (&o)[2]) { o[0] = v.x; o[1] = v.y; }
__device__ __forceinline__ void unpacki(const int4& v, int (&o)[4]) {
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}

// MODE 0: y = scale * (A x);  MODE 1: y = b - A x with ||y||^2 reduced.
template <class TV, class TX, class TY, int MODE>
__global__ void __launch_bounds__(SPMV_THREADS, 4)
k_spmv_csr(int n, const int* __restrict__ rp, const int* __restrict__ ci,
           const TV* __restrict__ val, const TX* __restrict__ x, TY* __restrict__ y,
           const double* __restrict__ scale, const int* __restrict__ active,
           const double* __restrict__ b, double* partials, unsigned* counter, SolveState* st) {
    if (active && *active == 0) return;
    constexpr int VN = VecT<TV>::N;
    constexpr int CAP = 32 * VN * 4;
    using VV = typename VecT<TV>::V;
    using VI = typename VecT<TV>::I;
    __shared__ TV buf[SPMV_WARPS][CAP];
    // MODE 1 keeps values and gathered x apart, for fused multiply-adds
    __shared__ TV xbuf_all[MODE == 1 ? SPMV_WARPS : 1][MODE == 1 ? CAP : 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwarps = gridDim.x * SPMV_WARPS;
    TV* wbuf = buf[warp];
    TV* xbuf = xbuf_all[MODE == 1 ? warp : 0];
    double ss = 0.0;
    const TV sc = (MODE == 0 && scale) ? (TV)(*scale) : (TV)1;
    for (int tile = blockIdx.x * SPMV_WARPS + warp; tile * 32 < n; tile += nwarps) {
        const int r0 = tile * 32;
        const int r = r0 + lane;
        int rs = 0, re = 0;
        if (r < n) {
            rs = __ldg(&rp[r]);
            re = __ldg(&rp[r + 1]);
        }
        const int lastlane = min(31, n - 1 - r0);
        const int base = __shfl_sync(0xffffffffu, rs, 0);
        const int end = __shfl_sync(0xffffffffu, re, lastlane);
        TV sum = (TV)0;
        for (int ws = base; ws < end; ws += CAP) {
            const int we = min(ws + CAP, end);
            const int a0 = ws & ~(VN - 1);
            for (int e0 = a0 + lane * VN; e0 < we; e0 += 32 * VN) {
                TV v[VN];
                int c[VN];
                unpack<TV, VV>(__ldg(reinterpret_cast<const VV*>(val + e0)), v);
                unpacki(__ldg(reinterpret_cast<const VI*>(ci + e0)), c);
#pragma unroll
                for (int q = 0; q < VN; ++q) {
                    const int e = e0 + q;
                    if (e >= ws && e < we) {
                        if (MODE == 1) {
                            wbuf[e - ws] = v[q];
                            xbuf[e - ws] = (TV)__ldg(&x[c[q]]);
                        } else {
                            wbuf[e - ws] = pmul(v[q], (TV)__ldg(&x[c[q]]));
                        }
                    }
                }
            }
            __syncwarp();
            const int lo = max(rs, ws), hi = min(re, we);
            if (MODE == 1) {
                // the solver's FP64 true residual: fused multiply-adds in
                // entry order, the same bits as the SELL kernel
                for (int e = lo; e < hi; ++e) sum = fma(wbuf[e - ws], xbuf[e - ws], sum);
            } else {
                for (int e = lo; e < hi; ++e) sum = padd(sum, wbuf[e - ws]);
            }
            __syncwarp();
        }
        if (r < n) {
            if (MODE == 0) {
                y[r] = (TY)(MODE == 0 && scale ? pmul(sum, sc) : sum);
            } else {
                const double rv = __dsub_rn(b[r], (double)sum);
                y[r] = (TY)rv;
                ss += rv * rv;
            }
        }
    }
    if (MODE == 1) {
        __shared__ double red[SPMV_WARPS];
        __shared__ double bs[1], tot[1];
        double v1[1] = {ss};
        block_sum_multi<1>(v1, 1, red, bs);
        if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0) {
            const double rn = sqrt(tot[0]);
            st->rnorm = rn;
            // a new cycle starts from here: no basis vectors yet
            st->kcount = 0;
            st->j = 0;
            if (!isfinite(rn)) {
                st->nonfinite = 1;
                st->done = 1;
                st->cycle_active = 0;
            } else if (st->tol_kind != SG_TOL_REF_ABS && rn <= st->tol * st->bnorm) {
                st->converged = 1;
                st->done = 1;
                st->cycle_active = 0;
            } else {
                st->cycle_active = st->done ? 0 : 1;
            }
        }
    }
}

// column of SELL entry: absolute int32, or a 16-bit offset from the row
__device__ __forceinline__ int sell_col(const int* col, long long e, int, uint64_t pol) {
    return ldg_stream(&col[e], pol);
}
__device__ __forceinline__ int sell_col(const int16_t* col, long long e, int r, uint64_t pol) {
    return r + (int)ldg_stream(&col[e], pol);
}

// SELL-32 SpMV: a warp per slice of 32 rows, a lane per row; every load of
// a step k is one contiguous 32-element segment.  MODE 0: same per-row order
// and rounding as the CSR kernel (padding adds exact zeros at the end of a
// row); MODE 1 (the solver's true residual) fuses each product into the sum.
// TC = int: absolute columns; TC = int16_t: column - row (banded matrices
// such as grid stencils), 6 instead of 8 bytes per FP32 entry.
template <class TV, class TX, class TY, int MODE, class TC = int, int MINB = 4>
__global__ void __launch_bounds__(SPMV_THREADS, MINB)
k_spmv_sell(int n, int nslices, const long long* __restrict__ sptr, const int* __restrict__ sw,
            const TC* __restrict__ col, const TV* __restrict__ val, const TX* __restrict__ x,
            TY* __restrict__ y, const double* __restrict__ scale, const int* __restrict__ active,
            const double* __restrict__ b, double* partials, unsigned* counter, SolveState* st) {
    if (active && *active == 0) return;
    const int lane = threadIdx.x & 31;
    const uint64_t pol = policy_evict_first();  // the matrix streams past the basis
    const int nwarps = gridDim.x * SPMV_WARPS;
    double ss = 0.0;
    const TV sc = (MODE == 0 && scale) ? (TV)(*scale) : (TV)1;
    for (int sl = blockIdx.x * SPMV_WARPS + (threadIdx.x >> 5); sl < nslices; sl += nwarps) {
        const long long base = sptr[sl] + lane;
        const int w = sw[sl];
        const int row = sl * 32 + lane;
        TV sum = (TV)0;
        // up to 8 entries of a row per round: all value/column loads first,
        // then all gathers of x, then the sum in entry order
        for (int k = 0; k < w; k += 8) {
            TV v[8];
            int c[8];
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (k + q < w) {
                    v[q] = ldg_stream(&val[base + (long long)(k + q) * 32], pol);
                    c[q] = sell_col(col, base + (long long)(k + q) * 32, row, pol);
                }
            }
            TV p[8];
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (k + q < w) p[q] = (TV)__ldg(&x[c[q]]);
            if (MODE == 1) {
                // the solver's FP64 true residual: fused multiply-adds in
                // entry order (one FP64 instruction per entry instead of two)
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (k + q < w) sum = fma(v[q], p[q], sum);
            } else {
#pragma unroll
                for (int q = 0; q < 8; ++q)
                    if (k + q < w) sum = padd(sum, pmul(v[q], p[q]));
            }
        }
        const int r = sl * 32 + lane;
        if (r < n) {
            if (MODE == 0) {
                y[r] = (TY)(scale ? pmul(sum, sc) : sum);
            } else {
                const double rv = __dsub_rn(b[r], (double)sum);
                y[r] = (TY)rv;
                ss += rv * rv;
            }
        }
    }
    if (MODE == 1) {
        __shared__ double red[SPMV_WARPS];
        __shared__ double bs[1], tot[1];
        double v1[1] = {ss};
        block_sum_multi<1>(v1, 1, red, bs);
        if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0) {
            const double rn = sqrt(tot[0]);
            st->rnorm = rn;
            st->kcount = 0;
            st->j = 0;
            if (!isfinite(rn)) {
                st->nonfinite = 1;
                st->done = 1;
                st->cycle_active = 0;
            } else if (st->tol_kind != SG_TOL_REF_ABS && rn <= st->tol * st->bnorm) {
                st->converged = 1;
                st->done = 1;
                st->cycle_active = 0;
            } else {
                st->cycle_active = st->done ? 0 : 1;
            }
        }
    }
}

// SELL-32 for matrices whose slices hold at most 8 entries per row (grid
// stencils), software-pipelined: a warp issues the value/column loads of its
// next slice before it gathers x for the current one, so its DRAM requests
// stay in flight while the gathers (mostly L2 hits) complete.  Same per-row
// order and rounding as k_spmv_sell.
template <class TV, class TX, class TY, class TC, int MINB>
__global__ void __launch_bounds__(SPMV_THREADS, MINB)
k_spmv_sell_pipe(int n, int nslices, const long long* __restrict__ sptr,
                 const int* __restrict__ sw, const TC* __restrict__ col,
                 const TV* __restrict__ val, const TX* __restrict__ x, TY* __restrict__ y,
                 const double* __restrict__ scale, const int* __restrict__ active) {
    if (active && *active == 0) return;
    const int lane = threadIdx.x & 31;
    const uint64_t pol = policy_evict_first();
    const int nwarps = gridDim.x * SPMV_WARPS;
    const TV sc = scale ? (TV)(*scale) : (TV)1;
    int sl = blockIdx.x * SPMV_WARPS + (threadIdx.x >> 5);
    TV v[8], vn[8];
    int c[8], cn[8];
    int w = 0, wn = 0;
    auto load = [&](int s, TV (&vv)[8], int (&cc)[8], int& ww) {
        ww = sw[s];
        const long long base = sptr[s] + lane;
        const int row = s * 32 + lane;
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            if (q < ww) {
                vv[q] = ldg_stream(&val[base + (long long)q * 32], pol);
                cc[q] = sell_col(col, base + (long long)q * 32, row, pol);
            }
        }
    };
    if (sl < nslices) load(sl, v, c, w);
    while (sl < nslices) {
        const int nx = sl + nwarps;
        if (nx < nslices) load(nx, vn, cn, wn);
        TV p[8];
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < w) p[q] = pmul(v[q], (TV)__ldg(&x[c[q]]));
        TV sum = (TV)0;
#pragma unroll
        for (int q = 0; q < 8; ++q)
            if (q < w) sum = padd(sum, p[q]);
        const int r = sl * 32 + lane;
        if (r < n) y[r] = (TY)(scale ? pmul(sum, sc) : sum);
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            v[q] = vn[q];
            c[q] = cn[q];
        }
        w = wn;
        sl = nx;
    }
}

// grid of the SELL kernel: at most `per_sm` blocks per SM, warps loop over
// slices (MODE 1 reduces per block into the context's partials: 8 per SM)
int sell_grid(sg_ctx* ctx, int nslices, int per_sm = 8) {
    long long blocks = ((long long)nslices + SPMV_WARPS - 1) / SPMV_WARPS;
    const long long cap = (long long)ctx->num_sms * per_sm;
    if (blocks > cap) blocks = cap;
    return blocks < 1 ? 1 : (int)blocks;
}



template <class TV>
const TV* sell_vals(const sg_csr* A);
template <>
const double* sell_vals<double>(const sg_csr* A) { return A->sl_val.p; }
template <>
const float* sell_vals<float>(const sg_csr* A) { return A->sl_val32.p; }
template <class TV>
const TV* csr_vals(const sg_csr* A);
template <>
const double* csr_vals<double>(const sg_csr* A) { return A->val.p; }
template <>
const float* csr_vals<float>(const sg_csr* A) { return A->val32.p; }

// SELL launch variants the autotuner chooses from: columns (int32 or 16-bit
// offsets), registers (min 4 or 6 blocks per SM) and grid (blocks per SM)
struct SellCfg {
    bool dcol;
    int minb;
    int per_sm;
    bool pipe;  // software-pipelined kernel (slices of at most 8 entries per row)
};
constexpr SellCfg kSellCfgs[] = {
    {false, 4, 8, false}, {false, 6, 12, false}, {false, 6, 24, false},
    {true, 4, 8, false},  {true, 6, 12, false},  {true, 6, 24, false},
    {false, 4, 8, true},  {false, 4, 16, true},  {true, 4, 8, true},  {true, 4, 16, true}};
constexpr int kNumSellCfgs = (int)(sizeof(kSellCfgs) / sizeof(kSellCfgs[0]));

template <class TV, class TX, class TY>
void launch_sell(sg_ctx* ctx, const sg_csr* A, int cfg, const TX* x, TY* y, const double* scale,
                 const int* active) {
    const SellCfg c = kSellCfgs[cfg];
    const int grid = sell_grid(ctx, A->nslices, c.per_sm);
    if (c.pipe) {
        if (c.dcol)
            k_spmv_sell_pipe<TV, TX, TY, int16_t, 4><<<grid, SPMV_THREADS, 0, ctx->stream>>>(
                A->nrows, A->nslices, A->sl_ptr.p, A->sl_w.p, A->sl_dcol.p, sell_vals<TV>(A), x, y,
                scale, active);
        else
            k_spmv_sell_pipe<TV, TX, TY, int, 4><<<grid, SPMV_THREADS, 0, ctx->stream>>>(
                A->nrows, A->nslices, A->sl_ptr.p, A->sl_w.p, A->sl_col.p, sell_vals<TV>(A), x, y,
                scale, active);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        return;
    }
#define SG_SELL(TC, MB, COLS)                                                                   \
    k_spmv_sell<TV, TX, TY, 0, TC, MB><<<grid, SPMV_THREADS, 0, ctx->stream>>>(                  \
        A->nrows, A->nslices, A->sl_ptr.p, A->sl_w.p, COLS, sell_vals<TV>(A), x, y, scale, active, \
        nullptr, nullptr, nullptr, nullptr)
    if (c.dcol) {
        if (c.minb == 6) SG_SELL(int16_t, 6, A->sl_dcol.p);
        else SG_SELL(int16_t, 4, A->sl_dcol.p);
    } else {
        if (c.minb == 6) SG_SELL(int, 6, A->sl_col.p);
        else SG_SELL(int, 4, A->sl_col.p);
    }
#undef SG_SELL
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

__global__ void k_bnorm(const double* __restrict__ v, int n, double* partials, unsigned* counter,
                        SolveState* st) {
    double ss = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const double t = v[i];
        ss += t * t;
    }
    __shared__ double red[32];
    __shared__ double bs[1], tot[1];
    double v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0) {
        st->bnorm = sqrt(tot[0]);
        if (!isfinite(st->bnorm)) {
            st->nonfinite = 1;
            st->done = 1;
            st->cycle_active = 0;
        }
    }
}

int spmv_grid(sg_ctx* ctx, int n) {
    const long long tiles = (n + 31) / 32;
    long long blocks = (tiles + SPMV_WARPS - 1) / SPMV_WARPS;
    const long long cap = (long long)ctx->num_sms * 8;
    if (blocks > cap) blocks = cap;
    if (blocks < 1) blocks = 1;
    return (int)blocks;
}

}  // namespace

template <class TV, class TX, class TY>
void launch_spmv(sg_ctx* ctx, int n, const int* rp, const int* ci, const TV* val, const TX* x,
                 TY* y, const double* scale, const int* active) {
    if (n <= 0) return;
    k_spmv_csr<TV, TX, TY, 0><<<spmv_grid(ctx, n), SPMV_THREADS, 0, ctx->stream>>>(
        n, rp, ci, val, x, y, scale, active, nullptr, nullptr, nullptr, nullptr);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

void launch_residual(sg_ctx* ctx, const sg_csr* A, const double* b, const double* x, double* r,
                     SolveState* st) {
    if (A->format == 3 && A->sell_ok && A->sl_dcol.p) {
        k_spmv_sell<double, double, double, 1, int16_t><<<sell_grid(ctx, A->nslices),
                                                          SPMV_THREADS, 0, ctx->stream>>>(
            A->nrows, A->nslices, A->sl_ptr.p, A->sl_w.p, A->sl_dcol.p, A->sl_val.p, x, r,
            nullptr, nullptr, b, ctx->partials.p, ctx->counter.p, st);
    } else if (A->format >= 2 && A->sell_ok) {
        k_spmv_sell<double, double, double, 1><<<sell_grid(ctx, A->nslices), SPMV_THREADS, 0,
                                                 ctx->stream>>>(
            A->nrows, A->nslices, A->sl_ptr.p, A->sl_w.p, A->sl_col.p, A->sl_val.p, x, r, nullptr,
            nullptr, b, ctx->partials.p, ctx->counter.p, st);
    } else {
        k_spmv_csr<double, double, double, 1><<<spmv_grid(ctx, A->nrows), SPMV_THREADS, 0,
                                                ctx->stream>>>(
            A->nrows, A->rp.p, A->ci.p, A->val.p, x, r, nullptr, nullptr, b, ctx->partials.p,
            ctx->counter.p, st);
    }
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

// SELL launch variants (for sg_csr_set_spmv_variant): count, and per
// variant 0 = 16-bit column offsets, 1 = pipelined kernel
int sell_variant_count() { return kNumSellCfgs; }
int sell_variant_info(int v, int what) {
    return what == 0 ? (int)kSellCfgs[v].dcol : (int)kSellCfgs[v].pipe;
}

template <class TV>
int sell_cfg_of(const sg_csr* A);
template <>
int sell_cfg_of<double>(const sg_csr* A) { return A->sell_cfg; }
template <>
int sell_cfg_of<float>(const sg_csr* A) { return A->sell_cfg32; }

template <class TV>
int format_of(const sg_csr* A);
template <>
int format_of<double>(const sg_csr* A) { return A->format; }
template <>
int format_of<float>(const sg_csr* A) { return A->format32 ? A->format32 : A->format; }

template <class TV, class TX, class TY>
void launch_spmv_a(sg_ctx* ctx, const sg_csr* A, const TX* x, TY* y, const double* scale,
                   const int* active) {
    if (A->nrows <= 0) return;
    const int fmt = format_of<TV>(A);
    if (fmt >= 2 && A->sell_ok && (fmt == 2 || A->sl_dcol.p)) {
        // the tuned launch variant of this format (default: first of the format)
        int cfg = sell_cfg_of<TV>(A);
        if (cfg < 0 || kSellCfgs[cfg].dcol != (fmt == 3)) cfg = fmt == 3 ? 3 : 0;
        launch_sell<TV, TX, TY>(ctx, A, cfg, x, y, scale, active);
    } else {
        launch_spmv<TV, TX, TY>(ctx, A->nrows, A->rp.p, A->ci.p, csr_vals<TV>(A), x, y, scale,
                                active);
    }
}

// Autotuner: times CSR and the SELL launch variants (int32 or 16-bit column
// offsets, 4 or 6 resident blocks per SM, 8 to 24 blocks per SM in the grid)
// on A (5 launches each after a warm-up) and keeps the fastest, separately
// for the FP64 values and for the FP32 copy.  All formats give the same bits, so the
// choice never changes a result.  A format set by the caller
// (sg_csr_set_format) is left alone.
void spmv_autotune(sg_ctx* ctx, sg_csr* A) {
    if (A->format_user) return;
    const bool need64 = A->format == 0;
    const bool need32 = A->val32.p && A->format32 == 0;
    if (!need64 && !need32) return;
    if (!A->sell_ok || A->nrows < 4096) {
        if (need64) A->format = 1;
        if (need32) A->format32 = 1;
        return;
    }
    cudaEvent_t e0, e1;
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    auto time_it = [&](auto&& run) {
        run();
        SG_CUDA(cudaEventRecord(e0, ctx->stream));
        for (int i = 0; i < 5; ++i) run();
        SG_CUDA(cudaEventRecord(e1, ctx->stream));
        SG_CUDA(cudaEventSynchronize(e1));
        float ms = 0.f;
        SG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        return ms;
    };
    if (need64) {
        DBuf<double> xb, yb;
        xb.alloc(A->ncols);
        yb.alloc(A->nrows);
        xb.zero(ctx->stream);
        A->format = 1;
        float best = time_it([&] {
            launch_spmv_a<double, double, double>(ctx, A, xb.p, yb.p, nullptr, nullptr);
        });
        int bf = 1, bc = -1;
        for (int c = 0; c < kNumSellCfgs; ++c) {
            if (kSellCfgs[c].dcol && !A->sl_dcol.p) continue;
            if (kSellCfgs[c].pipe && A->sell_maxw > 8) continue;
            const float t = time_it([&] {
                launch_sell<double, double, double>(ctx, A, c, xb.p, yb.p, nullptr, nullptr);
            });
            if (t < best) {
                best = t;
                bf = kSellCfgs[c].dcol ? 3 : 2;
                bc = c;
            }
        }
        A->format = bf;
        A->sell_cfg = bc;
    }
    if (need32 && A->sl_val32.p) {
        DBuf<float> xb, yb;
        xb.alloc(A->ncols);
        yb.alloc(A->nrows);
        xb.zero(ctx->stream);
        A->format32 = 1;
        float best = time_it([&] {
            launch_spmv_a<float, float, float>(ctx, A, xb.p, yb.p, nullptr, nullptr);
        });
        int bf = 1, bc = -1;
        for (int c = 0; c < kNumSellCfgs; ++c) {
            if (kSellCfgs[c].dcol && !A->sl_dcol.p) continue;
            if (kSellCfgs[c].pipe && A->sell_maxw > 8) continue;
            const float t = time_it([&] {
                launch_sell<float, float, float>(ctx, A, c, xb.p, yb.p, nullptr, nullptr);
            });
            if (t < best) {
                best = t;
                bf = kSellCfgs[c].dcol ? 3 : 2;
                bc = c;
            }
        }
        A->format32 = bf;
        A->sell_cfg32 = bc;
    } else if (need32) {
        A->format32 = 1;
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

void launch_bnorm(sg_ctx* ctx, const double* v, int n, SolveState* st) {
    int blocks = ctx->num_sms * 2;
    k_bnorm<<<blocks, 512, 0, ctx->stream>>>(v, n, ctx->partials.p, ctx->counter.p, st);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template void launch_spmv<double, double, double>(sg_ctx*, int, const int*, const int*,
                                                  const double*, const double*, double*,
                                                  const double*, const int*);
template void launch_spmv<float, float, float>(sg_ctx*, int, const int*, const int*,
                                               const float*, const float*, float*,
                                               const double*, const int*);
template void launch_spmv_a<double, double, double>(sg_ctx*, const sg_csr*, const double*,
                                                    double*, const double*, const int*);
template void launch_spmv_a<float, float, float>(sg_ctx*, const sg_csr*, const float*, float*,
                                                 const double*, const int*);
// FP32 values, FP64 input (the learned stage's residual inside an FP64 cycle)
template void launch_spmv_a<float, double, float>(sg_ctx*, const sg_csr*, const double*, float*,
                                                  const double*, const int*);

}  // namespace sg
