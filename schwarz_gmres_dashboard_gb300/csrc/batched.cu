// batched.cu -- many independent systems solved at once: A_s x = b_{s,r} for
// s < S systems of uneven sizes and r < R right-hand sides each, every
// (s, r) pair an independent restarted GMRES(m) (src/core/gmres.cpp:34-160)
// with its own Krylov space, Givens rotations and stopping test.
//
// Layout.  The systems form one block-diagonal matrix A (rows of system s at
// [row_ptr[s], row_ptr[s+1])) and the preconditioner is set up on A with a
// partition whose parts never cross a system, so one set-up and one launch of
// the subdomain sweeps serve every system (the sweeps of all subdomains of
// all systems run as one batched kernel).  Vectors of the batch are laid out
// [r][N] (N = rows of A); instance i = r * S + s owns the segment
// [r*N + row_ptr[s], r*N + row_ptr[s+1]).
//
// Reductions.  Every instance is cut into chunks of at most 2048 rows, one
// block per chunk.  A block writes its partial sums to its chunk's slot; the
// last block of an instance to arrive (per-instance ticket) adds the chunk
// partials in chunk order (deterministic) and updates that instance's state.
// All instances step in lockstep through the restart cycle (one CUDA graph);
// an instance that converges, breaks down or reaches the end of its cycle
// clears its active flag and every later kernel of the cycle skips it.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int BT = 256;               // threads per block
constexpr int BRPT = 8;               // rows per thread
constexpr int BCH = BT * BRPT;        // rows per chunk
constexpr int BMMAX = 32;             // restart limit of the batched solver
constexpr int BLD = BMMAX + 1;        // stride of the chunk partials

struct BatchDev {
    // instances (I = S * R)
    const long long* ioff;  // first element of instance i
    const int* in;          // rows
    const int* ich0;        // first chunk
    const int* inch;        // number of chunks
    // chunks
    const int* cinst;
    const long long* coff;
    const int* clen;
    // per-instance state
    int* active;     // 1 while the steps of the current cycle run
    int* done;       // finished (converged, out of iterations or failed)
    int* conv;
    int* iters;
    int* cycles;
    int* kcount;     // basis vectors of the current cycle
    int* ran;        // took part in the current cycle
    int* flags;      // bit 0 non-finite, bit 1 breakdown
    double* bnorm;
    double* rnorm;
    double* est;     // rnorm / beta of the cycle start
    double* lastres;
    double* g;       // [I][m+1]
    double* cs;      // [I][m]
    double* sn;
    double* H;       // [I][(m+1) m], column-major, ld m+1
    double* vscale;  // [I][m+1]
    double* y;       // [I][m]
    float* yf;       // [I][m] y_k * vscale_k in FP32 (update of an FP32 basis)
    double* yd;      // [I][m] y_k * vscale_k in FP64
    double* h;       // [I][m+1] coefficients of the current pass
    double* hs;      // [I][m+1] h1 + h2
    unsigned* ticket;
    double* part;    // [chunks][BLD]
    int* notdone;
    // lagged CGS2 (ortho 0): the basis is V = S T over the stored vectors S
    double* lagT;    // [I][BLD * BLD] T(l, i) at l + i * BLD (upper triangle)
    double* lagH;    // [I][BLD * BMMAX] unrotated Hessenberg H(i, k) at i + k * BLD
    double* lagc;    // [I][BLD] v_j = T(j,j) raw_j - sum_{k<j} lagc[k] v_k
    double* cfu;     // [I][BLD] update coefficients on the stored vectors
    int lagged;
    // compacted launches (late cycles): the chunks of the instances still
    // running and the SELL slices of their systems; null = all
    const int* clist;
    const int* slist;
    int nslist;
    int m, I, S, R;
    long long N;
    double tol;
    int tol_kind, max_iter;
};

// the chunk of this block: block b of a compacted launch takes the b-th
// chunk of the list, otherwise chunk b
__device__ __forceinline__ int chunk_of(const BatchDev& B) {
    return B.clist ? B.clist[blockIdx.x] : (int)blockIdx.x;
}

__device__ void b_rot_compute(double& c, double& s, double a, double b) {
    // src/core/gmres.cpp:9-30
    if (fabs(b) < 1e-30) {
        c = 1.0;
        s = 0.0;
    } else if (fabs(b) > fabs(a)) {
        const double t = -a / b;
        s = 1.0 / sqrt(1.0 + t * t);
        c = s * t;
    } else {
        const double t = -b / a;
        c = 1.0 / sqrt(1.0 + t * t);
        s = c * t;
    }
}
__device__ void b_rot_apply(double c, double s, double& h1, double& h2) {
    const double t1 = c * h1 - s * h2;
    const double t2 = s * h1 + c * h2;
    h1 = t1;
    h2 = t2;
}

// Block sums of nv per-thread values (warp shuffles, then one pass over the
// warps), then the instance-level sum by the last chunk of the instance.
// Returns true in that last block with the totals in out[0..nv).
__device__ bool seg_reduce(const BatchDev& B, int c, int inst, double (*red)[BLD], int nv,
                           double* bsum, double* out) {
    __shared__ unsigned s_t;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < BT / 32; ++w) s += red[w][k];
        bsum[k] = s;
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += blockDim.x) B.part[(size_t)c * BLD + k] = bsum[k];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_t = atomicAdd(&B.ticket[inst], 1u);
    __syncthreads();
    if (s_t != (unsigned)B.inch[inst] - 1) return false;
    __threadfence();
    const int c0 = B.ich0[inst], nc = B.inch[inst];
    for (int k = warp; k < nv; k += BT / 32) {
        double s = 0.0;
        for (int q = lane; q < nc; q += 32) s += __ldcg(&B.part[(size_t)(c0 + q) * BLD + k]);
        s = warp_sum(s);
        if (lane == 0) out[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) B.ticket[inst] = 0u;
    return true;
}

// ---- FP64 residual r = b - A x per instance (mode 1), or ||b|| (mode 0);
// the last block of an instance runs the restart test.
template <int MODE>
__global__ void __launch_bounds__(BT)
k_b_residual(BatchDev B, const int* __restrict__ rp, const int* __restrict__ ci,
             const double* __restrict__ val, const double* __restrict__ b,
             const double* __restrict__ x, double* __restrict__ r) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (MODE == 1 && B.done[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[1], tot[1];
    const long long off = B.coff[c];
    const int len = B.clen[c];
    const int rr = inst / B.S;
    const long long base = (long long)rr * B.N;
    double ss = 0.0;
    for (int q = threadIdx.x; q < len; q += BT) {
        const long long e = off + q;
        double v = b[e];
        if (MODE == 1) {
            const long long mr = e - base;
            double ax = 0.0;
            for (int k = rp[mr]; k < rp[mr + 1]; ++k) ax = fma(val[k], x[base + ci[k]], ax);
            v = v - ax;
            r[e] = v;
        }
        ss += v * v;
    }
    ss = warp_sum(ss);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = ss;
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, 1, bsum, tot) || threadIdx.x != 0) return;
    const double rn = sqrt(tot[0]);
    if (MODE == 0) {
        B.bnorm[inst] = rn;
        if (!isfinite(rn)) {
            B.flags[inst] |= 1;
            B.done[inst] = 1;
        }
        return;
    }
    B.rnorm[inst] = rn;
    B.kcount[inst] = 0;
    if (!isfinite(rn)) {
        B.flags[inst] |= 1;
        B.done[inst] = 1;
    } else if (B.tol_kind != SG_TOL_REF_ABS && rn <= B.tol * B.bnorm[inst]) {
        B.conv[inst] = 1;
        B.done[inst] = 1;
    }
    B.active[inst] = B.done[inst] ? 0 : 1;
}

// ---- cycle start: beta = ||raw_0|| per instance, g = beta e1, vscale_0 = 1/beta
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_cycle_init(BatchDev B, const TV* __restrict__ raw0) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[1], tot[1];
    const long long off = B.coff[c];
    const int len = B.clen[c];
    TV ssv = (TV)0;
    for (int q = threadIdx.x; q < len; q += BT) {
        const TV t = ld_stream(&raw0[off + q]);
        ssv += t * t;
    }
    const double ss = warp_sum((double)ssv);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = ss;
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, 1, bsum, tot)) return;
    const int m = B.m, ld = m + 1;
    for (int i = threadIdx.x; i < ld * m; i += BT) B.H[(size_t)inst * ld * m + i] = 0.0;
    for (int i = threadIdx.x; i <= m; i += BT) B.g[(size_t)inst * ld + i] = 0.0;
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double beta = sqrt(tot[0]);
    B.kcount[inst] = 0;
    B.ran[inst] = 1;
    B.flags[inst] &= ~2;
    if (!isfinite(beta)) {
        B.flags[inst] |= 1;
        B.done[inst] = 1;
        B.active[inst] = 0;
        return;
    }
    if (B.tol_kind == SG_TOL_REF_ABS && beta < B.tol) {
        B.conv[inst] = 1;
        B.done[inst] = 1;
        B.active[inst] = 0;
        return;
    }
    if (!(beta > 0.0)) {
        B.done[inst] = 1;
        B.active[inst] = 0;
        return;
    }
    B.vscale[(size_t)inst * ld] = 1.0 / beta;
    if (B.lagged) B.lagT[(size_t)inst * BLD * BLD] = 1.0 / beta;  // v_0 = raw_0 / beta
    B.g[(size_t)inst * ld] = beta;
    B.est[inst] = B.rnorm[inst] / beta;
}

// ---- y = vscale_j * (A x) for the active instances (FP32 or FP64 basis)
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_spmv(BatchDev B, const int* __restrict__ rp, const int* __restrict__ ci,
         const TV* __restrict__ val, const int* __restrict__ row_sys, const TV* __restrict__ x,
         TV* __restrict__ y, int j) {
    const long long total = B.N * B.R;
    const int ld = B.m + 1;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int rr = (int)(q / B.N);
        const long long mr = q - (long long)rr * B.N;
        const int inst = rr * B.S + row_sys[mr];
        if (!B.active[inst]) continue;
        const TV* xb = x + (long long)rr * B.N;
        TV acc = (TV)0;
        for (int k = rp[mr]; k < rp[mr + 1]; ++k) acc += val[k] * xb[ci[k]];
        y[q] = (TV)((double)acc * B.vscale[(size_t)inst * ld + j]);
    }
}

// The same product from the SELL-32 copy of A (slices of 32 rows, entries
// column-major within a slice: a warp's loads of values and columns are
// coalesced), for up to four right-hand sides at once: each matrix entry is
// read once for all of them.  Per row the products are summed in the CSR
// order (padding adds exact zeros at the end), as k_b_spmv does.
constexpr int BSR = 4;  // right-hand sides per pass over the matrix
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_spmv_sell(BatchDev B, const long long* __restrict__ sl_ptr, const int* __restrict__ sl_w,
              const int* __restrict__ sl_col, const TV* __restrict__ sl_val,
              const int* __restrict__ row_sys, int nslices, const TV* __restrict__ x,
              TV* __restrict__ y, int j) {
    const int lane = threadIdx.x & 31;
    const int ld = B.m + 1;
    const int wstride = (gridDim.x * blockDim.x) >> 5;
    const int nsl = B.slist ? B.nslist : nslices;
    for (int li = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; li < nsl; li += wstride) {
        const int sl = B.slist ? B.slist[li] : li;
        const long long row = (long long)sl * 32 + lane;
        const bool in = row < B.N;
        const int sys = in ? row_sys[row] : 0;
        const long long base = sl_ptr[sl] + lane;
        const int w = sl_w[sl];
        for (int r0 = 0; r0 < B.R; r0 += BSR) {
            bool act[BSR];
            bool any = false;
#pragma unroll
            for (int u = 0; u < BSR; ++u) {
                act[u] = in && r0 + u < B.R && B.active[(r0 + u) * B.S + sys];
                any |= act[u];
            }
            if (!__any_sync(0xffffffffu, any)) continue;
            TV acc[BSR];
#pragma unroll
            for (int u = 0; u < BSR; ++u) acc[u] = (TV)0;
            for (int k = 0; k < w; ++k) {
                const int c = __ldg(&sl_col[base + 32ll * k]);
                const TV v = ld_stream(&sl_val[base + 32ll * k]);
#pragma unroll
                for (int u = 0; u < BSR; ++u)
                    if (act[u]) acc[u] += v * x[(long long)(r0 + u) * B.N + c];
            }
#pragma unroll
            for (int u = 0; u < BSR; ++u)
                if (act[u])
                    y[(long long)(r0 + u) * B.N + row] =
                        (TV)((double)acc[u] * B.vscale[(size_t)((r0 + u) * B.S + sys) * ld + j]);
        }
    }
}

// red[warp][k] = warp sums of raw_k . wv (k <= j) for a chunk: four
// vectors' loads in flight at a time; per vector the products are summed
// over the thread's rows in row order, then across the warp
constexpr int BKG = 4;
template <class TV>
__device__ __forceinline__ void chunk_dots(const TV* V, size_t ldv, long long off, int len, int j,
                                           const TV (&wv)[BRPT], double (*red)[BLD]) {
    for (int k0 = 0; k0 <= j; k0 += BKG) {
        TV a[BKG][BRPT];
#pragma unroll
        for (int kk = 0; kk < BKG; ++kk) {
            const TV* vk = V + (size_t)(k0 + kk) * ldv + off;
#pragma unroll
            for (int q = 0; q < BRPT; ++q) {
                const int row = threadIdx.x + q * BT;
                a[kk][q] = (k0 + kk <= j && row < len) ? ld_stream(&vk[row]) : (TV)0;
            }
        }
#pragma unroll
        for (int kk = 0; kk < BKG; ++kk) {
            if (k0 + kk > j) break;
            TV acc = (TV)0;
#pragma unroll
            for (int q = 0; q < BRPT; ++q) {
                const int row = threadIdx.x + q * BT;
                if (row < len) acc += a[kk][q] * wv[q];
            }
            const double v = warp_sum((double)acc);
            if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][k0 + kk] = v;
        }
    }
}

// wv -= sum_{k <= j} cf[k] raw_k over a chunk, k in order, four vectors'
// loads in flight at a time
template <class TV>
__device__ __forceinline__ void chunk_update(const TV* V, size_t ldv, long long off, int len, int j,
                                             const TV* cf, TV (&wv)[BRPT]) {
    for (int k0 = 0; k0 <= j; k0 += BKG) {
        TV a[BKG][BRPT];
#pragma unroll
        for (int kk = 0; kk < BKG; ++kk) {
            const TV* vk = V + (size_t)(k0 + kk) * ldv + off;
#pragma unroll
            for (int q = 0; q < BRPT; ++q) {
                const int row = threadIdx.x + q * BT;
                a[kk][q] = (k0 + kk <= j && row < len) ? ld_stream(&vk[row]) : (TV)0;
            }
        }
#pragma unroll
        for (int kk = 0; kk < BKG; ++kk) {
            if (k0 + kk > j) break;
            const TV ck = cf[k0 + kk];
#pragma unroll
            for (int q = 0; q < BRPT; ++q) {
                const int row = threadIdx.x + q * BT;
                if (row < len) wv[q] -= ck * a[kk][q];
            }
        }
    }
}

// ---- CGS2 pass A: h1_k = vscale_k (raw_k . w), k <= j
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_dots(BatchDev B, const TV* __restrict__ V, size_t ldv, int j) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[BLD], tot[BLD];
    const long long off = B.coff[c];
    const int len = B.clen[c];
    const TV* w = V + (size_t)(j + 1) * ldv + off;
    // per-thread products and sums in the basis precision (FP64 arithmetic
    // is scarce on this GPU), warp and block sums in FP64; the vectors are
    // streamed (256-byte L2 fetches)
    TV wv[BRPT];
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        wv[q] = row < len ? ld_stream(&w[row]) : (TV)0;
    }
    chunk_dots<TV>(V, ldv, off, len, j, wv, red);
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, j + 1, bsum, tot)) return;
    const int ld = B.m + 1;
    for (int k = threadIdx.x; k <= j; k += BT)
        B.h[(size_t)inst * ld + k] = B.vscale[(size_t)inst * ld + k] * tot[k];
}

// ---- CGS2 pass B: w' = w - sum_k h1_k v_k ; h2_k = vscale_k (raw_k . w');
// hs = h1 + h2, h = h2
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_upd_dots(BatchDev B, TV* __restrict__ V, size_t ldv, int j) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[BLD], tot[BLD];
    __shared__ TV cf[BLD];
    const int ld = B.m + 1;
    for (int k = threadIdx.x; k <= j; k += BT)
        cf[k] = (TV)(B.h[(size_t)inst * ld + k] * B.vscale[(size_t)inst * ld + k]);
    __syncthreads();
    const long long off = B.coff[c];
    const int len = B.clen[c];
    TV* w = V + (size_t)(j + 1) * ldv + off;
    TV wv[BRPT];
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        wv[q] = row < len ? ld_stream(&w[row]) : (TV)0;
    }
    chunk_update<TV>(V, ldv, off, len, j, cf, wv);
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        if (row < len) w[row] = wv[q];
    }
    chunk_dots<TV>(V, ldv, off, len, j, wv, red);
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, j + 1, bsum, tot)) return;
    for (int k = threadIdx.x; k <= j; k += BT) {
        const double h2 = B.vscale[(size_t)inst * ld + k] * tot[k];
        B.hs[(size_t)inst * ld + k] = B.h[(size_t)inst * ld + k] + h2;
        B.h[(size_t)inst * ld + k] = h2;
    }
}

// End of Arnoldi step j of one instance (one thread), as the single-system
// solver: the Hessenberg column (h_{0..j} from hs, h_{j+1} = nrm), the
// Givens rotations, the residual estimate and the stopping tests.  Returns
// true while the instance continues with step j + 1 (vscale_{j+1} = 1/nrm).
__device__ bool b_arnoldi_end(const BatchDev& B, int inst, int j, double nrm) {
    const int m = B.m, ld = m + 1;
    double* Hc = B.H + (size_t)inst * ld * m + (size_t)j * ld;
    double* g = B.g + (size_t)inst * ld;
    double* cs = B.cs + (size_t)inst * m;
    double* sn = B.sn + (size_t)inst * m;
    for (int i = 0; i <= j; ++i) Hc[i] = B.hs[(size_t)inst * ld + i];
    Hc[j + 1] = nrm;
    if (!(nrm >= 1e-30)) {
        if (!isfinite(nrm)) {
            B.flags[inst] |= 1;
            B.done[inst] = 1;
        }
        B.flags[inst] |= 2;
        B.kcount[inst] = j + 1;
        B.active[inst] = 0;
        return false;
    }
    B.vscale[(size_t)inst * ld + j + 1] = 1.0 / nrm;
    for (int i = 0; i < j; ++i) b_rot_apply(cs[i], sn[i], Hc[i], Hc[i + 1]);
    b_rot_compute(cs[j], sn[j], Hc[j], Hc[j + 1]);
    b_rot_apply(cs[j], sn[j], Hc[j], Hc[j + 1]);
    b_rot_apply(cs[j], sn[j], g[j], g[j + 1]);
    const double res = fabs(g[j + 1]);
    B.lastres[inst] = res;
    B.iters[inst] += 1;
    B.kcount[inst] = j + 1;
    bool stop = false;
    if (B.tol_kind == SG_TOL_REF_ABS) {
        if (res < B.tol) {
            B.conv[inst] = 1;
            B.done[inst] = 1;
            stop = true;
        }
    } else if (B.tol_kind == SG_TOL_TRUE_REL) {
        if (res * B.est[inst] <= 0.5 * B.tol * B.bnorm[inst]) stop = true;
    }
    if (!isfinite(res)) {
        B.flags[inst] |= 1;
        B.done[inst] = 1;
        stop = true;
    }
    if (j + 1 >= m) stop = true;
    if (stop) B.active[inst] = 0;
    return !stop;
}

// ---- CGS2 pass C: w'' = w' - sum_k h2_k v_k, ||w''||, then the instance's
// Hessenberg column, Givens rotations and stopping test
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_upd_norm(BatchDev B, TV* __restrict__ V, size_t ldv, int j) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[1], tot[1];
    __shared__ TV cf[BLD];
    const int m = B.m, ld = m + 1;
    for (int k = threadIdx.x; k <= j; k += BT)
        cf[k] = (TV)(B.h[(size_t)inst * ld + k] * B.vscale[(size_t)inst * ld + k]);
    __syncthreads();
    const long long off = B.coff[c];
    const int len = B.clen[c];
    TV* w = V + (size_t)(j + 1) * ldv + off;
    TV wv[BRPT];
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        wv[q] = row < len ? ld_stream(&w[row]) : (TV)0;
    }
    chunk_update<TV>(V, ldv, off, len, j, cf, wv);
    TV ssv = (TV)0;
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        if (row < len) {
            w[row] = wv[q];
            ssv += wv[q] * wv[q];
        }
    }
    double ss = warp_sum((double)ssv);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][0] = ss;
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, 1, bsum, tot) || threadIdx.x != 0) return;
    b_arnoldi_end(B, inst, j, sqrt(tot[0]));
}

// ---- lagged CGS2 (ortho 0, restart < 32), as the single-system solver.
// Step j orthogonalises z = B (vscale_j raw_j), where the stored raw_j still
// lacks its second projection: v_j = T(j,j) raw_j - sum_{k<j} c_k v_k, so
// B v_j = z - V g with g = H(0..j, 0..j-1) c (Arnoldi relation), and two
// passes over the stored vectors S (V = S T) do the work of three:
//   A  d = S^T z; p = T^T d; hs = p - g; update coefficients u = T p
//   B  w' = z - S u; r = S^T w'; ||w'||^2; h2 = T^T r; the column is hs +
//      h2, ||w''||^2 = ||w'||^2 - ||h2||^2, and w' is stored as raw_{j+1}
//      with its pending correction c = h2 / ||w''||.
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_lag_a(BatchDev B, const TV* __restrict__ V, size_t ldv, int j) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[BLD], tot[BLD];
    __shared__ double Ts[BLD][BLD + 1];
    __shared__ double ps[BLD], csh[BLD];
    const long long off = B.coff[c];
    const int len = B.clen[c];
    const TV* w = V + (size_t)(j + 1) * ldv + off;
    TV wv[BRPT];
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        wv[q] = row < len ? ld_stream(&w[row]) : (TV)0;
    }
    chunk_dots<TV>(V, ldv, off, len, j, wv, red);
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, j + 1, bsum, tot)) return;
    const int ld = B.m + 1, n1 = j + 1;
    const double* T = B.lagT + (size_t)inst * BLD * BLD;
    const double* Hn = B.lagH + (size_t)inst * BLD * BMMAX;
    for (int idx = threadIdx.x; idx < n1 * n1; idx += BT) {
        const int l = idx % n1, i = idx / n1;
        Ts[l][i] = l <= i ? T[l + i * BLD] : 0.0;
    }
    for (int k = threadIdx.x; k < j; k += BT) csh[k] = B.lagc[(size_t)inst * BLD + k];
    __syncthreads();
    for (int i = threadIdx.x; i <= j; i += BT) {
        double sp = 0.0;
        for (int l = 0; l <= i; ++l) sp += Ts[l][i] * tot[l];
        ps[i] = sp;
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= j; i += BT) {
        double g = 0.0;
        for (int k = (i > 0 ? i - 1 : 0); k < j; ++k) g += Hn[i + k * BLD] * csh[k];
        B.hs[(size_t)inst * ld + i] = ps[i] - g;
        double u = 0.0;
        for (int k = i; k <= j; ++k) u += Ts[i][k] * ps[k];
        B.cfu[(size_t)inst * BLD + i] = u;
    }
}

template <class TV>
__global__ void __launch_bounds__(BT)
k_b_lag_b(BatchDev B, TV* __restrict__ V, size_t ldv, int j) {
    const int c = chunk_of(B);
    const int inst = B.cinst[c];
    if (!B.active[inst]) return;
    __shared__ double red[BT / 32][BLD];
    __shared__ double bsum[BLD], tot[BLD];
    __shared__ TV cf[BLD];
    __shared__ double Ts[BLD][BLD + 1];
    __shared__ double h2s[BLD], csn[BLD];
    __shared__ double s_vs;
    for (int k = threadIdx.x; k <= j; k += BT) cf[k] = (TV)B.cfu[(size_t)inst * BLD + k];
    __syncthreads();
    const long long off = B.coff[c];
    const int len = B.clen[c];
    TV* w = V + (size_t)(j + 1) * ldv + off;
    TV wv[BRPT];
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        wv[q] = row < len ? ld_stream(&w[row]) : (TV)0;
    }
    chunk_update<TV>(V, ldv, off, len, j, cf, wv);
    TV ssv = (TV)0;
#pragma unroll
    for (int q = 0; q < BRPT; ++q) {
        const int row = threadIdx.x + q * BT;
        if (row < len) {
            w[row] = wv[q];
            ssv += wv[q] * wv[q];
        }
    }
    chunk_dots<TV>(V, ldv, off, len, j, wv, red);
    const double ss = warp_sum((double)ssv);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5][j + 1] = ss;
    __syncthreads();
    if (!seg_reduce(B, c, inst, red, j + 2, bsum, tot)) return;
    const int ld = B.m + 1, n1 = j + 1;
    double* T = B.lagT + (size_t)inst * BLD * BLD;
    double* Hn = B.lagH + (size_t)inst * BLD * BMMAX;
    for (int idx = threadIdx.x; idx < n1 * n1; idx += BT) {
        const int l = idx % n1, i = idx / n1;
        Ts[l][i] = l <= i ? T[l + i * BLD] : 0.0;
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= j; i += BT) {
        double h2 = 0.0;
        for (int l = 0; l <= i; ++l) h2 += Ts[l][i] * tot[l];
        h2s[i] = h2;
        const double hc = B.hs[(size_t)inst * ld + i] + h2;  // the Hessenberg column
        B.hs[(size_t)inst * ld + i] = hc;
        Hn[i + j * BLD] = hc;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double nrm2 = tot[j + 1];
        for (int i = 0; i <= j; ++i) nrm2 -= h2s[i] * h2s[i];
        if (!(nrm2 > 0.0)) nrm2 = isfinite(nrm2) ? 0.0 : nrm2;
        const double nrm = sqrt(nrm2);
        Hn[j + 1 + j * BLD] = nrm;
        s_vs = b_arnoldi_end(B, inst, j, nrm) ? 1.0 / nrm : 0.0;
    }
    __syncthreads();
    const double vs = s_vs;
    if (vs == 0.0) return;
    // the pending correction of the new stored vector and its column of T:
    // T(:, j+1) = T(j+1, j+1) e_{j+1} - T(:, 0..j) c
    for (int k = threadIdx.x; k <= j; k += BT) {
        csn[k] = h2s[k] * vs;
        B.lagc[(size_t)inst * BLD + k] = csn[k];
    }
    if (threadIdx.x == 0) T[(j + 1) + (j + 1) * BLD] = vs;
    __syncthreads();
    for (int l = threadIdx.x; l <= j; l += BT) {
        double sc = 0.0;
        for (int k = l; k <= j; ++k) sc += Ts[l][k] * csn[k];
        T[l + (j + 1) * BLD] = -sc;
    }
}

// ---- y = H^{-1} g per instance (src/core/gmres.cpp:131-137)
__global__ void k_b_backsolve(BatchDev B) {
    const int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= B.I || !B.ran[inst]) return;
    const int k = B.kcount[inst];
    const int m = B.m, ld = m + 1;
    const double* H = B.H + (size_t)inst * ld * m;
    const double* g = B.g + (size_t)inst * ld;
    double* y = B.y + (size_t)inst * m;
    for (int i = k - 1; i >= 0; --i) {
        double yi = g[i];
        for (int l = i + 1; l < k; ++l) yi -= H[i + l * ld] * y[l];
        y[i] = yi / H[i + i * ld];
    }
    // coefficients of the update x += sum_k (y_k vscale_k) raw_k; lagged
    // CGS2: V y = S (T y)
    const double* vs = B.vscale + (size_t)inst * ld;
    const double* T = B.lagged ? B.lagT + (size_t)inst * BLD * BLD : nullptr;
    for (int i = 0; i < k; ++i) {
        double c = 0.0;
        if (T) {
            for (int l = i; l < k; ++l) c += T[i + l * BLD] * y[l];
        } else {
            c = y[i] * vs[i];
        }
        B.yd[(size_t)inst * m + i] = c;
        B.yf[(size_t)inst * m + i] = (float)c;
    }
}

template <class TV>
__device__ __forceinline__ const TV* ycoef(const BatchDev& B);
template <>
__device__ __forceinline__ const float* ycoef<float>(const BatchDev& B) { return B.yf; }
template <>
__device__ __forceinline__ const double* ycoef<double>(const BatchDev& B) { return B.yd; }

// ---- x += sum_k y_k vscale_k raw_k (correction in the basis precision)
template <class TV>
__global__ void __launch_bounds__(BT)
k_b_update_x(BatchDev B, const TV* __restrict__ V, size_t ldv, const int* __restrict__ row_sys,
             double* __restrict__ x) {
    const long long total = B.N * B.R;
    const int m = B.m;
    for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < total;
         q += (long long)gridDim.x * blockDim.x) {
        const int rr = (int)(q / B.N);
        const int inst = rr * B.S + row_sys[q - (long long)rr * B.N];
        if (!B.ran[inst]) continue;
        const int k = B.kcount[inst];
        const TV* cf = ycoef<TV>(B) + (size_t)inst * m;
        TV d = (TV)0;
        for (int i = 0; i < k; ++i) d += cf[i] * ld_stream(&V[(size_t)i * ldv + q]);
        x[q] += (double)d;
    }
}

// ---- per-subdomain switches of the next applies: subdomain p of the
// preconditioner is swept for rhs r only while instance r*S + psys[p] is active
__global__ void k_b_subon(BatchDev B, const int* __restrict__ psys, int P, int* __restrict__ on) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= P * B.R) return;
    const int rr = q / P, p = q - rr * P;
    on[q] = B.active[rr * B.S + psys[p]];
}

// ---- restart bookkeeping per instance; counts the unfinished instances
__global__ void k_b_cycle_end(BatchDev B) {
    const int inst = blockIdx.x * blockDim.x + threadIdx.x;
    if (inst >= B.I) return;
    if (B.ran[inst]) {
        B.cycles[inst] += 1;
        B.ran[inst] = 0;
    }
    if (!B.done[inst] && B.iters[inst] >= B.max_iter) B.done[inst] = 1;
    B.active[inst] = B.done[inst] ? 0 : 1;
    if (!B.done[inst]) atomicAdd(B.notdone, 1);
}

int bgrid(sg_ctx* ctx, long long n) {
    const long long need = (n + BT - 1) / BT;
    const long long cap = (long long)ctx->num_sms * 8;
    return (int)std::max<long long>(1, std::min(need, cap));
}

template <class T>
void dalloc(DBuf<T>& b, size_t n) {
    if (b.n < n) b.alloc(n);
}

}  // namespace

struct BatchWork {
    DBuf<long long> ioff, coff;
    DBuf<int> in, ich0, inch, cinst, clen, row_sys;
    DBuf<int> active, done, conv, iters, cycles, kcount, ran, flags, notdone;
    DBuf<double> bnorm, rnorm, est, lastres, g, cs, sn, H, vscale, y, yd, h, hs, part;
    DBuf<double> lagT, lagH, lagc, cfu;
    // compacted launches: chunk and SELL-slice lists, host copies of the
    // instances' chunk ranges
    DBuf<int> clist, slist;
    std::vector<int> h_ich0, h_inch;
    DBuf<float> yf;
    DBuf<unsigned> ticket;
    DBuf<double> b64, x64, r64;
    DBuf<float> V32, t32;
    DBuf<double> V64, t64;
    int* h_notdone = nullptr;
    // what the instance/chunk tables and the checks were made for
    const sg_csr* key_A = nullptr;
    long long key_nnz = -1;
    int key_nrhs = -1;
    std::vector<int> key_rows;
    const sg_precond* key_pc = nullptr;
    uint64_t key_pc_structure = 0;
    int nchunks = 0;
    // subdomain -> system of key_pc, and the per-rhs subdomain switches
    DBuf<int> psys, sub_on;
    int psys_parts = 0;
    ~BatchWork() {
        if (h_notdone) cudaFreeHost(h_notdone);
    }
};

void destroy_batch_work(BatchWork* w) { delete w; }

namespace {

template <class TV>
struct BBasis;
template <>
struct BBasis<float> {
    static DBuf<float>& V(BatchWork* w) { return w->V32; }
    static DBuf<float>& T(BatchWork* w) { return w->t32; }
    static const float* vals(const sg_csr* A) { return A->val32.p; }
    static const float* sell_vals(const sg_csr* A) { return A->sl_val32.p; }
};
template <>
struct BBasis<double> {
    static DBuf<double>& V(BatchWork* w) { return w->V64; }
    static DBuf<double>& T(BatchWork* w) { return w->t64; }
    static const double* vals(const sg_csr* A) { return A->val.p; }
    static const double* sell_vals(const sg_csr* A) { return A->sl_val.p; }
};

template <class TV>
void apply_pc_batched(sg_ctx* ctx, sg_precond* pc, const BatchDev& B, BatchWork* w,
                      const double* r64, TV* out, bool first, const TV* tin) {
    const long long N = B.N;
    // sweep only the subdomains of instances still running
    const bool gate = pc && w->key_pc == pc && w->psys_parts == pc->nparts && pc->nparts > 1;
    if (gate) {
        const int q = pc->nparts * B.R;
        k_b_subon<<<(q + 255) / 256, 256, 0, ctx->stream>>>(B, w->psys.p, pc->nparts,
                                                            w->sub_on.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    }
    struct Reset {
        sg_precond* pc;
        ~Reset() {
            if (pc) pc->sub_on = nullptr;
        }
    } reset{pc};
    for (int rr = 0; rr < B.R; ++rr) {
        // four right-hand sides through one sweep that reads each level
        // record once for all of them (RAS with FP32 sweeps)
        if constexpr (std::is_same<TV, float>::value) {
            if (pc && rr + 4 <= B.R && pc->kind == SG_PC_RAS) {
                const int* gsw = gate ? w->sub_on.p + (size_t)rr * pc->nparts : nullptr;
                pc->sub_on = nullptr;
                const bool done4 = first ? sweep_tma4<double, float>(pc, r64 + rr * N, out + rr * N, N, gsw)
                                         : sweep_tma4<float, float>(pc, tin + rr * N, out + rr * N, N, gsw);
                if (done4) {
                    rr += 3;
                    continue;
                }
            }
        }
        if (gate) pc->sub_on = w->sub_on.p + (size_t)rr * pc->nparts;
        if (first) {
            if (pc && pc->kind != SG_PC_NONE)
                precond_apply_device<double, TV>(pc, r64 + rr * N, out + rr * N, nullptr, false);
            else
                launch_copy<double, TV>(ctx, r64 + rr * N, out + rr * N, (int)N, nullptr);
        } else {
            if (pc && pc->kind != SG_PC_NONE)
                precond_apply_device<TV, TV>(pc, tin + rr * N, out + rr * N, nullptr, false);
            else
                launch_copy<TV, TV>(ctx, tin + rr * N, out + rr * N, (int)N, nullptr);
        }
    }
}

template <class TV>
void enqueue_batch_cycle(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, const BatchDev& B,
                         BatchWork* w, int nchunks, size_t ldv) {
    cudaStream_t st = ctx->stream;
    TV* V = BBasis<TV>::V(w).p;
    TV* t = BBasis<TV>::T(w).p;
    const TV* val = BBasis<TV>::vals(A);
    const long long total = B.N * B.R;
    SG_CUDA(cudaMemsetAsync(B.notdone, 0, sizeof(int), st));
    {
        ClassTimer tm(ctx, TK_PRECOND);
        apply_pc_batched<TV>(ctx, pc, B, w, w->r64.p, V, true, nullptr);
    }
    {
        ClassTimer tm(ctx, TK_ORTHO);
        k_b_cycle_init<TV><<<nchunks, BT, 0, st>>>(B, V);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    }
    for (int j = 0; j < B.m; ++j) {
        {
            ClassTimer tm(ctx, TK_SPMV);
            const TV* sval = BBasis<TV>::sell_vals(A);
            if (A->sell_ok && sval) {
                k_b_spmv_sell<TV><<<bgrid(ctx, (long long)(B.slist ? B.nslist : A->nslices) * 32), BT, 0, st>>>(
                    B, A->sl_ptr.p, A->sl_w.p, A->sl_col.p, sval, w->row_sys.p, A->nslices,
                    V + (size_t)j * ldv, t, j);
            } else {
                k_b_spmv<TV><<<bgrid(ctx, total), BT, 0, st>>>(B, A->rp.p, A->ci.p, val,
                                                               w->row_sys.p, V + (size_t)j * ldv,
                                                               t, j);
            }
            SG_CUDA(cudaGetLastError());
            count_launch(ctx);
        }
        {
            ClassTimer tm(ctx, TK_PRECOND);
            apply_pc_batched<TV>(ctx, pc, B, w, nullptr, V + (size_t)(j + 1) * ldv, false, t);
        }
        ClassTimer tm(ctx, TK_ORTHO);
        if (B.lagged) {
            k_b_lag_a<TV><<<nchunks, BT, 0, st>>>(B, V, ldv, j);
            SG_CUDA(cudaGetLastError());
            k_b_lag_b<TV><<<nchunks, BT, 0, st>>>(B, V, ldv, j);
            SG_CUDA(cudaGetLastError());
            count_launch(ctx);
            count_launch(ctx);
            continue;
        }
        k_b_dots<TV><<<nchunks, BT, 0, st>>>(B, V, ldv, j);
        SG_CUDA(cudaGetLastError());
        k_b_upd_dots<TV><<<nchunks, BT, 0, st>>>(B, V, ldv, j);
        SG_CUDA(cudaGetLastError());
        k_b_upd_norm<TV><<<nchunks, BT, 0, st>>>(B, V, ldv, j);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        count_launch(ctx);
        count_launch(ctx);
    }
    {
        ClassTimer tm(ctx, TK_UPDATE);
        k_b_backsolve<<<(B.I + 127) / 128, 128, 0, st>>>(B);
        SG_CUDA(cudaGetLastError());
        k_b_update_x<TV><<<bgrid(ctx, total), BT, 0, st>>>(B, V, ldv, w->row_sys.p, w->x64.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        count_launch(ctx);
    }
    {
        ClassTimer tm(ctx, TK_RESIDUAL);
        k_b_residual<1><<<nchunks, BT, 0, st>>>(B, A->rp.p, A->ci.p, A->val.p, w->b64.p, w->x64.p,
                                                w->r64.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    }
    k_b_cycle_end<<<(B.I + 127) / 128, 128, 0, st>>>(B);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

}  // namespace

void solve_batched_device(sg_ctx* ctx, const sg_csr* A, sg_precond* pc, int nsys,
                          const int* sys_row_ptr, int nrhs, const double* b, double* x,
                          const sg_solve_params& prm, sg_batch_result* results, double* time_s) {
    const long long N = A->nrows;
    const int m = prm.restart;
    SG_CHECK_ARG(m >= 1 && m <= BMMAX, "batched restart must be in [1,%d] (got %d)", BMMAX, m);
    SG_CHECK_ARG(prm.max_iter >= 0, "max_iter must be >= 0");
    SG_CHECK_ARG(prm.precision == SG_FP64 || prm.precision == SG_FP32,
                 "solve precision must be SG_FP64 or SG_FP32");
    SG_CHECK_ARG(prm.tol_kind >= SG_TOL_REF_ABS && prm.tol_kind <= SG_TOL_TRUE_REL,
                 "unknown tol_kind %d", prm.tol_kind);
    SG_CHECK_ARG((long long)nrhs * N < (1ll << 31), "batch too large (nrhs * rows >= 2^31)");
    const bool fp32 = prm.precision == SG_FP32;
    const int S = nsys, R = nrhs, I = S * R;
    if (!ctx->batch) ctx->batch = new BatchWork();
    BatchWork* w = ctx->batch;
    cudaStream_t st = ctx->stream;
    const std::vector<int> rows(sys_row_ptr, sys_row_ptr + S + 1);
    const bool same_tables =
        w->key_A == A && w->key_nnz == A->nnz && w->key_nrhs == R && w->key_rows == rows;
    if (!same_tables) {
        w->key_A = nullptr;
        w->key_pc = nullptr;
        // the matrix must be block diagonal over the systems
        for (int s = 0; s < S; ++s)
            for (int i = sys_row_ptr[s]; i < sys_row_ptr[s + 1]; ++i)
                for (int q = A->h_rp[i]; q < A->h_rp[i + 1]; ++q)
                    SG_CHECK_ARG(A->h_ci[q] >= sys_row_ptr[s] && A->h_ci[q] < sys_row_ptr[s + 1],
                                 "row %d couples system %d to column %d outside it", i, s,
                                 A->h_ci[q]);
        // ---- host tables: instances and chunks
        std::vector<int> row_sys((size_t)N);
        for (int s = 0; s < S; ++s)
            for (int i = sys_row_ptr[s]; i < sys_row_ptr[s + 1]; ++i) row_sys[i] = s;
        std::vector<long long> ioff(I), coff;
        std::vector<int> in(I), ich0(I), inch(I), cinst, clen;
        for (int rr = 0; rr < R; ++rr)
            for (int s = 0; s < S; ++s) {
                const int i = rr * S + s;
                const int n = sys_row_ptr[s + 1] - sys_row_ptr[s];
                ioff[i] = (long long)rr * N + sys_row_ptr[s];
                in[i] = n;
                ich0[i] = (int)cinst.size();
                for (int q = 0; q < n; q += BCH) {
                    cinst.push_back(i);
                    coff.push_back(ioff[i] + q);
                    clen.push_back(std::min(BCH, n - q));
                }
                inch[i] = (int)cinst.size() - ich0[i];
            }
        w->ioff.upload(ioff, st);
        w->in.upload(in, st);
        w->ich0.upload(ich0, st);
        w->inch.upload(inch, st);
        w->cinst.upload(cinst, st);
        w->coff.upload(coff, st);
        w->clen.upload(clen, st);
        w->row_sys.upload(row_sys, st);
        SG_CUDA(cudaStreamSynchronize(st));
        w->nchunks = (int)cinst.size();
        w->h_ich0 = ich0;
        w->h_inch = inch;
        w->key_A = A;
        w->key_nnz = A->nnz;
        w->key_nrhs = R;
        w->key_rows = rows;
    }
    // every subdomain inside one system (checked once per set-up)
    if (pc && !(w->key_pc == pc && w->key_pc_structure == pc->structure_key) &&
        !pc->part.empty() && pc->nparts > 1) {
        w->key_pc = nullptr;
        std::vector<int> psys(pc->nparts, -1);
        for (int s = 0; s < S; ++s)
            for (int i = sys_row_ptr[s]; i < sys_row_ptr[s + 1]; ++i) {
                int& ps = psys[pc->part[i]];
                SG_CHECK_ARG(ps < 0 || ps == s, "subdomain %d spans systems %d and %d",
                             pc->part[i], ps, s);
                ps = s;
            }
        w->psys.upload(psys, st);
        w->psys_parts = pc->nparts;
        w->key_pc = pc;
        w->key_pc_structure = pc->structure_key;
    }
    if (pc && w->key_pc == pc) dalloc(w->sub_on, (size_t)pc->nparts * R);
    const int nchunks = w->nchunks;
    const size_t ld = (size_t)m + 1;
    for (DBuf<int>* p : {&w->active, &w->done, &w->conv, &w->iters, &w->cycles, &w->kcount,
                         &w->ran, &w->flags}) {
        dalloc(*p, (size_t)I);
        p->zero(st);
    }
    dalloc(w->notdone, 1);
    for (DBuf<double>* p : {&w->bnorm, &w->rnorm, &w->est, &w->lastres}) dalloc(*p, (size_t)I);
    dalloc(w->g, I * ld);
    dalloc(w->cs, (size_t)I * m);
    dalloc(w->sn, (size_t)I * m);
    dalloc(w->H, I * ld * m);
    dalloc(w->vscale, I * ld);
    dalloc(w->y, (size_t)I * m);
    dalloc(w->yd, (size_t)I * m);
    dalloc(w->yf, (size_t)I * m);
    dalloc(w->h, I * ld);
    dalloc(w->hs, I * ld);
    dalloc(w->part, (size_t)nchunks * BLD);
    const bool lagged = prm.ortho == 0 && m < SG_LAGM;
    if (lagged) {
        dalloc(w->lagT, (size_t)I * BLD * BLD);
        dalloc(w->lagH, (size_t)I * BLD * BMMAX);
        dalloc(w->lagc, (size_t)I * BLD);
        dalloc(w->cfu, (size_t)I * BLD);
    }
    dalloc(w->ticket, (size_t)I);
    w->ticket.zero(st);
    const size_t tot = (size_t)N * R;
    const size_t ldv = ((tot + 31) & ~(size_t)31) + 32;
    dalloc(w->r64, tot);
    if (fp32) {
        const_cast<sg_csr*>(A)->ensure_fp32();
        if (w->V32.n < ldv * (m + 1)) {
            w->V32.alloc(ldv * (m + 1));
            w->V32.zero(st);
        }
        if (w->t32.n < ldv) {
            w->t32.alloc(ldv);
            w->t32.zero(st);
        }
    } else {
        if (w->V64.n < ldv * (m + 1)) {
            w->V64.alloc(ldv * (m + 1));
            w->V64.zero(st);
        }
        if (w->t64.n < ldv) {
            w->t64.alloc(ldv);
            w->t64.zero(st);
        }
    }
    if (!w->h_notdone) SG_CUDA(cudaMallocHost(reinterpret_cast<void**>(&w->h_notdone), sizeof(int)));
    BatchDev B{};
    B.ioff = w->ioff.p; B.in = w->in.p; B.ich0 = w->ich0.p; B.inch = w->inch.p;
    B.cinst = w->cinst.p; B.coff = w->coff.p; B.clen = w->clen.p;
    B.active = w->active.p; B.done = w->done.p; B.conv = w->conv.p; B.iters = w->iters.p;
    B.cycles = w->cycles.p; B.kcount = w->kcount.p; B.ran = w->ran.p; B.flags = w->flags.p;
    B.bnorm = w->bnorm.p; B.rnorm = w->rnorm.p; B.est = w->est.p; B.lastres = w->lastres.p;
    B.g = w->g.p; B.cs = w->cs.p; B.sn = w->sn.p; B.H = w->H.p; B.vscale = w->vscale.p;
    B.y = w->y.p; B.yd = w->yd.p; B.yf = w->yf.p; B.h = w->h.p; B.hs = w->hs.p; B.ticket = w->ticket.p; B.part = w->part.p;
    B.notdone = w->notdone.p;
    B.lagT = w->lagT.p; B.lagH = w->lagH.p; B.lagc = w->lagc.p; B.cfu = w->cfu.p;
    B.lagged = lagged ? 1 : 0;
    B.clist = nullptr;
    B.slist = nullptr;
    B.nslist = 0;
    B.m = m; B.I = I; B.S = S; B.R = R; B.N = N;
    B.tol = prm.tol; B.tol_kind = prm.tol_kind; B.max_iter = prm.max_iter;
    // four right-hand sides per sweep: planned once per set-up, before any capture
    if (fp32 && pc && R >= 4) sweep_plan4(pc);
    const auto t0 = std::chrono::high_resolution_clock::now();
    // b and x (device copies in the batch layout)
    if (w->b64.n < tot) w->b64.alloc(tot);
    if (w->x64.n < tot) w->x64.alloc(tot);
    SG_CUDA(cudaMemcpyAsync(w->b64.p, b, sizeof(double) * tot, cudaMemcpyDefault, st));
    SG_CUDA(cudaMemcpyAsync(w->x64.p, x, sizeof(double) * tot, cudaMemcpyDefault, st));
    k_b_residual<0><<<nchunks, BT, 0, st>>>(B, A->rp.p, A->ci.p, A->val.p, w->b64.p, w->x64.p,
                                            w->r64.p);
    SG_CUDA(cudaGetLastError());
    k_b_residual<1><<<nchunks, BT, 0, st>>>(B, A->rp.p, A->ci.p, A->val.p, w->b64.p, w->x64.p,
                                            w->r64.p);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
    count_launch(ctx);
    const bool use_graph = prm.use_graph != 0 && prm.max_iter > 0;
    cudaGraphExec_t exec = nullptr;
    // The cycle's launches cover `covered` instances: all at first; once at
    // most a quarter of them are still running, the chunk kernels are launched
    // over the chunks of the running instances only and the SELL SpMV over
    // their systems' slices (each block still takes one chunk, so the
    // reductions and their order are unchanged), and the graph is captured
    // again for the new grids.  Instances only ever finish, so a list stays
    // a superset of the running instances until the next rebuild.
    BatchDev Bc = B;
    int ncl = nchunks, covered = I;
    auto rebuild = [&](int left) {
        std::vector<int> done(I);
        SG_CUDA(cudaMemcpyAsync(done.data(), w->done.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
        SG_CUDA(cudaStreamSynchronize(st));
        std::vector<int> cl;
        std::vector<char> mark(A->sell_ok ? A->nslices : 0, 0);
        for (int i = 0; i < I; ++i) {
            if (done[i]) continue;
            for (int c = w->h_ich0[i]; c < w->h_ich0[i] + w->h_inch[i]; ++c) cl.push_back(c);
            const int sy = i % S;
            if (A->sell_ok && rows[sy + 1] > rows[sy])
                for (int q = rows[sy] / 32; q <= (rows[sy + 1] - 1) / 32; ++q) mark[q] = 1;
        }
        std::vector<int> sl;
        for (int q = 0; q < (int)mark.size(); ++q)
            if (mark[q]) sl.push_back(q);
        if (cl.empty()) return;
        dalloc(w->clist, cl.size());
        w->clist.upload(cl, st);
        Bc.clist = w->clist.p;
        if (!sl.empty()) {
            dalloc(w->slist, sl.size());
            w->slist.upload(sl, st);
            Bc.slist = w->slist.p;
            Bc.nslist = (int)sl.size();
        }
        SG_CUDA(cudaStreamSynchronize(st));
        ncl = (int)cl.size();
        covered = left;
    };
    auto capture = [&]() {
        if (exec) {
            cudaGraphExecDestroy(exec);
            exec = nullptr;
        }
        cudaGraph_t gph = nullptr;
        SG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed));
        ctx->capturing = true;
        ctx->captured = 0;
        try {
            if (fp32) enqueue_batch_cycle<float>(ctx, A, pc, Bc, w, ncl, ldv);
            else enqueue_batch_cycle<double>(ctx, A, pc, Bc, w, ncl, ldv);
        } catch (...) {
            ctx->capturing = false;
            cudaStreamEndCapture(st, &gph);
            if (gph) cudaGraphDestroy(gph);
            throw;
        }
        ctx->capturing = false;
        SG_CUDA(cudaStreamEndCapture(st, &gph));
        const cudaError_t e = cudaGraphInstantiate(&exec, gph, 0);
        cudaGraphDestroy(gph);
        SG_CUDA(e);
    };
    const int max_cycles = prm.max_iter > 0 ? (prm.max_iter + m - 1) / m + 1 : 0;
    try {
        if (use_graph) capture();
        for (int cyc = 0; cyc < max_cycles; ++cyc) {
            if (use_graph) {
                SG_CUDA(cudaGraphLaunch(exec, st));
                ctx->launches += ctx->captured;
            } else if (fp32) {
                enqueue_batch_cycle<float>(ctx, A, pc, Bc, w, ncl, ldv);
            } else {
                enqueue_batch_cycle<double>(ctx, A, pc, Bc, w, ncl, ldv);
            }
            SG_CUDA(cudaMemcpyAsync(w->h_notdone, w->notdone.p, sizeof(int),
                                    cudaMemcpyDeviceToHost, st));
            SG_CUDA(cudaStreamSynchronize(st));
            if (ctx->timing) collect_timers(ctx);
            const int left = *w->h_notdone;
            if (left == 0) break;
            if (4 * left <= covered && cyc + 1 < max_cycles) {
                rebuild(left);
                if (use_graph) capture();
            }
        }
    } catch (...) {
        if (exec) cudaGraphExecDestroy(exec);
        throw;
    }
    if (exec) cudaGraphExecDestroy(exec);
    SG_CUDA(cudaMemcpyAsync(x, w->x64.p, sizeof(double) * tot, cudaMemcpyDefault, st));
    std::vector<int> h_iters(I), h_cycles(I), h_conv(I), h_flags(I);
    std::vector<double> h_rn(I), h_bn(I);
    SG_CUDA(cudaMemcpyAsync(h_iters.data(), w->iters.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaMemcpyAsync(h_cycles.data(), w->cycles.p, sizeof(int) * I, cudaMemcpyDeviceToHost,
                            st));
    SG_CUDA(cudaMemcpyAsync(h_conv.data(), w->conv.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaMemcpyAsync(h_flags.data(), w->flags.p, sizeof(int) * I, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaMemcpyAsync(h_rn.data(), w->rnorm.p, sizeof(double) * I, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaMemcpyAsync(h_bn.data(), w->bnorm.p, sizeof(double) * I, cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    const auto t1 = std::chrono::high_resolution_clock::now();
    if (time_s) *time_s = std::chrono::duration<double>(t1 - t0).count();
    bool nonfinite = false;
    for (int i = 0; i < I; ++i) {
        if (h_flags[i] & 1) nonfinite = true;
        if (!results) continue;
        results[i].iterations = h_iters[i];
        results[i].cycles = h_cycles[i];
        results[i].converged = h_conv[i];
        results[i].status = (h_flags[i] & 1) ? SG_ERR_NONFINITE : SG_OK;
        results[i].true_rel_residual = h_bn[i] > 0 ? h_rn[i] / h_bn[i] : h_rn[i];
    }
    if (pc && sweep_error(pc))
        fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
    if (nonfinite)
        fail(SG_ERR_NONFINITE, "non-finite value in a right-hand side or iteration of the batch");
}

}  // namespace sg
