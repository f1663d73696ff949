// krylov.cu -- Arnoldi / least-squares kernels of restarted GMRES(m) and
// FGMRES (src/core/gmres.cpp:34-160, src/core/fgmres.cpp:28-144; replaces the
// host-driven cuBLAS loop of src/gpu/gmres_gpu.cu:10-138).
//
// Basis storage: raw_k (k <= m) are the columns of a (m+1) x ldv array; the
// orthonormal vector is v_k = vscale[k] * raw_k, so a new vector never needs
// a separate normalisation pass.
//
// One Arnoldi step orthogonalises w = raw_{j+1} against raw_0..raw_j by
// classical Gram-Schmidt applied twice (CGS2), in three streaming passes:
//   A  h1 = V^T w                          (dot products, one pass)
//   B  w' = w - V h1 ; h2 = V^T w'          (update and second dots, one pass)
//   C  w'' = w' - V h2 ; ||w''||           (update and norm, one pass)
// Every pass reduces per block, and the last block to finish sums the block
// partials in block order; after pass C it also writes the Hessenberg column,
// applies the Givens rotations (same formulas as src/core/gmres.cpp:9-30)
// and tests convergence, so no value travels to the host inside a cycle.
#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int KT = 256;    // threads of the Krylov kernels
constexpr int BS_T = 256;  // threads of the back substitution (loads; one warp solves)

// Givens rotation of src/core/gmres.cpp:9-30
__device__ void rot_compute(double& c, double& s, double a, double b) {
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
__device__ void rot_apply(double c, double s, double& h1, double& h2) {
    const double t1 = c * h1 - s * h2;
    const double t2 = s * h1 + c * h2;
    h1 = t1;
    h2 = t2;
}

// State the serial end of an Arnoldi step reads, brought to shared memory
// (and, for thread 0, registers) in one round of loads: the column h(0..j),
// the earlier rotations, g(j..j+1) and the stopping-test scalars.
struct FinalizeIn {
    double hc[SG_MMAX + 2], csv[SG_MMAX], snv[SG_MMAX], gv[2];
    double tol, bnorm, est_scale;
    int tol_kind, hist_len, total_iter;
};

// all threads of the block: loads everything but hc (the caller's column)
__device__ __forceinline__ void finalize_load(FinalizeIn& f, const SolveState* st, int j) {
    for (int i = threadIdx.x; i < j; i += blockDim.x) {
        f.csv[i] = st->cs[i];
        f.snv[i] = st->sn[i];
    }
    if (threadIdx.x == 0) {
        f.gv[0] = st->g[j];
        f.gv[1] = st->g[j + 1];
        f.tol = st->tol;
        f.bnorm = st->bnorm;
        f.est_scale = st->est_scale;
        f.tol_kind = st->tol_kind;
        f.hist_len = st->hist_len;
        f.total_iter = st->total_iter;
    }
}

// Thread 0: completes Arnoldi step j from f (hc[0..j] holds the column) and
// ss = ||w''||^2: normalisation, Givens rotations, residual estimate and
// stopping test.  Returns the new vector's scale 1/||w''|| when the cycle
// goes on, 0 when it stops here (breakdown, convergence, last step).
__device__ double finalize_core(SolveState* st, FinalizeIn& f, int j, int m, double ss,
                                double* hist, int hist_cap) {
    const int ld = m + 1;
    double* hc = f.hc;
    const double nrm = sqrt(ss);
    double* Hc = st->H + (size_t)j * ld;
    hc[j + 1] = nrm;
    if (!(nrm >= 1e-30)) {
        // breakdown (src/core/gmres.cpp:297-300): this column is used as is
        for (int i = 0; i <= j + 1; ++i) Hc[i] = hc[i];
        if (!isfinite(nrm)) {
            st->nonfinite = 1;
            st->done = 1;
        }
        st->breakdown = 1;
        st->kcount = j + 1;
        st->cycle_active = 0;
        return 0.0;
    }
    const double vs = 1.0 / nrm;
    st->vscale[j + 1] = vs;
    for (int i = 0; i < j; ++i) rot_apply(f.csv[i], f.snv[i], hc[i], hc[i + 1]);
    double c, sn;
    rot_compute(c, sn, hc[j], hc[j + 1]);
    rot_apply(c, sn, hc[j], hc[j + 1]);
    rot_apply(c, sn, f.gv[0], f.gv[1]);
    st->cs[j] = c;
    st->sn[j] = sn;
    st->g[j] = f.gv[0];
    st->g[j + 1] = f.gv[1];
    for (int i = 0; i <= j + 1; ++i) Hc[i] = hc[i];
    const double res = fabs(f.gv[1]);
    if (hist && f.hist_len < hist_cap) hist[f.hist_len] = res;
    st->hist_len = f.hist_len + 1;
    st->last_res = res;
    st->total_iter = f.total_iter + 1;
    st->kcount = j + 1;
    st->j = j + 1;
    bool stop = false;
    if (f.tol_kind == SG_TOL_REF_ABS) {
        if (res < f.tol) {
            st->converged = 1;
            st->done = 1;
            stop = true;
        }
    } else if (f.tol_kind == SG_TOL_TRUE_REL) {
        // estimated true residual; the restart verifies it in FP64
        if (res * f.est_scale <= 0.5 * f.tol * f.bnorm) stop = true;
    }
    if (!isfinite(res)) {
        st->nonfinite = 1;
        st->done = 1;
        stop = true;
    }
    if (j + 1 >= m) stop = true;
    if (stop) {
        st->cycle_active = 0;
        return 0.0;
    }
    return vs;
}

// Completes Arnoldi step j once ||w''||^2 is known (all threads of the last
// block; the column is hsum(0..j)).
__device__ void arnoldi_finalize(SolveState* st, int j, int m, double ss, double* hist,
                                 int hist_cap) {
    __shared__ FinalizeIn f;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) f.hc[i] = st->hsum[i];
    finalize_load(f, st, j);
    __syncthreads();
    if (threadIdx.x == 0) finalize_core(st, f, j, m, ss, hist, hist_cap);
}

template <class T>
struct Vec;
template <>
struct Vec<double> {
    static constexpr int N = 2;
    using V = double2;
};
template <>
struct Vec<float> {
    static constexpr int N = 4;
    using V = float4;
};

template <class T>
__device__ __forceinline__ void vload(const T* p, T (&o)[Vec<T>::N]);
template <>
__device__ __forceinline__ void vload<double>(const double* p, double (&o)[2]) {
    const double2 v = ld_stream(reinterpret_cast<const double2*>(p));
    o[0] = v.x; o[1] = v.y;
}
template <>
__device__ __forceinline__ void vload<float>(const float* p, float (&o)[4]) {
    const float4 v = ld_stream(reinterpret_cast<const float4*>(p));
    o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
}
template <class T>
__device__ __forceinline__ void vstore(T* p, const T (&o)[Vec<T>::N]);
template <>
__device__ __forceinline__ void vstore<double>(double* p, const double (&o)[2]) {
    *reinterpret_cast<double2*>(p) = make_double2(o[0], o[1]);
}
template <>
__device__ __forceinline__ void vstore<float>(float* p, const float (&o)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(o[0], o[1], o[2], o[3]);
}

// ---- pass A (and generic second dots): s_k = raw_{k0+k} . w for k < kc.
// A row tile is 32 lanes x one 16-byte vector of elements.  The kc <= 32
// vectors of a launch are spread over a group of nwg warps that share a tile
// (vector k is held by warp k % nwg of the group, so a thread keeps at most 4
// accumulators); the block's 8 / nwg groups walk different tiles, so a step
// with few vectors still keeps every warp loading.
constexpr int KW = KT / 32;  // warps per block
constexpr int KPW = 4;       // basis vectors per warp

// warps per tile group: the fewest that hold kc vectors at KPW per warp
__device__ __forceinline__ int warps_per_tile(int kc) {
    return kc <= KPW ? 1 : (kc <= 2 * KPW ? 2 : (kc <= 4 * KPW ? 4 : 8));
}

template <class TV>
__device__ __forceinline__ TV dotv(const TV (&a)[Vec<TV>::N], const TV (&b)[Vec<TV>::N]) {
    TV s = (TV)0;
#pragma unroll
    for (int e = 0; e < Vec<TV>::N; ++e) s += a[e] * b[e];
    return s;
}

// per-warp accumulators -> block sums bs[k] (k < kc): the warp trees run in
// the basis precision, the groups' sums of vector k are added in FP64 in
// group order (fixed: deterministic)
template <class TV>
__device__ __forceinline__ void group_sums(const TV (&acc)[KPW], int kc, int nwg, double* bs) {
    __shared__ double red[KW][KPW];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int q = 0; q < KPW; ++q) {
        const double v = (double)warp_sum(acc[q]);
        if (lane == 0) red[warp][q] = v;
    }
    __syncthreads();
    if ((int)threadIdx.x < kc) {
        const int k = threadIdx.x, slot = k % nwg, q = k / nwg;
        double v = red[slot][q];
        for (int g = 1; g < KW / nwg; ++g) v += red[g * nwg + slot][q];
        bs[k] = v;
    }
    __syncthreads();
}

// barrier among the nwg >= 2 warps of tile group grp < 4 (named barrier
// 1 + grp; immediate ids keep the block's barrier count at five)
__device__ __forceinline__ void group_sync(int grp, int nwg) {
    const int cnt = nwg * 32;
    switch (grp) {
    case 0: asm volatile("bar.sync 1, %0;" ::"r"(cnt) : "memory"); break;
    case 1: asm volatile("bar.sync 2, %0;" ::"r"(cnt) : "memory"); break;
    case 2: asm volatile("bar.sync 3, %0;" ::"r"(cnt) : "memory"); break;
    default: asm volatile("bar.sync 4, %0;" ::"r"(cnt) : "memory"); break;
    }
}

// ---- lagged CGS2 (left-preconditioned GMRES, FP32 or FP64 basis, restart < SG_LAGM).
// Step j orthogonalises z = B (vscale_j raw_j), where the stored raw_j still
// lacks its second projection: v_j = T(j,j) raw_j - sum_{k<j} c_k v_k.  By
// linearity B v_j = z - V_j g with g = H(0..j, 0..j-1) c (the Arnoldi relation
// B v_k = V H(:,k)), so the projections of z give the Hessenberg column after
// subtracting g, and the orthogonalised vector is the same.  Two passes:
//   A  d = S^T z over the stored vectors; p = T^T d; hsum = p - g;
//      update coefficients on the stored vectors u = T p
//   B  w' = z - S u; r = S^T w'; ||w'||^2; then h2 = T^T r, the column is
//      hsum + h2, ||w''||^2 = ||w'||^2 - ||h2||^2 (Pythagoras), and w' is
//      stored as raw_{j+1} with its pending correction c = h2 / ||w''||.
// In exact arithmetic this is CGS2; the stored vectors are never rewritten.

// the leading n x n block of the column-major SG_LAGM matrix M into
// shared memory (upper triangle only when `upper`)
__device__ __forceinline__ void stage_lag(double (*dst)[SG_LAGM + 1], const double* M, int n,
                                          int ncol, bool upper) {
    for (int idx = threadIdx.x; idx < n * ncol; idx += blockDim.x) {
        const int i = idx % n, k = idx / n;
        dst[i][k] = (!upper || i <= k) ? M[i + k * SG_LAGM] : 0.0;
    }
}

// what the pass A epilogue reads from the state (T, the lagged Hessenberg
// block, the pending correction), loaded by the last block with its partials
struct LagAIn {
    double Ts[SG_LAGM][SG_LAGM + 1], Hs[SG_LAGM][SG_LAGM + 1];
    double cs[SG_LAGM];
};
__device__ __forceinline__ void lagged_a_load(LagAIn& in, const SolveState* st, int j) {
    const int n1 = j + 1;
    stage_lag(in.Ts, st->lagT, n1, n1, true);
    stage_lag(in.Hs, st->lagH, n1, j, false);
    for (int i = threadIdx.x; i < j; i += blockDim.x) in.cs[i] = st->lagc[i];
}

// pass A epilogue (all threads of the last block; d = tot[0..j], `in` loaded
// and visible): p = T^T d, hsum = p - g, update coefficients u = T p
__device__ void lagged_pass_a(SolveState* st, int j, const double* d, const LagAIn& in) {
    __shared__ double p_s[SG_LAGM];
    const auto& Ts = in.Ts;
    const auto& Hs = in.Hs;
    const double* cs = in.cs;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double s = 0.0;
        for (int l = 0; l <= i; ++l) s += Ts[l][i] * d[l];
        p_s[i] = s;
    }
    __syncthreads();
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double g = 0.0;
        for (int k = (i > 0 ? i - 1 : 0); k < j; ++k) g += Hs[i][k] * cs[k];
        st->h[i] = p_s[i];
        st->hsum[i] = p_s[i] - g;
        double u = 0.0;
        for (int k = i; k <= j; ++k) u += Ts[i][k] * p_s[k];
        st->cfu[i] = u;
    }
    __syncthreads();
}

// pass B epilogue (all threads of the last block; r = tot[0..j], ss =
// ||w'||^2).  Everything it reads from the state (T, the column's pass A
// part, the rotations, g, the stopping-test scalars) is loaded by
// lagged_b_load with the partials; the step's end runs on thread 0 from
// shared memory.
struct LagBIn {
    double Ts[SG_LAGM][SG_LAGM + 1];
    FinalizeIn f;
};
__device__ __forceinline__ void lagged_b_load(LagBIn& in, const SolveState* st, int j) {
    const int n1 = j + 1;
    stage_lag(in.Ts, st->lagT, n1, n1, true);
    for (int i = threadIdx.x; i <= j; i += blockDim.x) in.f.hc[i] = st->hsum[i];
    finalize_load(in.f, st, j);
}

__device__ void lagged_pass_b(SolveState* st, int j, int m, const double* r, double ss,
                              double* hist, int hist_cap, LagBIn& in) {
    __shared__ double h2_s[SG_LAGM], c_s[SG_LAGM];
    __shared__ double s_vs;
    const auto& Ts = in.Ts;
    FinalizeIn& f = in.f;
    for (int i = threadIdx.x; i <= j; i += blockDim.x) {
        double s = 0.0;
        for (int l = 0; l <= i; ++l) s += Ts[l][i] * r[l];
        h2_s[i] = s;
        const double hs = f.hc[i] + s;  // the Hessenberg column
        f.hc[i] = hs;
        st->hsum[i] = hs;
        st->lagH[i + j * SG_LAGM] = hs;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        double nrm2 = ss;
        for (int i = 0; i <= j; ++i) nrm2 -= h2_s[i] * h2_s[i];
        if (!(nrm2 > 0.0)) nrm2 = isfinite(nrm2) ? 0.0 : nrm2;
        st->lagH[j + 1 + j * SG_LAGM] = sqrt(nrm2);
        const double vs = finalize_core(st, f, j, m, nrm2, hist, hist_cap);
        s_vs = j + 1 < SG_LAGM ? vs : 0.0;
    }
    __syncthreads();
    // the pending correction of the new stored vector
    const double vs = s_vs;
    if (vs == 0.0) return;
    for (int k = threadIdx.x; k <= j; k += blockDim.x) {
        c_s[k] = h2_s[k] * vs;
        st->lagc[k] = c_s[k];
    }
    if (threadIdx.x == 0) st->lagT[(j + 1) + (j + 1) * SG_LAGM] = vs;
    __syncthreads();
    // T(:, j+1) = T(j+1,j+1) e_{j+1} - T(:, 0..j) c
    for (int l = threadIdx.x; l <= j; l += blockDim.x) {
        double s = 0.0;
        for (int k = l; k <= j; ++k) s += Ts[l][k] * c_s[k];
        st->lagT[l + (j + 1) * SG_LAGM] = -s;
    }
}

template <class TV>
__global__ void __launch_bounds__(KT)
k_dots(const TV* __restrict__ raw, size_t ldv, int n, int k0, int kc, const TV* __restrict__ w,
       SolveState* st, int second, int lagged, double* partials, unsigned* counter) {
    if (!st->cycle_active) return;
    constexpr int VN = Vec<TV>::N;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwg = warps_per_tile(kc), ngrp = KW / nwg;
    const int grp = warp / nwg, slot = warp % nwg;
    TV acc[KPW];
#pragma unroll
    for (int q = 0; q < KPW; ++q) acc[q] = (TV)0;
    const int nvec = n / VN;
    const int stride = gridDim.x * ngrp * 32;
    // two tiles per round: all their loads are in flight before the first
    // product (a step with few vectors has only a few rounds per thread, each
    // a full memory latency); the tiles are still added in ascending order
    int u = (blockIdx.x * ngrp + grp) * 32 + lane;
    for (; u + stride < nvec; u += 2 * stride) {
        TV w0[VN], w1[VN], v0[KPW][VN], v1[KPW][VN];
        vload<TV>(w + (size_t)u * VN, w0);
        vload<TV>(w + (size_t)(u + stride) * VN, w1);
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = slot + nwg * q;
            if (k < kc) {
                vload<TV>(raw + (size_t)(k0 + k) * ldv + (size_t)u * VN, v0[q]);
                vload<TV>(raw + (size_t)(k0 + k) * ldv + (size_t)(u + stride) * VN, v1[q]);
            }
        }
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = slot + nwg * q;
            if (k < kc) {
                acc[q] += dotv<TV>(v0[q], w0);
                acc[q] += dotv<TV>(v1[q], w1);
            }
        }
    }
    if (u < nvec) {
        TV wv[VN];
        vload<TV>(w + (size_t)u * VN, wv);
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = slot + nwg * q;
            if (k < kc) {
                TV vv[VN];
                vload<TV>(raw + (size_t)(k0 + k) * ldv + (size_t)u * VN, vv);
                acc[q] += dotv<TV>(vv, wv);
            }
        }
    }
    if (blockIdx.x == 0 && grp == 0) {  // elements past the last full vector
        const int i = nvec * VN + lane;
        if (lane < n - nvec * VN) {
#pragma unroll
            for (int q = 0; q < KPW; ++q) {
                const int k = slot + nwg * q;
                if (k < kc) acc[q] += raw[(size_t)(k0 + k) * ldv + i] * w[i];
            }
        }
    }
    __shared__ double bs[KW * KPW], tot[KW * KPW];
    __shared__ LagAIn lag_in;
    group_sums<TV>(acc, kc, nwg, bs);
    if (last_block_reduce(partials, counter, bs, kc, tot, [&] {
            if (lagged) lagged_a_load(lag_in, st, kc - 1);
        })) {
        if (lagged) {
            lagged_pass_a(st, kc - 1, tot, lag_in);
            return;
        }
        for (int k = threadIdx.x; k < kc; k += blockDim.x) {
            const double h = st->vscale[k0 + k] * tot[k];
            st->h[k0 + k] = h;
            st->hsum[k0 + k] = second ? st->hsum[k0 + k] + h : h;
        }
    }
}

// ---- pass B fused (nk <= 32): w' = w - sum_k c_k raw_k ; s2_k = raw_k . w'.
// Each warp of a tile group forms the update of its own vectors for the
// tile.  A one-warp group holds every vector: w' = w - share directly.  In a
// larger group the shares meet in shared memory, the group's threads each
// form w' = w - (sum of the shares, in warp order) for some elements of the
// tile (and store them), and every warp dots w' with the vector values it
// still holds.
template <class TV>
__global__ void __launch_bounds__(KT)
k_upd_dots(const TV* __restrict__ raw, size_t ldv, int n, int nk, TV* __restrict__ w,
           SolveState* st, double* partials, unsigned* counter, int lagged, int m,
           double* hist, int hist_cap) {
    if (!st->cycle_active) return;
    constexpr int VN = Vec<TV>::N;
    constexpr int TE = 32 * VN;  // elements of a tile
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nwg = warps_per_tile(nk), ngrp = KW / nwg;
    const int grp = warp / nwg, slot = warp % nwg;
    const int gsz = nwg * 32, gt = slot * 32 + lane;  // threads of the group, rank
    __shared__ TV cf[KW * KPW];
    __shared__ TV upd[KW][TE];
    __shared__ TV wsh[KW / 2][TE];
    for (int k = threadIdx.x; k < nk; k += blockDim.x)
        cf[k] = lagged ? (TV)st->cfu[k] : (TV)(st->h[k] * st->vscale[k]);
    __syncthreads();
    TV ss = (TV)0;  // ||w'||^2 (lagged): slot 0 of each group counts its elements
    TV acc[KPW];
#pragma unroll
    for (int q = 0; q < KPW; ++q) acc[q] = (TV)0;
    const int nvec = n / VN;
    const int ntiles = (nvec + 31) / 32;
    const int nfull = nvec * VN;  // elements covered by whole vectors
    // registers of the current tile and of the next one (loaded ahead): the
    // warp's vector values, and the w elements this thread turns into w'
    // (its lanes' elements in a one-warp group; else elements gt + r * gsz)
    TV vv[KPW][VN], nv[KPW][VN], we[VN], nwe[VN];
    // tiles are walked in reverse: pass A (k_dots) has just streamed the
    // basis in ascending order, so its last tiles are still in L2
    auto load_tile = [&](int tile_l, TV (&v)[KPW][VN], TV (&wl)[VN]) {
        const int tile = ntiles - 1 - tile_l;
        const int u = tile * 32 + lane;
        const bool ok = u < nvec;
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = slot + nwg * q;
            if (k < nk && ok) {
                vload<TV>(raw + (size_t)k * ldv + (size_t)u * VN, v[q]);
            } else {
#pragma unroll
                for (int e = 0; e < VN; ++e) v[q][e] = (TV)0;
            }
        }
        if (nwg == 1) {
            if (ok) {
                vload<TV>(w + (size_t)u * VN, wl);
            } else {
#pragma unroll
                for (int e = 0; e < VN; ++e) wl[e] = (TV)0;
            }
        } else {
#pragma unroll
            for (int r = 0; r < VN; ++r) {
                const int t = gt + r * gsz, i = tile * TE + t;
                wl[r] = (t < TE && i < nfull) ? w[i] : (TV)0;
            }
        }
    };
    const int gstride = gridDim.x * ngrp;
    int tile = blockIdx.x * ngrp + grp;
    if (tile < ntiles) load_tile(tile, vv, we);
    for (; tile < ntiles; tile += gstride) {
        const int next = tile + gstride;
        if (next < ntiles) load_tile(next, nv, nwe);
        // this warp's share of the update for its lanes' elements
        TV part[VN];
#pragma unroll
        for (int e = 0; e < VN; ++e) part[e] = (TV)0;
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            const int k = slot + nwg * q;
            if (k < nk) {
#pragma unroll
                for (int e = 0; e < VN; ++e) part[e] += cf[k] * vv[q][e];
            }
        }
        TV wn[VN];
        const int ptile = ntiles - 1 - tile;  // the physical tile
        if (nwg == 1) {
#pragma unroll
            for (int e = 0; e < VN; ++e) wn[e] = we[e] - ((TV)0 + part[e]);
            const int u = ptile * 32 + lane;
            if (u < nvec) vstore<TV>(w + (size_t)u * VN, wn);
#pragma unroll
            for (int e = 0; e < VN; ++e) ss += wn[e] * wn[e];
        } else {
#pragma unroll
            for (int e = 0; e < VN; ++e) upd[warp][lane * VN + e] = part[e];
            group_sync(grp, nwg);
            // w' = w - (sum of the shares, in warp order), once per element
#pragma unroll
            for (int r = 0; r < VN; ++r) {
                const int t = gt + r * gsz;
                if (t < TE) {
                    TV sum = (TV)0;
                    for (int g = 0; g < nwg; ++g) sum += upd[grp * nwg + g][t];
                    const TV x = we[r] - sum;
                    wsh[grp][t] = x;
                    const int i = ptile * TE + t;
                    if (i < nfull) w[i] = x;
                }
            }
            group_sync(grp, nwg);
#pragma unroll
            for (int e = 0; e < VN; ++e) wn[e] = wsh[grp][lane * VN + e];
            if (slot == 0) {
#pragma unroll
                for (int e = 0; e < VN; ++e) ss += wn[e] * wn[e];
            }
        }
#pragma unroll
        for (int q = 0; q < KPW; ++q) {
            TV d = (TV)0;
#pragma unroll
            for (int e = 0; e < VN; ++e) d += vv[q][e] * wn[e];
            acc[q] += d;
        }
#pragma unroll
        for (int q = 0; q < KPW; ++q)
#pragma unroll
            for (int e = 0; e < VN; ++e) vv[q][e] = nv[q][e];
#pragma unroll
        for (int e = 0; e < VN; ++e) we[e] = nwe[e];
    }
    if (blockIdx.x == 0 && warp == 0) {  // tail elements: one warp, serial over k
        const int i = nfull + lane;
        if (lane < n - nfull) {
            TV wi = w[i];
            for (int k = 0; k < nk; ++k) wi -= cf[k] * raw[(size_t)k * ldv + i];
            w[i] = wi;
            ss += wi * wi;
        }
    }
    __syncthreads();
    if (blockIdx.x == 0 && grp == 0) {
        const int i = nfull + lane;
        if (lane < n - nfull) {
#pragma unroll
            for (int q = 0; q < KPW; ++q) {
                const int k = slot + nwg * q;
                if (k < nk) acc[q] += raw[(size_t)k * ldv + i] * w[i];
            }
        }
    }
    __shared__ double bs[KW * KPW + 1], tot[KW * KPW + 1];
    group_sums<TV>(acc, nk, nwg, bs);
    if (lagged) {
        // block sum of ||w'||^2 next to the dots
        __shared__ double red_ss[KW];
        const double v = (double)warp_sum(ss);
        if (lane == 0) red_ss[warp] = v;
        __syncthreads();
        if (threadIdx.x == 0) {
            double t = red_ss[0];
            for (int g = 1; g < KW; ++g) t += red_ss[g];
            bs[nk] = t;
        }
        __syncthreads();
        __shared__ LagBIn lag_in;
        if (last_block_reduce(partials, counter, bs, nk + 1, tot,
                              [&] { lagged_b_load(lag_in, st, nk - 1); }))
            lagged_pass_b(st, nk - 1, m, tot, tot[nk], hist, hist_cap, lag_in);
        return;
    }
    if (last_block_reduce(partials, counter, bs, nk, tot)) {
        for (int k = threadIdx.x; k < nk; k += blockDim.x) {
            const double h = st->vscale[k] * tot[k];
            st->h[k] = h;
            st->hsum[k] += h;
        }
    }
}

// ---- generic update: w -= sum_k c_k raw_k (any nk)
template <class TV>
__global__ void __launch_bounds__(KT)
k_upd(const TV* __restrict__ raw, size_t ldv, int n, int nk, TV* __restrict__ w,
      SolveState* st) {
    if (!st->cycle_active) return;
    __shared__ TV cf[SG_MMAX + 1];
    for (int k = threadIdx.x; k < nk; k += blockDim.x) cf[k] = (TV)(st->h[k] * st->vscale[k]);
    __syncthreads();
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        TV wi = w[i];
        for (int k = 0; k < nk; ++k) wi -= cf[k] * raw[(size_t)k * ldv + i];
        w[i] = wi;
    }
}

// ---- pass C: w'' = w' - sum c_k raw_k ; ||w''||^2 -> Arnoldi finalize.
// 16-byte vectors of elements per thread, the k loop unrolled by 4 so four
// basis loads are in flight per thread.
template <class TV>
__global__ void __launch_bounds__(KT)
k_upd_norm(const TV* __restrict__ raw, size_t ldv, int n, int j, int m, TV* __restrict__ w,
           SolveState* st, double* partials, unsigned* counter, double* hist, int hist_cap) {
    if (!st->cycle_active) return;
    constexpr int VN = Vec<TV>::N;
    const int nk = j + 1;
    __shared__ TV cf[SG_MMAX + 1];
    for (int k = threadIdx.x; k < nk; k += blockDim.x) cf[k] = (TV)(st->h[k] * st->vscale[k]);
    __syncthreads();
    TV ss = (TV)0;
    const int nvec = n / VN;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nvec; u += gridDim.x * blockDim.x) {
        TV wv[VN];
        vload<TV>(w + (size_t)u * VN, wv);
        int k = 0;
        for (; k + 4 <= nk; k += 4) {
            TV a[4][VN];
#pragma unroll
            for (int q = 0; q < 4; ++q) vload<TV>(raw + (size_t)(k + q) * ldv + (size_t)u * VN, a[q]);
#pragma unroll
            for (int q = 0; q < 4; ++q)
#pragma unroll
                for (int e = 0; e < VN; ++e) wv[e] -= cf[k + q] * a[q][e];
        }
        for (; k < nk; ++k) {
            TV a[VN];
            vload<TV>(raw + (size_t)k * ldv + (size_t)u * VN, a);
#pragma unroll
            for (int e = 0; e < VN; ++e) wv[e] -= cf[k] * a[e];
        }
        vstore<TV>(w + (size_t)u * VN, wv);
#pragma unroll
        for (int e = 0; e < VN; ++e) ss += wv[e] * wv[e];
    }
    for (int i = nvec * VN + blockIdx.x * blockDim.x + threadIdx.x; i < n;
         i += gridDim.x * blockDim.x) {
        TV wi = w[i];
        for (int k = 0; k < nk; ++k) wi -= cf[k] * raw[(size_t)k * ldv + i];
        w[i] = wi;
        ss += wi * wi;
    }
    __shared__ double red[KT / 32];
    __shared__ double bs[1], tot[1];
    TV v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (last_block_reduce(partials, counter, bs, 1, tot))
        arnoldi_finalize(st, j, m, tot[0], hist, hist_cap);
}

// ---- cycle start: beta = ||raw0||
template <class TV>
__global__ void __launch_bounds__(KT)
k_cycle_init(const TV* __restrict__ raw0, int n, SolveState* st, int m, int flexible,
             double* partials, unsigned* counter) {
    if (st->done) return;
    constexpr int VN = Vec<TV>::N;
    TV ss = (TV)0;  // per-thread sum in the basis precision
    const int nvec = n / VN;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nvec; u += gridDim.x * blockDim.x) {
        TV v[VN];
        vload<TV>(raw0 + (size_t)u * VN, v);
#pragma unroll
        for (int e = 0; e < VN; ++e) ss += v[e] * v[e];
    }
    if (blockIdx.x == 0 && (int)threadIdx.x < n - nvec * VN) {
        const TV t = raw0[nvec * VN + threadIdx.x];
        ss += t * t;
    }
    __shared__ double red[KT / 32];
    __shared__ double bs[1], tot[1];
    TV v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (!last_block_reduce(partials, counter, bs, 1, tot)) return;
    const int ld = m + 1;
    for (int i = threadIdx.x; i < ld * m; i += blockDim.x) st->H[i] = 0.0;
    for (int i = threadIdx.x; i <= m; i += blockDim.x) st->g[i] = 0.0;
    __syncthreads();
    if (threadIdx.x != 0) return;
    const double beta = sqrt(tot[0]);
    st->beta = beta;
    st->j = 0;
    st->kcount = 0;
    st->breakdown = 0;
    if (!isfinite(beta)) {
        st->nonfinite = 1;
        st->done = 1;
        st->cycle_active = 0;
        return;
    }
    if (st->tol_kind == SG_TOL_REF_ABS && beta < st->tol) {
        // src/core/gmres.cpp:264-269
        st->converged = 1;
        st->done = 1;
        st->cycle_active = 0;
        return;
    }
    if (!(beta > 0.0)) {
        st->done = 1;
        st->cycle_active = 0;
        return;
    }
    st->vscale[0] = 1.0 / beta;
    st->lagT[0] = 1.0 / beta;  // lagged CGS2: v_0 = raw_0 / beta
    st->g[0] = beta;
    st->est_scale = flexible ? 1.0 : st->rnorm / beta;
    st->cycle_active = 1;
}

// y = H^{-1} g on the k x k upper triangle of the rotated Hessenberg
// (src/core/gmres.cpp:131-137).  Up to SG_LAGM columns one warp solves it in
// shared memory column by column (y_i, then every lane updates its rows);
// longer triangles use one thread.  Lagged CGS2: also the coefficients on
// the stored vectors, cfu = T y.
__global__ void __launch_bounds__(BS_T) k_backsolve(SolveState* st, int m) {
    if (blockIdx.x != 0) return;
    const int k = st->kcount;
    const int ld = m + 1;
    const int tid = threadIdx.x, lane = tid & 31;
    if (k > SG_LAGM) {
        if (tid != 0) return;
        for (int i = k - 1; i >= 0; --i) {
            double yi = st->g[i];
            for (int l = i + 1; l < k; ++l) yi -= st->H[i + l * ld] * st->y[l];
            st->y[i] = yi / st->H[i + i * ld];
        }
        return;
    }
    // the whole block loads R (and T) with independent loads; one warp then
    // solves, the block forms T y
    __shared__ double Hs[SG_LAGM][SG_LAGM + 1], Ts[SG_LAGM][SG_LAGM + 1];
    __shared__ double gs[SG_LAGM], ys[SG_LAGM];
    const bool lagged = st->lagged != 0;
    for (int idx = tid; idx < k * k; idx += blockDim.x) {
        const int i = idx % k, l = idx / k;
        Hs[i][l] = i <= l ? st->H[i + l * ld] : 0.0;
        if (lagged) Ts[i][l] = i <= l ? st->lagT[i + l * SG_LAGM] : 0.0;
    }
    for (int i = tid; i < k; i += blockDim.x) gs[i] = st->g[i];
    __syncthreads();
    if (tid < 32) {
        for (int i = k - 1; i >= 0; --i) {
            const double yi = gs[i] / Hs[i][i];
            if (lane == 0) ys[i] = yi;
            for (int t = lane; t < i; t += 32) gs[t] -= Hs[t][i] * yi;
            __syncwarp();
        }
    }
    __syncthreads();
    for (int i = tid; i < k; i += blockDim.x) st->y[i] = ys[i];
    if (!lagged) return;
    // V y = S (T y): coefficients on the stored vectors
    for (int i = tid; i < k; i += blockDim.x) {
        double u = 0.0;
        for (int l = i; l < k; ++l) u += Ts[i][l] * ys[l];
        st->cfu[i] = u;
    }
}

// x += V y: the correction is formed in the basis precision (FP32 for the
// mixed solver: the inner solve's precision) and added to x in FP64.  A
// thread takes one 16-byte vector of elements and four basis vectors' loads
// at a time; per element the terms are summed in basis order.
template <class TV>
__global__ void __launch_bounds__(KT)
k_update_x(const TV* __restrict__ basis, size_t ldv, int n, double* __restrict__ x,
           SolveState* st) {
    const int k = st->kcount;
    if (k <= 0) return;
    constexpr int VN = Vec<TV>::N;
    __shared__ TV cf[SG_MMAX];
    for (int i = threadIdx.x; i < k; i += blockDim.x)
        cf[i] = st->lagged ? (TV)st->cfu[i] : (TV)(st->y[i] * st->vscale[i]);
    __syncthreads();
    const int nvec = n / VN;
    const int stride = gridDim.x * blockDim.x;
    for (int u = blockIdx.x * blockDim.x + threadIdx.x; u < nvec; u += stride) {
        TV d[VN];
#pragma unroll
        for (int e = 0; e < VN; ++e) d[e] = (TV)0;
        int q = 0;
        for (; q + 4 <= k; q += 4) {
            TV a[4][VN];
#pragma unroll
            for (int r = 0; r < 4; ++r) vload<TV>(basis + (size_t)(q + r) * ldv + (size_t)u * VN, a[r]);
#pragma unroll
            for (int r = 0; r < 4; ++r)
#pragma unroll
                for (int e = 0; e < VN; ++e) d[e] += cf[q + r] * a[r][e];
        }
        for (; q < k; ++q) {
            TV a[VN];
            vload<TV>(basis + (size_t)q * ldv + (size_t)u * VN, a);
#pragma unroll
            for (int e = 0; e < VN; ++e) d[e] += cf[q] * a[e];
        }
#pragma unroll
        for (int e = 0; e < VN; ++e) x[(size_t)u * VN + e] += (double)d[e];
    }
    for (int i = nvec * VN + blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
        TV d = (TV)0;
        for (int q = 0; q < k; ++q) d += cf[q] * basis[(size_t)q * ldv + i];
        x[i] += (double)d;
    }
}

template <class TI, class TO>
__global__ void k_copy(const TI* __restrict__ x, TO* __restrict__ y, int n,
                       const int* __restrict__ active) {
    if (active && *active == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = (TO)x[i];
}

__global__ void k_cycle_end(SolveState* st) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    st->cycles++;
    if (!st->done && st->total_iter >= st->max_iter) st->done = 1;
    st->cycle_active = st->done ? 0 : 1;
}

// ---- BLAS-1 of src/core/vector.h:11-44
// dot: per-thread sums in a fixed grid-stride order, block sums, then the
// last block adds the block partials in block order (deterministic).
__global__ void __launch_bounds__(KT)
k_dot(const double* __restrict__ x, const double* __restrict__ y, int n, double* partials,
      unsigned* counter, double* out) {
    double acc = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        acc = fma(x[i], y[i], acc);
    __shared__ double red[KT / 32];
    __shared__ double bs[1], tot[1];
    double v1[1] = {acc};
    block_sum_multi<1>(v1, 1, red, bs);
    if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0) *out = tot[0];
}

// y += alpha x, product and sum rounded separately (the reference's bits)
__global__ void k_axpy(double alpha, const double* __restrict__ x, double* __restrict__ y, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        y[i] = __dadd_rn(y[i], __dmul_rn(alpha, x[i]));
}

__global__ void k_scale(double alpha, double* __restrict__ x, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        x[i] = __dmul_rn(x[i], alpha);
}

int kgrid(sg_ctx* ctx, int n, int per_sm) {
    long long need = ((long long)n + KT - 1) / KT;
    long long cap = (long long)ctx->num_sms * per_sm;
    if (need > cap) need = cap;
    return need < 1 ? 1 : (int)need;
}

}  // namespace

template <class TV>
void launch_cycle_init(sg_ctx* ctx, const TV* raw0, int n, SolveState* st, int m, bool flexible) {
    k_cycle_init<TV><<<kgrid(ctx, (n + 3) / 4, 4), KT, 0, ctx->stream>>>(
        raw0, n, st, m, flexible ? 1 : 0, ctx->partials.p, ctx->counter.p);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template <class TV>
static void dots_any(sg_ctx* ctx, const TV* raw, size_t ldv, int n, int nk, const TV* w,
                     SolveState* st, int second, int lagged = 0) {
    for (int k0 = 0; k0 < nk; k0 += KW * KPW) {
        const int kc = nk - k0 < KW * KPW ? nk - k0 : KW * KPW;
        k_dots<TV><<<kgrid(ctx, (n + 3) / 4 * 8, 4), KT, 0, ctx->stream>>>(
            raw, ldv, n, k0, kc, w, st, second, lagged, ctx->partials.p, ctx->counter.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    }
}

template <class TV>
void launch_cgs2(sg_ctx* ctx, TV* raw, size_t ldv, int n, int j, int m, SolveState* st,
                 bool lagged) {
    const int nk = j + 1;
    TV* w = raw + (size_t)(j + 1) * ldv;
    if (lagged) {
        // two passes (see lagged_pass_a / lagged_pass_b); m < SG_LAGM <= 32
        if (m >= SG_LAGM || nk > KW * KPW) fail(SG_ERR_INTERNAL, "lagged CGS2 needs m < %d", SG_LAGM);
        dots_any<TV>(ctx, raw, ldv, n, nk, w, st, 0, 1);
        k_upd_dots<TV><<<kgrid(ctx, (n + 3) / 4 * 8, 3), KT, 0, ctx->stream>>>(
            raw, ldv, n, nk, w, st, ctx->partials.p, ctx->counter.p, 1, m, ctx->hist_d,
            ctx->hist_cap);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        return;
    }
    // pass A
    dots_any<TV>(ctx, raw, ldv, n, nk, w, st, 0);
    // pass B
    if (nk <= KW * KPW) {
        k_upd_dots<TV><<<kgrid(ctx, (n + 3) / 4 * 8, 3), KT, 0, ctx->stream>>>(
            raw, ldv, n, nk, w, st, ctx->partials.p, ctx->counter.p, 0, m, nullptr, 0);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
    } else {
        k_upd<TV><<<kgrid(ctx, n, 4), KT, 0, ctx->stream>>>(raw, ldv, n, nk, w, st);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        dots_any<TV>(ctx, raw, ldv, n, nk, w, st, 1);
    }
    // pass C
    k_upd_norm<TV><<<kgrid(ctx, n / Vec<TV>::N + 1, 4), KT, 0, ctx->stream>>>(
        raw, ldv, n, j, m, w, st, ctx->partials.p, ctx->counter.p, ctx->hist_d, ctx->hist_cap);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

void launch_backsolve(sg_ctx* ctx, SolveState* st, int m) {
    k_backsolve<<<1, BS_T, 0, ctx->stream>>>(st, m);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template <class TV>
void launch_update_x(sg_ctx* ctx, const TV* basis, size_t ldv, int n, double* x, SolveState* st) {
    k_update_x<TV><<<kgrid(ctx, n, 4), KT, 0, ctx->stream>>>(basis, ldv, n, x, st);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template <class TI, class TO>
void launch_copy(sg_ctx* ctx, const TI* x, TO* y, int n, const int* active) {
    k_copy<TI, TO><<<kgrid(ctx, n, 4), KT, 0, ctx->stream>>>(x, y, n, active);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

// grid of the dot-product reduction: at most 1024 blocks
int dot_grid(int num_sms, int n) {
    long long need = ((long long)n + KT - 1) / KT;
    long long cap = (long long)num_sms * 2;
    if (cap > 1024) cap = 1024;
    if (need > cap) need = cap;
    return need < 1 ? 1 : (int)need;
}

void launch_dot(sg_ctx* ctx, const double* x, const double* y, int n, double* out_dev) {
    k_dot<<<dot_grid(ctx->num_sms, n), KT, 0, ctx->stream>>>(x, y, n, ctx->partials.p,
                                                              ctx->counter.p, out_dev);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

void launch_dot_scratch(cudaStream_t stream, const double* x, const double* y, int n,
                        int blocks, double* partials, unsigned* counter, double* out_dev) {
    k_dot<<<blocks, KT, 0, stream>>>(x, y, n, partials, counter, out_dev);
    SG_CUDA(cudaGetLastError());
}

void launch_axpy(sg_ctx* ctx, double alpha, const double* x, double* y, int n) {
    k_axpy<<<kgrid(ctx, n, 8), KT, 0, ctx->stream>>>(alpha, x, y, n);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

void launch_scale(sg_ctx* ctx, double alpha, double* x, int n) {
    k_scale<<<kgrid(ctx, n, 8), KT, 0, ctx->stream>>>(alpha, x, n);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

void launch_cycle_end(sg_ctx* ctx, SolveState* st) {
    k_cycle_end<<<1, 32, 0, ctx->stream>>>(st);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template void launch_cycle_init<double>(sg_ctx*, const double*, int, SolveState*, int, bool);
template void launch_cycle_init<float>(sg_ctx*, const float*, int, SolveState*, int, bool);
template void launch_cgs2<double>(sg_ctx*, double*, size_t, int, int, int, SolveState*, bool);
template void launch_cgs2<float>(sg_ctx*, float*, size_t, int, int, int, SolveState*, bool);
template void launch_update_x<double>(sg_ctx*, const double*, size_t, int, double*, SolveState*);
template void launch_update_x<float>(sg_ctx*, const float*, size_t, int, double*, SolveState*);
template void launch_copy<double, double>(sg_ctx*, const double*, double*, int, const int*);
template void launch_copy<double, float>(sg_ctx*, const double*, float*, int, const int*);
template void launch_copy<float, float>(sg_ctx*, const float*, float*, int, const int*);
template void launch_copy<float, double>(sg_ctx*, const float*, double*, int, const int*);

}  // namespace sg
