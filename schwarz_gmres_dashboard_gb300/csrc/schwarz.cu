// schwarz.cu -- device side of the preconditioners: Jacobi
// (src/precond/jacobi.h:10-27), ILU(0) (src/precond/ilu0.h:13-79), one-level
// ASM/RAS (src/precond/asm.h:34-60, src/precond/ras.h:45-70) and the
// piecewise-constant two-level coarse space (src/precond/coarse_space.h:26-78,
// src/precond/coarse_solve.h:15-67).  Replaces the host-staged GPU path of
// src/gpu/asm_gpu.h:108-165 and the single-thread sweep kernel of
// src/gpu/local_solve_kernel.cu:13-74.
//
// Every subdomain stays resident on the device.  One CTA owns one subdomain:
// it gathers its overlapped right-hand side from the global vector (the
// restriction that replaces the MPI halo exchange), runs the ILU(0) forward
// and backward sweeps in shared memory level by level (rows of one level are
// independent; one __syncthreads per level), and scatters its owned rows
// (RAS) or all rows with atomics (ASM), adding the coarse correction of its
// own part.  Factors are stored per level in ELL slices, so the threads of a
// level read them with coalesced loads.
#include <algorithm>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int SWEEP_T = 512;

// ---------------------------------------------------------------- Jacobi
__global__ void k_jacobi_setup(int n, const int* __restrict__ rp, const int* __restrict__ ci,
                               const double* __restrict__ v, double* inv, float* inv32) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        // CSRMatrix::diagonal (src/core/sparse_matrix.h:45-51): first match, else 0
        double d = 0.0;
        for (int e = rp[i]; e < rp[i + 1]; ++e)
            if (ci[e] == i) {
                d = v[e];
                break;
            }
        const double r = (fabs(d) > 1e-15) ? 1.0 / d : 1.0;
        inv[i] = r;
        inv32[i] = (float)r;
    }
}

template <class TI, class TO, class TD>
__global__ void k_jacobi(int n, const TD* __restrict__ inv, const TI* __restrict__ x,
                         TO* __restrict__ y, const int* __restrict__ active) {
    if (active && *active == 0) return;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (sizeof(TD) == 8) y[i] = (TO)__dmul_rn((double)inv[i], (double)x[i]);
        else y[i] = (TO)((float)inv[i] * (float)x[i]);
    }
}

// ---------------------------------------------------------------- ILU(0) set-up
__global__ void k_gather_vals(long long nz, const int* __restrict__ map,
                              const double* __restrict__ aval, double* __restrict__ lu) {
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < nz;
         e += (long long)gridDim.x * blockDim.x)
        lu[e] = aval[map[e]];
}

// In-place ILU(0) of every subdomain, rows in forward-level order; the
// arithmetic of one row is src/precond/ilu0.h:313-333 step for step (same
// skip rule, same first-match search, product and difference rounded
// separately).
template <class TC>
__global__ void __launch_bounds__(SWEEP_T, 2)
k_factor(const SubInfo* __restrict__ info, const int* __restrict__ lrp,
         const int* __restrict__ lci, const int* __restrict__ ldiag,
         const TC* __restrict__ perm_f, const int* __restrict__ lev_f, double* lu) {
    const SubInfo inf = info[blockIdx.x];
    const int* rp = lrp + inf.csr_row_off;
    const int* ci = lci + inf.csr_nz_off;
    double* v = lu + inf.csr_nz_off;
    const int* dg = ldiag + inf.row_off;
    const TC* pf = perm_f + inf.row_off;
    const int* lf = lev_f + inf.lev_off_f;
    for (int l = 0; l < inf.nlev_f; ++l) {
        const int p0 = lf[l], p1 = lf[l + 1];
        for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
            const int i = pf[p];
            const int rs = rp[i], re = rp[i + 1];
            for (int jp = rs; jp < re; ++jp) {
                const int k = ci[jp];
                if (k >= i) break;
                const int dk = dg[k];
                if (dk < 0 || fabs(v[dk]) < 1e-30) continue;
                const double a = v[jp] / v[dk];
                v[jp] = a;
                const int ke = rp[k + 1];
                for (int kp = dk + 1; kp < ke; ++kp) {
                    const int col = ci[kp];
                    for (int ip = rs; ip < re; ++ip) {
                        if (ci[ip] == col) {
                            v[ip] = __dsub_rn(v[ip], __dmul_rn(a, v[kp]));
                            break;
                        }
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <class TF>
__device__ __forceinline__ TF cvt_factor(double v);
template <>
__device__ __forceinline__ double cvt_factor<double>(double v) { return v; }
template <>
__device__ __forceinline__ float cvt_factor<float>(double v) { return (float)v; }
template <>
__device__ __forceinline__ uint16_t cvt_factor<uint16_t>(double v) {
    return __bfloat16_as_ushort(__float2bfloat16_rn((float)v));
}

// Factored local CSR -> level-major ELL slices of type TF.
template <class TF, class TC>
__global__ void __launch_bounds__(SWEEP_T, 2)
k_pack(const SubInfo* __restrict__ info, const int* __restrict__ lrp,
       const int* __restrict__ lci, const int* __restrict__ ldiag,
       const double* __restrict__ lu, const TC* __restrict__ perm_f,
       const TC* __restrict__ perm_b, TC* lcol, TF* lval, TC* ucol, TF* uval, TF* udiag) {
    const SubInfo inf = info[blockIdx.x];
    const int n = inf.n;
    const int* rp = lrp + inf.csr_row_off;
    const int* ci = lci + inf.csr_nz_off;
    const double* v = lu + inf.csr_nz_off;
    const int* dg = ldiag + inf.row_off;
    for (int p = threadIdx.x; p < n; p += blockDim.x) {
        const int r = perm_f[inf.row_off + p];
        int k = 0;
        for (int e = rp[r]; e < rp[r + 1] && k < inf.wl; ++e) {
            const int c = ci[e];
            if (c >= r) break;
            lcol[inf.fl_off + (long long)k * n + p] = (TC)c;
            lval[inf.fl_off + (long long)k * n + p] = cvt_factor<TF>(v[e]);
            ++k;
        }
        for (; k < inf.wl; ++k) {
            lcol[inf.fl_off + (long long)k * n + p] = (TC)n;
            lval[inf.fl_off + (long long)k * n + p] = cvt_factor<TF>(0.0);
        }
        const int rb = perm_b[inf.row_off + p];
        k = 0;
        for (int e = dg[rb] + 1; e < rp[rb + 1] && k < inf.wu; ++e) {
            ucol[inf.fu_off + (long long)k * n + p] = (TC)ci[e];
            uval[inf.fu_off + (long long)k * n + p] = cvt_factor<TF>(v[e]);
            ++k;
        }
        for (; k < inf.wu; ++k) {
            ucol[inf.fu_off + (long long)k * n + p] = (TC)n;
            uval[inf.fu_off + (long long)k * n + p] = cvt_factor<TF>(0.0);
        }
        udiag[inf.row_off + p] = cvt_factor<TF>(v[dg[rb]]);
    }
}

// ---------------------------------------------------------------- sweeps
// One triangular sweep of a subdomain held in shared memory `t`.  Rows of a
// level are independent; a __syncthreads separates levels.  The factor
// entries, columns and row index of the next level are loaded into registers
// before the current level is computed, so the global-memory latency of level
// l+1 overlaps the arithmetic and the barrier of level l.  The per-row order
// of the subtractions (and the final division of the backward sweep) is the
// reference's (src/precond/ilu0.h:62-76).
constexpr int SWEEP_WP = 4;  // ELL widths up to this are prefetched

template <class TS, class TF, class TC, bool BACK>
__device__ __forceinline__ void sweep_levels(TS* t, int n, int nlev, const int* __restrict__ lptr,
                                             const TC* __restrict__ perm,
                                             const TC* __restrict__ col,
                                             const TF* __restrict__ val,
                                             const TF* __restrict__ diag, int w) {
    if (w > SWEEP_WP) {
        for (int l = 0; l < nlev; ++l) {
            const int p0 = lptr[l], p1 = lptr[l + 1];
            for (int p = p0 + threadIdx.x; p < p1; p += blockDim.x) {
                const int r = perm[p];
                TS acc = t[r];
                for (int k = 0; k < w; ++k)
                    acc = msub(acc, Load<TS>::f(val[(size_t)k * n + p]), t[col[(size_t)k * n + p]]);
                if (BACK) acc = div_diag(acc, Load<TS>::f(diag[p]));
                t[r] = acc;
            }
            __syncthreads();
        }
        return;
    }
    // registers for the first pass of the next level
    bool have = false;
    int r = 0;
    TS v[SWEEP_WP];
    int c[SWEEP_WP];
    TS d = (TS)1;
    auto fetch = [&](int p) {
        r = perm[p];
#pragma unroll
        for (int k = 0; k < SWEEP_WP; ++k) {
            if (k < w) {
                v[k] = Load<TS>::f(val[(size_t)k * n + p]);
                c[k] = col[(size_t)k * n + p];
            }
        }
        if (BACK) d = Load<TS>::f(diag[p]);
    };
    if (nlev > 0) {
        const int p = lptr[0] + threadIdx.x;
        have = p < lptr[1];
        if (have) fetch(p);
    }
    for (int l = 0; l < nlev; ++l) {
        const int p0 = lptr[l], p1 = lptr[l + 1];
        const bool cur = have;
        const int rc = r;
        TS vc[SWEEP_WP];
        int cc[SWEEP_WP];
#pragma unroll
        for (int k = 0; k < SWEEP_WP; ++k) {
            vc[k] = v[k];
            cc[k] = c[k];
        }
        const TS dc = d;
        have = false;
        if (l + 1 < nlev) {
            const int q = p1 + threadIdx.x;
            have = q < lptr[l + 2];
            if (have) fetch(q);
        }
        if (cur) {
            TS acc = t[rc];
#pragma unroll
            for (int k = 0; k < SWEEP_WP; ++k)
                if (k < w) acc = msub(acc, vc[k], t[cc[k]]);
            if (BACK) acc = div_diag(acc, dc);
            t[rc] = acc;
        }
        // rows of this level beyond the first pass
        for (int q = p0 + threadIdx.x + blockDim.x; q < p1; q += blockDim.x) {
            const int rr = perm[q];
            TS acc = t[rr];
            for (int k = 0; k < w; ++k)
                acc = msub(acc, Load<TS>::f(val[(size_t)k * n + q]), t[col[(size_t)k * n + q]]);
            if (BACK) acc = div_diag(acc, Load<TS>::f(diag[q]));
            t[rr] = acc;
        }
        __syncthreads();
    }
}

// mode 0: RAS (owned rows written), 1: ASM (all rows added atomically).
template <class TI, class TO, class TS, class TF, class TC>
__global__ void __launch_bounds__(SWEEP_T, 2)
k_sweep(const SubInfo* __restrict__ info, const int* __restrict__ order,
        const int* __restrict__ dofs, const TC* __restrict__ perm_f,
        const int* __restrict__ lev_f, const TC* __restrict__ lcol, const TF* __restrict__ lval,
        const TC* __restrict__ perm_b, const int* __restrict__ lev_b,
        const TC* __restrict__ ucol, const TF* __restrict__ uval,
        const TF* __restrict__ udiag, const int* __restrict__ ownloc,
        const int* __restrict__ owned_glob, const TI* __restrict__ x, TO* __restrict__ y,
        int mode, int coarse, const double* __restrict__ a0inv, const double* __restrict__ r0,
        int nc, TS* gscratch, int use_smem, const int* __restrict__ active,
        const int* __restrict__ sub_on) {
    if (active && *active == 0) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double s_zc;
    const int s = order[blockIdx.x];
    if (sub_on && !sub_on[s]) return;  // subdomain not needed by this apply
    const SubInfo inf = info[s];
    const int n = inf.n;
    TS* t = use_smem ? reinterpret_cast<TS*>(smraw) : gscratch + inf.row_off + s;
    const int* dof = dofs + inf.row_off;
    // restriction R_s x (gather with overlap)
    gather_rows<TS>(t, x, dof, n, blockDim.x);
    if (threadIdx.x == 0) t[n] = (TS)0;
    if (coarse) {
        // z0_s = (A0^{-1} r0)_s, scaled by the part's coarse basis value
        if (threadIdx.x < 32) {
            const double z = coarse_dot_warp0(a0inv + (size_t)s * nc, r0, nc);
            if (threadIdx.x == 0) s_zc = inf.cscale * z;
        }
        __syncthreads();
    }
    __syncthreads();
    // forward sweep (unit lower triangle), then backward sweep (upper
    // triangle and diagonal), level by level
    sweep_levels<TS, TF, TC, false>(t, n, inf.nlev_f, lev_f + inf.lev_off_f, perm_f + inf.row_off,
                                    lcol + inf.fl_off, lval + inf.fl_off, nullptr, inf.wl);
    sweep_levels<TS, TF, TC, true>(t, n, inf.nlev_b, lev_b + inf.lev_off_b, perm_b + inf.row_off,
                                   ucol + inf.fu_off, uval + inf.fu_off, udiag + inf.row_off,
                                   inf.wu);
    const double zc = coarse ? s_zc : 0.0;
    if (mode == 0) {
        // restricted prolongation: owned rows only (src/precond/ras.h:64-68)
        const int* ol = ownloc + inf.own_off;
        const int* og = owned_glob + inf.own_off;
        scatter_owned<TS, TO>(t, y, ol, og, inf.n_own, coarse, zc, blockDim.x);
    } else {
        // additive prolongation of every row (src/precond/asm.h:138-142)
        for (int li = threadIdx.x; li < n; li += blockDim.x)
            atomicAdd(&y[dof[li]], Store<TO>::f(t[li]));
        if (coarse) {
            const int* og = owned_glob + inf.own_off;
            for (int q = threadIdx.x; q < inf.n_own; q += blockDim.x)
                atomicAdd(&y[og[q]], Store<TO>::f(zc));
        }
    }
}

// ---------------------------------------------------------------- sync-free sweeps
// The same forward/backward sweeps without a barrier per level.  Thread t
// takes the rows at level-order positions t, t + blockDim, ... and, before
// using row c, waits until c's ready flag (one byte in shared memory) shows
// the current sweep; it then publishes its own row (value, block fence,
// flag).  Every dependency sits at an earlier position and each thread walks
// its positions in increasing order, so the waits always end; they are
// bounded anyway (on expiry the thread records an error word and carries on).
// The next row's factor entries are loaded before the current row's waits,
// so their global-memory latency overlaps the dependency chain.
constexpr long long SF_SPIN_LIMIT = 1ll << 24;

template <class TS, bool EXACT>
__device__ __forceinline__ TS sf_sub(TS acc, TS a, TS b) {
    if (EXACT) return msub(acc, a, b);
    return acc - a * b;  // contracts to a fused multiply-add
}

template <class TS, class TF, class TC, bool BACK, bool EXACT>
__device__ __forceinline__ void sweep_sf(TS* t, volatile unsigned char* fl, int n,
                                         const TC* __restrict__ perm, const TC* __restrict__ col,
                                         const TF* __restrict__ val, const TF* __restrict__ diag,
                                         int w, unsigned char epoch, int* err) {
    auto wait_row = [&](int c) {
        long long it = 0;
        while (fl[c] < epoch) {
            if (++it > SF_SPIN_LIMIT) {
                atomicExch(err, 2);
                break;
            }
        }
        __threadfence_block();
    };
    if (w > SWEEP_WP) {
        for (int p = threadIdx.x; p < n; p += blockDim.x) {
            const int r = perm[p];
            TS acc = t[r];
            for (int k = 0; k < w; ++k) {
                const int c = col[(size_t)k * n + p];
                const TS v = Load<TS>::f(val[(size_t)k * n + p]);
                wait_row(c);
                acc = sf_sub<TS, EXACT>(acc, v, t[c]);
            }
            if (BACK) acc = div_diag(acc, Load<TS>::f(diag[p]));
            t[r] = acc;
            __threadfence_block();
            fl[r] = epoch;
        }
        return;
    }
    int r = 0, c[SWEEP_WP];
    TS v[SWEEP_WP], d = (TS)1;
    auto fetch = [&](int p) {
        r = perm[p];
#pragma unroll
        for (int k = 0; k < SWEEP_WP; ++k)
            if (k < w) {
                c[k] = col[(size_t)k * n + p];
                v[k] = Load<TS>::f(val[(size_t)k * n + p]);
            }
        if (BACK) d = Load<TS>::f(diag[p]);
    };
    int p = threadIdx.x;
    if (p < n) fetch(p);
    for (; p < n; p += blockDim.x) {
        const int rc = r;
        int cc[SWEEP_WP];
        TS vc[SWEEP_WP];
#pragma unroll
        for (int k = 0; k < SWEEP_WP; ++k) {
            cc[k] = c[k];
            vc[k] = v[k];
        }
        const TS dc = d;
        if (p + (int)blockDim.x < n) fetch(p + blockDim.x);
        TS acc = t[rc];
#pragma unroll
        for (int k = 0; k < SWEEP_WP; ++k) {
            if (k < w) {
                wait_row(cc[k]);
                acc = sf_sub<TS, EXACT>(acc, vc[k], t[cc[k]]);
            }
        }
        if (BACK) acc = div_diag(acc, dc);
        t[rc] = acc;
        __threadfence_block();
        fl[rc] = epoch;
    }
}

template <class TI, class TO, class TS, class TF, class TC, bool EXACT>
__global__ void __launch_bounds__(SWEEP_T, 2)
k_sweep_sf(const SubInfo* __restrict__ info, const int* __restrict__ order,
           const int* __restrict__ dofs, const TC* __restrict__ perm_f,
           const TC* __restrict__ lcol, const TF* __restrict__ lval,
           const TC* __restrict__ perm_b, const TC* __restrict__ ucol,
           const TF* __restrict__ uval, const TF* __restrict__ udiag,
           const int* __restrict__ ownloc, const int* __restrict__ owned_glob,
           const TI* __restrict__ x, TO* __restrict__ y, int mode, int coarse,
           const double* __restrict__ a0inv, const double* __restrict__ r0, int nc, int* err,
           const int* __restrict__ active, const int* __restrict__ sub_on) {
    if (active && *active == 0) return;
    extern __shared__ __align__(16) unsigned char smraw[];
    __shared__ double s_zc;
    const int s = order[blockIdx.x];
    if (sub_on && !sub_on[s]) return;  // subdomain not needed by this apply
    const SubInfo inf = info[s];
    const int n = inf.n;
    TS* t = reinterpret_cast<TS*>(smraw);
    volatile unsigned char* fl =
        smraw + (((size_t)(n + 1) * sizeof(TS) + 15) & ~(size_t)15);
    const int* dof = dofs + inf.row_off;
    gather_rows<TS>(t, x, dof, n, blockDim.x);
    for (int li = threadIdx.x; li < n; li += blockDim.x) fl[li] = 0;
    if (threadIdx.x == 0) {
        t[n] = (TS)0;  // padded entries read this zero
        fl[n] = 2;
    }
    if (coarse) {
        if (threadIdx.x < 32) {
            const double z = coarse_dot_warp0(a0inv + (size_t)s * nc, r0, nc);
            if (threadIdx.x == 0) s_zc = inf.cscale * z;
        }
        __syncthreads();
    }
    __syncthreads();
    sweep_sf<TS, TF, TC, false, EXACT>(t, fl, n, perm_f + inf.row_off, lcol + inf.fl_off,
                                       lval + inf.fl_off, nullptr, inf.wl, 1, err);
    __syncthreads();  // every forward read is done before rows change again
    sweep_sf<TS, TF, TC, true, EXACT>(t, fl, n, perm_b + inf.row_off, ucol + inf.fu_off,
                                      uval + inf.fu_off, udiag + inf.row_off, inf.wu, 2, err);
    __syncthreads();
    const double zc = coarse ? s_zc : 0.0;
    if (mode == 0) {
        const int* ol = ownloc + inf.own_off;
        const int* og = owned_glob + inf.own_off;
        scatter_owned<TS, TO>(t, y, ol, og, inf.n_own, coarse, zc, blockDim.x);
    } else {
        for (int li = threadIdx.x; li < n; li += blockDim.x)
            atomicAdd(&y[dof[li]], Store<TO>::f(t[li]));
        if (coarse) {
            const int* og = owned_glob + inf.own_off;
            for (int q = threadIdx.x; q < inf.n_own; q += blockDim.x)
                atomicAdd(&y[og[q]], Store<TO>::f(zc));
        }
    }
}

// ---------------------------------------------------------------- coarse space
// A0[i][j] in the reference's summation order (see oracle notes): for every
// owned row k of part i ascending, the part-j sum of row k in entry order
// (from 0.0), then c_i times it accumulated into A0[i][j] (from 0.0), all
// rounded op by op.  Every (i, j) is its own fold over k, so one block per
// part i lists the parts j its rows touch and gives each j a thread; the
// threads of a warp walk the same rows and entries in lockstep (the loads
// are broadcasts) and each keeps only its own j's terms.
__global__ void __launch_bounds__(256)
k_a0_build(int nc, const int* __restrict__ owned_ptr, const int* __restrict__ owned,
           const int* __restrict__ rp, const int* __restrict__ ci, const double* __restrict__ v,
           const int* __restrict__ part, const double* __restrict__ cscale, double* a0) {
    extern __shared__ __align__(16) unsigned char smraw[];
    int* flag = reinterpret_cast<int*>(smraw);  // nc
    int* list = flag + nc;                      // nc
    __shared__ int s_nl;
    const int i = blockIdx.x;
    const int q0 = owned_ptr[i], q1 = owned_ptr[i + 1];
    for (int t = threadIdx.x; t < nc; t += blockDim.x) flag[t] = 0;
    __syncthreads();
    for (int q = q0 + (int)threadIdx.x; q < q1; q += blockDim.x) {
        const int k = owned[q];
        for (int e = rp[k]; e < rp[k + 1]; ++e) flag[part[ci[e]]] = 1;
    }
    __syncthreads();
    if (threadIdx.x < 32) {  // the touched parts, ascending
        const int lane = threadIdx.x;
        int base = 0;
        for (int t0 = 0; t0 < nc; t0 += 32) {
            const bool on = t0 + lane < nc && flag[t0 + lane];
            const unsigned m = __ballot_sync(0xffffffffu, on);
            if (on) list[base + __popc(m & ((1u << lane) - 1u))] = t0 + lane;
            base += __popc(m);
        }
        if (lane == 0) s_nl = base;
    }
    for (int t = threadIdx.x; t < nc; t += blockDim.x) a0[(size_t)i * nc + t] = 0.0;
    __syncthreads();
    const int nl = s_nl;
    const double c_i = cscale[i];
    for (int x = threadIdx.x; x < nl; x += blockDim.x) {
        const int jj = list[x];
        const double c_j = cscale[jj];
        double row = 0.0;
        for (int q = q0; q < q1; ++q) {
            const int k = owned[q];
            double acc = 0.0;
            bool any = false;
            for (int e = rp[k]; e < rp[k + 1]; ++e) {
                if (part[ci[e]] != jj) continue;
                acc = __dadd_rn(acc, __dmul_rn(v[e], c_j));
                any = true;
            }
            if (any) row = __dadd_rn(row, __dmul_rn(c_i, acc));
        }
        a0[(size_t)i * nc + jj] = row;
    }
}

// Dense LU with partial pivoting, one CTA (src/precond/coarse_solve.h:15-47:
// first strictly larger magnitude, full row swaps, rounded ops in order).
__global__ void __launch_bounds__(1024) k_lu(int n, double* L, int* piv, int* status) {
    __shared__ double s_val[1024];
    __shared__ int s_idx[1024];
    __shared__ int s_bad;
    if (threadIdx.x == 0) s_bad = 0;
    for (int k = 0; k < n; ++k) {
        double bv = -1.0;
        int bi = n;
        for (int i = k + threadIdx.x; i < n; i += blockDim.x) {
            const double a = fabs(L[(size_t)i * n + k]);
            if (a > bv) {
                bv = a;
                bi = i;
            }
        }
        s_val[threadIdx.x] = bv;
        s_idx[threadIdx.x] = bi;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (threadIdx.x < o) {
                const double a = s_val[threadIdx.x + o];
                const int ai = s_idx[threadIdx.x + o];
                if (a > s_val[threadIdx.x] || (a == s_val[threadIdx.x] && ai < s_idx[threadIdx.x])) {
                    s_val[threadIdx.x] = a;
                    s_idx[threadIdx.x] = ai;
                }
            }
            __syncthreads();
        }
        const int mr = s_idx[0];
        const double mv = s_val[0];
        if (threadIdx.x == 0) {
            piv[k] = mr;
            if (!(mv >= 1e-30)) {
                s_bad = 1;
                *status = 1;
            }
        }
        __syncthreads();
        if (s_bad) return;
        if (mr != k)
            for (int j = threadIdx.x; j < n; j += blockDim.x) {
                const double tmp = L[(size_t)k * n + j];
                L[(size_t)k * n + j] = L[(size_t)mr * n + j];
                L[(size_t)mr * n + j] = tmp;
            }
        __syncthreads();
        const double piv_v = L[(size_t)k * n + k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            L[(size_t)i * n + k] = L[(size_t)i * n + k] / piv_v;
        __syncthreads();
        const int rows = n - k - 1;
        const long long cnt = (long long)rows * rows;
        for (long long q = threadIdx.x; q < cnt; q += blockDim.x) {
            const int i = k + 1 + (int)(q / rows);
            const int j = k + 1 + (int)(q % rows);
            L[(size_t)i * n + j] =
                __dsub_rn(L[(size_t)i * n + j], __dmul_rn(L[(size_t)i * n + k], L[(size_t)k * n + j]));
        }
        __syncthreads();
    }
}

// Column t of A0^{-1} from the LU factors (one CTA per column): pivots and
// forward elimination as src/precond/coarse_solve.h:50-67, backward
// substitution by columns.
__global__ void __launch_bounds__(256) k_inv(int n, const double* __restrict__ L,
                                             const int* __restrict__ piv, double* inv) {
    extern __shared__ __align__(16) unsigned char smraw[];
    double* x = reinterpret_cast<double*>(smraw);
    const int t = blockIdx.x;
    for (int i = threadIdx.x; i < n; i += blockDim.x) x[i] = (i == t) ? 1.0 : 0.0;
    __syncthreads();
    for (int k = 0; k < n; ++k) {
        if (threadIdx.x == 0 && piv[k] != k) {
            const double tmp = x[k];
            x[k] = x[piv[k]];
            x[piv[k]] = tmp;
        }
        __syncthreads();
        const double xk = x[k];
        for (int i = k + 1 + threadIdx.x; i < n; i += blockDim.x)
            x[i] = __dsub_rn(x[i], __dmul_rn(L[(size_t)i * n + k], xk));
        __syncthreads();
    }
    for (int k = n - 1; k >= 0; --k) {
        if (threadIdx.x == 0) x[k] = x[k] / L[(size_t)k * n + k];
        __syncthreads();
        const double xk = x[k];
        for (int i = threadIdx.x; i < k; i += blockDim.x)
            x[i] = __dsub_rn(x[i], __dmul_rn(L[(size_t)i * n + k], xk));
        __syncthreads();
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) inv[(size_t)i * n + t] = x[i];
}

// r0[s] = c_s * sum of x over the owned rows of s
template <class TI>
__global__ void __launch_bounds__(1024)
k_restrict(const int* __restrict__ owned_ptr, const int* __restrict__ owned,
           const double* __restrict__ cscale, const TI* __restrict__ x, double* r0,
           const int* __restrict__ active) {
    if (active && *active == 0) return;
    __shared__ double red[RC_MAXCH];
    const int s = blockIdx.x;
    const int q0 = owned_ptr[s], q1 = owned_ptr[s + 1];
    const double z = restrict_chunks<TI>(owned + q0, x, q1 - q0, red);
    if (threadIdx.x == 0) r0[s] = cscale[s] * z;
}

template <class T>
T* dev_ptr(DBuf<T>& b) {
    return b.p;
}

template <class TS, class TF, class TC, class TI, class TO>
void sweep_launch(sg_precond* pc, const TF* lval, const TF* uval, const TF* udiag, const TI* x,
                  TO* y, int mode, bool coarse, const int* active, TS* gscratch) {
    sg_ctx* ctx = pc->ctx;
    // every buffer the kernel dereferences must exist (host-side guard)
    if (!pc->info.p || !pc->order.p || !pc->dofs.p || !pc->perm_f.p || !pc->perm_b.p ||
        !pc->lev_ptr_f.p || !pc->lev_ptr_b.p || !pc->lcol.p || !pc->ucol.p || !lval || !uval ||
        !udiag || !pc->ownloc_d.p || !pc->owned_d.p || (!pc->use_smem && !gscratch) ||
        (coarse && (!pc->a0inv.p || !pc->r0.p)))
        fail(SG_ERR_INTERNAL, "preconditioner device buffers missing for this apply");
    size_t smem = 0;
    if (pc->use_smem) {
        smem = ((size_t)(pc->max_n + 1) * sizeof(TS) + 15) & ~(size_t)15;
        SG_CUDA(cudaFuncSetAttribute(k_sweep<TI, TO, TS, TF, TC>,
                                     cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    }
    k_sweep<TI, TO, TS, TF, TC><<<pc->nparts, SWEEP_T, smem, ctx->stream>>>(
        pc->info.p, pc->order.p, pc->dofs.p, reinterpret_cast<const TC*>(pc->perm_f.p),
        pc->lev_ptr_f.p, reinterpret_cast<const TC*>(pc->lcol.p), lval,
        reinterpret_cast<const TC*>(pc->perm_b.p), pc->lev_ptr_b.p,
        reinterpret_cast<const TC*>(pc->ucol.p), uval, udiag, pc->ownloc_d.p, pc->owned_d.p,
        x, y, mode, coarse ? 1 : 0, pc->a0inv.p, pc->r0.p, pc->nc, gscratch,
        pc->use_smem ? 1 : 0, active, pc->sub_on);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

size_t sf_smem(const sg_precond* pc) {
    const size_t ts = pc->opts.sweep_dtype == SG_FP64 ? 8 : 4;
    return (((size_t)(pc->max_n + 1) * ts + 15) & ~(size_t)15) + (size_t)pc->max_n + 16;
}

template <class TS, class TF, class TC, bool EXACT, class TI, class TO>
void sf_launch(sg_precond* pc, const TF* lval, const TF* uval, const TF* udiag, const TI* x,
               TO* y, int mode, bool coarse, const int* active) {
    sg_ctx* ctx = pc->ctx;
    if (!pc->info.p || !pc->order.p || !pc->dofs.p || !pc->perm_f.p || !pc->perm_b.p ||
        !pc->lcol.p || !pc->ucol.p || !lval || !uval || !udiag || !pc->ownloc_d.p ||
        !pc->owned_d.p || !pc->err_d.p || (coarse && (!pc->a0inv.p || !pc->r0.p)))
        fail(SG_ERR_INTERNAL, "preconditioner device buffers missing for this apply");
    const size_t smem = sf_smem(pc);
    SG_CUDA(cudaFuncSetAttribute(k_sweep_sf<TI, TO, TS, TF, TC, EXACT>,
                                 cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    k_sweep_sf<TI, TO, TS, TF, TC, EXACT><<<pc->nparts, SWEEP_T, smem, ctx->stream>>>(
        pc->info.p, pc->order.p, pc->dofs.p, reinterpret_cast<const TC*>(pc->perm_f.p),
        reinterpret_cast<const TC*>(pc->lcol.p), lval, reinterpret_cast<const TC*>(pc->perm_b.p),
        reinterpret_cast<const TC*>(pc->ucol.p), uval, udiag, pc->ownloc_d.p, pc->owned_d.p, x, y,
        mode, coarse ? 1 : 0, pc->a0inv.p, pc->r0.p, pc->nc, pc->err_d.p, active, pc->sub_on);
    SG_CUDA(cudaGetLastError());
    count_launch(ctx);
}

template <class TC, class TI, class TO>
bool sf_dispatch(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse, bool exact,
                 const int* active) {
    if (!pc->use_sf) return false;
    if (pc->opts.sweep_dtype == SG_FP64) {
        if (exact)
            sf_launch<double, double, TC, true>(pc, pc->lval64.p, pc->uval64.p, pc->udiag64.p, x, y,
                                                mode, coarse, active);
        else
            sf_launch<double, double, TC, false>(pc, pc->lval64.p, pc->uval64.p, pc->udiag64.p, x,
                                                 y, mode, coarse, active);
    } else if (pc->opts.factor_dtype == SG_BF16) {
        sf_launch<float, uint16_t, TC, false>(pc, pc->lval16.p, pc->uval16.p, pc->udiag16.p, x, y,
                                              mode, coarse, active);
    } else {
        sf_launch<float, float, TC, false>(pc, pc->lval32.p, pc->uval32.p, pc->udiag32.p, x, y,
                                           mode, coarse, active);
    }
    return true;
}

template <class TC, class TI, class TO>
void sweep_dispatch(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse,
                    const int* active) {
    if (pc->opts.sweep_dtype == SG_FP64) {
        sweep_launch<double, double, TC>(pc, pc->lval64.p, pc->uval64.p, pc->udiag64.p, x, y, mode,
                                         coarse, active, pc->gscratch64.p);
    } else if (pc->opts.factor_dtype == SG_BF16) {
        sweep_launch<float, uint16_t, TC>(pc, pc->lval16.p, pc->uval16.p, pc->udiag16.p, x, y,
                                          mode, coarse, active, pc->gscratch32.p);
    } else {
        sweep_launch<float, float, TC>(pc, pc->lval32.p, pc->uval32.p, pc->udiag32.p, x, y, mode,
                                       coarse, active, pc->gscratch32.p);
    }
}

template <class TF, class TC>
void pack_launch(sg_precond* pc, TF* lval, TF* uval, TF* udiag) {
    k_pack<TF, TC><<<pc->nparts, SWEEP_T, 0, pc->ctx->stream>>>(
        pc->info.p, pc->lrp_d.p, pc->lci_d.p, pc->ldiag_d.p, pc->lu_d.p,
        reinterpret_cast<const TC*>(pc->perm_f.p), reinterpret_cast<const TC*>(pc->perm_b.p),
        reinterpret_cast<TC*>(pc->lcol.p), lval, reinterpret_cast<TC*>(pc->ucol.p), uval, udiag);
    SG_CUDA(cudaGetLastError());
}

template <class TC>
void factor_and_pack(sg_precond* pc) {
    sg_ctx* ctx = pc->ctx;
    k_factor<TC><<<pc->nparts, SWEEP_T, 0, ctx->stream>>>(
        pc->info.p, pc->lrp_d.p, pc->lci_d.p, pc->ldiag_d.p,
        reinterpret_cast<const TC*>(pc->perm_f.p), pc->lev_ptr_f.p, pc->lu_d.p);
    SG_CUDA(cudaGetLastError());
    // sweep variants: TMA-fed level records (default), a barrier per level
    // with the factors read from global memory (reserved[0] = 1), sync-free
    // with per-row ready flags (reserved[0] = 4)
    const int variant = pc->opts.reserved[0];  // 0 TMA records, 1 level, 4 sync-free
    if (variant != 0) pc->use_rec = false;
    rec_setup_device(pc);
    if (pc->use_rec) return;
    {
        int max_smem = 0;
        SG_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                       ctx->device));
        pc->use_sf = (variant & 4) && pc->use_smem && sf_smem(pc) + 1024 <= (size_t)max_smem;
    }
    if (!pc->err_d.p) {
        pc->err_d.alloc(1);
        pc->err_d.zero(ctx->stream);
    }
    if (pc->wide_cols) {
        pc->lcol.alloc((size_t)pc->fl_total * 2);
        pc->ucol.alloc((size_t)pc->fu_total * 2);
    } else {
        pc->lcol.alloc((size_t)pc->fl_total);
        pc->ucol.alloc((size_t)pc->fu_total);
    }
    const size_t fl = (size_t)pc->fl_total, fu = (size_t)pc->fu_total, nr = (size_t)pc->total_rows;
    if (pc->opts.sweep_dtype == SG_FP64) {
        pc->lval64.alloc(fl); pc->uval64.alloc(fu); pc->udiag64.alloc(nr);
        pack_launch<double, TC>(pc, pc->lval64.p, pc->uval64.p, pc->udiag64.p);
    } else if (pc->opts.factor_dtype == SG_BF16) {
        pc->lval16.alloc(fl); pc->uval16.alloc(fu); pc->udiag16.alloc(nr);
        pack_launch<uint16_t, TC>(pc, pc->lval16.p, pc->uval16.p, pc->udiag16.p);
    } else {
        pc->lval32.alloc(fl); pc->uval32.alloc(fu); pc->udiag32.alloc(nr);
        pack_launch<float, TC>(pc, pc->lval32.p, pc->uval32.p, pc->udiag32.p);
    }
}

}  // namespace

// ---------------------------------------------------------------- set-up
void precond_setup_device(sg_precond* pc, const sg_csr* A) {
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    const int n = A->nrows;
    if (pc->kind == SG_PC_NONE) return;
    if (pc->kind == SG_PC_JACOBI) {
        pc->inv_diag.alloc(n);
        pc->inv_diag32.alloc(n);
        k_jacobi_setup<<<ctx->num_sms * 4, 256, 0, st>>>(n, A->rp.p, A->ci.p, A->val.p,
                                                          pc->inv_diag.p, pc->inv_diag32.p);
        SG_CUDA(cudaGetLastError());
        return;
    }
    // ---- batched ILU(0): host structures -> device
    pc->info.upload(pc->h_info, st);
    pc->order.upload(pc->h_order, st);
    pc->dofs.upload(pc->sub, st);
    pc->lev_ptr_f.upload(pc->h_lev_ptr_f, st);
    pc->lev_ptr_b.upload(pc->h_lev_ptr_b, st);
    pc->lrp_d.upload(pc->lrp, st);
    pc->lci_d.upload(pc->lci, st);
    pc->ldiag_d.upload(pc->ldiag, st);
    pc->lmap_d.upload(pc->lmap, st);
    pc->ownloc_d.upload(pc->ownloc, st);
    pc->owned_ptr_d.upload(pc->owned_ptr, st);
    pc->owned_d.upload(pc->owned, st);
    
    if (pc->wide_cols) {
        pc->perm_f.upload(reinterpret_cast<const uint16_t*>(pc->h_perm_f32.data()),
                          pc->h_perm_f32.size() * 2, st);
        pc->perm_b.upload(reinterpret_cast<const uint16_t*>(pc->h_perm_b32.data()),
                          pc->h_perm_b32.size() * 2, st);
    } else {
        pc->perm_f.upload(pc->h_perm_f16, st);
        pc->perm_b.upload(pc->h_perm_b16, st);
    }
    const long long nz = (long long)pc->lci.size();
    pc->lu_d.alloc((size_t)nz);
    k_gather_vals<<<ctx->num_sms * 4, 256, 0, st>>>(nz, pc->lmap_d.p, A->val.p, pc->lu_d.p);
    SG_CUDA(cudaGetLastError());
    if (pc->wide_cols) factor_and_pack<int>(pc);
    else factor_and_pack<uint16_t>(pc);
    if (!pc->use_smem && !pc->use_rec) {
        const size_t cnt = (size_t)pc->total_rows + (size_t)pc->nparts;
        if (pc->opts.sweep_dtype == SG_FP64) pc->gscratch64.alloc(cnt);
        else pc->gscratch32.alloc(cnt);
    }
    // ---- two-level coarse space
    if (pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS) {
        const int nc = pc->nparts;
        pc->nc = nc;
        pc->part_d.upload(pc->part, st);
        pc->cscale_d.upload(pc->h_cscale, st);
        pc->a0.alloc((size_t)nc * nc);
        pc->lu0.alloc((size_t)nc * nc);
        pc->a0inv.alloc((size_t)nc * nc);
        pc->piv0.alloc(nc);
        pc->r0.alloc(nc);
        pc->status_d.alloc(1);
        pc->status_d.zero(st);
        const size_t smem = (size_t)nc * (4 + 4);
        SG_CUDA(cudaFuncSetAttribute(k_a0_build, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem));
        k_a0_build<<<nc, 256, smem, st>>>(nc, pc->owned_ptr_d.p, pc->owned_d.p, A->rp.p, A->ci.p,
                                         A->val.p, pc->part_d.p, pc->cscale_d.p, pc->a0.p);
        SG_CUDA(cudaGetLastError());
        SG_CUDA(cudaMemcpyAsync(pc->lu0.p, pc->a0.p, sizeof(double) * nc * nc,
                                cudaMemcpyDeviceToDevice, st));
        k_lu<<<1, 1024, 0, st>>>(nc, pc->lu0.p, pc->piv0.p, pc->status_d.p);
        SG_CUDA(cudaGetLastError());
        int bad = 0;
        SG_CUDA(cudaMemcpyAsync(&bad, pc->status_d.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        SG_CUDA(cudaStreamSynchronize(st));
        if (bad) fail(SG_ERR_SINGULAR, "Coarse matrix is singular");
        const size_t smem2 = (size_t)nc * 8;
        SG_CUDA(cudaFuncSetAttribute(k_inv, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)smem2));
        k_inv<<<nc, 256, smem2, st>>>(nc, pc->lu0.p, pc->piv0.p, pc->a0inv.p);
        SG_CUDA(cudaGetLastError());
    }
    SG_CUDA(cudaStreamSynchronize(st));
}

// ---------------------------------------------------------------- apply
template <class TI, class TO>
void precond_apply_device(sg_precond* pc, const TI* x, TO* y, const int* active, bool exact) {
    sg_ctx* ctx = pc->ctx;
    const int n = pc->n;
    const int grid = ctx->num_sms * 4;
    switch (pc->kind) {
    case SG_PC_NONE:
        launch_copy<TI, TO>(ctx, x, y, n, active);
        return;
    case SG_PC_HOST:
        host_precond_apply<TI, TO>(pc, x, y, active, nullptr);
        return;
    case SG_PC_JACOBI:
        if (pc->opts.sweep_dtype == SG_FP64)
            k_jacobi<TI, TO, double><<<grid, 256, 0, ctx->stream>>>(n, pc->inv_diag.p, x, y, active);
        else
            k_jacobi<TI, TO, float><<<grid, 256, 0, ctx->stream>>>(n, pc->inv_diag32.p, x, y, active);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        return;
    default:
        break;
    }
    const bool asm_mode = (pc->kind == SG_PC_ASM || pc->kind == SG_PC_TWOLEVEL_ASM);
    const bool coarse = (pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS);
    if (coarse) {
        if (!pc->owned_ptr_d.p || !pc->owned_d.p || !pc->cscale_d.p || !pc->r0.p)
            fail(SG_ERR_INTERNAL, "coarse-space device buffers missing");
        if (!sweep_fuses_restrict(pc)) {
            k_restrict<TI><<<pc->nc, 1024, 0, ctx->stream>>>(pc->owned_ptr_d.p, pc->owned_d.p,
                                                            pc->cscale_d.p, x, pc->r0.p, active);
            SG_CUDA(cudaGetLastError());
            count_launch(ctx);
        }
    }
    if (asm_mode) SG_CUDA(cudaMemsetAsync(y, 0, sizeof(TO) * (size_t)n, ctx->stream));
    if (sweep_tma<TI, TO>(pc, x, y, asm_mode ? 1 : 0, coarse, exact, active)) return;
    if (pc->wide_cols) {
        if (sf_dispatch<int, TI, TO>(pc, x, y, asm_mode ? 1 : 0, coarse, exact, active)) return;
    } else {
        if (sf_dispatch<uint16_t, TI, TO>(pc, x, y, asm_mode ? 1 : 0, coarse, exact, active))
            return;
    }
    if (pc->wide_cols) sweep_dispatch<int, TI, TO>(pc, x, y, asm_mode ? 1 : 0, coarse, active);
    else sweep_dispatch<uint16_t, TI, TO>(pc, x, y, asm_mode ? 1 : 0, coarse, active);
}

void precond_read_factors(sg_precond* pc, int s, double* lu_out) {
    const SubInfo& inf = pc->h_info[s];
    const int nnz = pc->lrp[inf.csr_row_off + inf.n];
    SG_CUDA(cudaMemcpyAsync(lu_out, pc->lu_d.p + inf.csr_nz_off, sizeof(double) * nnz,
                            cudaMemcpyDeviceToHost, pc->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(pc->ctx->stream));
}

void precond_read_coarse(sg_precond* pc, double* a0_out) {
    SG_CUDA(cudaMemcpyAsync(a0_out, pc->a0.p, sizeof(double) * (size_t)pc->nc * pc->nc,
                            cudaMemcpyDeviceToHost, pc->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(pc->ctx->stream));
}

template void precond_apply_device<double, double>(sg_precond*, const double*, double*,
                                                  const int*, bool);
template void precond_apply_device<double, float>(sg_precond*, const double*, float*,
                                                 const int*, bool);
template void precond_apply_device<float, float>(sg_precond*, const float*, float*, const int*,
                                                bool);

}  // namespace sg
