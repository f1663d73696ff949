// sweep.cu -- the batched ILU(0) subdomain solve fed by TMA bulk copies.
//
// One CTA owns one subdomain (RAS/ASM, src/precond/ras.h:45-70,
// src/precond/asm.h:34-60).  The overlapped right-hand side is gathered into
// shared memory (the restriction that replaces the reference's MPI halo
// exchange), then the forward and backward sweeps of src/precond/ilu0.h:57-79
// run level by level: rows of one level are independent and a __syncthreads
// separates levels.
//
// A level's factor data is one contiguous, 16-byte-aligned record
//   [row slot u16 x C][column slot u16 x C x w][value x C x w](diagonal x C)
// (C = rows rounded up to 8; a slot is the row's place in the shared-memory
// vector, tslot, whose per-subdomain padding keeps the rows of a level in
// distinct banks).  A subdomain's records form one stream (forward levels,
// then backward) that flows through a shared-memory byte ring in groups of
// whole levels: the block's last thread copies a group with one
// cp.async.bulk tracked by an mbarrier, as far ahead as the ring allows (at
// 128^3 all CTAs together stream ~120 MB of records per apply, so the copies
// need tens of KB in flight each).  Where each group lands in the ring and
// after which level it may be issued is a static schedule computed at
// set-up, which also checks that no level can wait for a copy not yet
// issued.  A level costs shared-memory latency plus one barrier; the width
// of the rows is a template parameter of each sweep direction's loop.  Every
// mbarrier wait is bounded (about one second of clock cycles); on expiry
// the CTA records an error word, waits (bounded again) for the copies it
// issued, and returns without touching the output.
#include <algorithm>
#include <type_traits>

#include "dev_common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace sg {

namespace {

constexpr int SW_T = 512;
template <class TS, bool EXACT>
__device__ __forceinline__ TS sub_mul(TS acc, TS a, TS b);
template <>
__device__ __forceinline__ double sub_mul<double, true>(double acc, double a, double b) {
    return __dsub_rn(acc, __dmul_rn(a, b));
}
template <>
__device__ __forceinline__ double sub_mul<double, false>(double acc, double a, double b) {
    return fma(-a, b, acc);
}
template <>
__device__ __forceinline__ float sub_mul<float, true>(float acc, float a, float b) {
    return fmaf(-a, b, acc);
}
template <>
__device__ __forceinline__ float sub_mul<float, false>(float acc, float a, float b) {
    return fmaf(-a, b, acc);
}

template <class TF>
__device__ __forceinline__ TF to_factor(double v);
template <>
__device__ __forceinline__ double to_factor<double>(double v) { return v; }
template <>
__device__ __forceinline__ float to_factor<float>(double v) { return (float)v; }
template <>
__device__ __forceinline__ uint16_t to_factor<uint16_t>(double v) {
    return __bfloat16_as_ushort(__float2bfloat16_rn((float)v));
}

// ---- shared-memory accesses by 32-bit shared-window address.  The level
// loop's row updates are chains of dependent shared-memory loads; explicit
// 32-bit addressing keeps the address arithmetic between them short.
__device__ __forceinline__ uint32_t lds_u16(uint32_t a) {
    uint16_t v;
    asm volatile("ld.shared.u16 %0, [%1];" : "=h"(v) : "r"(a) : "memory");
    return v;
}
template <class T>
__device__ __forceinline__ T lds(uint32_t a);
template <>
__device__ __forceinline__ float lds<float>(uint32_t a) {
    float v;
    asm volatile("ld.shared.f32 %0, [%1];" : "=f"(v) : "r"(a) : "memory");
    return v;
}
template <>
__device__ __forceinline__ double lds<double>(uint32_t a) {
    double v;
    asm volatile("ld.shared.f64 %0, [%1];" : "=d"(v) : "r"(a) : "memory");
    return v;
}
template <>
__device__ __forceinline__ uint16_t lds<uint16_t>(uint32_t a) {
    return (uint16_t)lds_u16(a);
}
__device__ __forceinline__ void sts(uint32_t a, float v) {
    asm volatile("st.shared.f32 [%0], %1;" ::"r"(a), "f"(v) : "memory");
}
__device__ __forceinline__ void sts(uint32_t a, double v) {
    asm volatile("st.shared.f64 [%0], %1;" ::"r"(a), "d"(v) : "memory");
}

// The rows of one level record with W nonzeros per row (W fixed: the 5-, 7-
// and 9-point stencils give 2, 3 and 4).  Record at shared address R:
//   rows u16[C] | columns u16[W][C] | values TF[W][C] | (diagonal TF[C]).
// A row computes acc = t[r]; acc -= v_k t[c_k] for k = 0..W-1 in order;
// backward: acc /= d -- every load of the row issued before the first
// multiply-add.  Row and column entries are shared-memory slots of t
// (tslot); padding entries hold the slot of row n, where t is 0, and value 0.
template <int W, bool BACK, class TS, class TF, bool EXACT>
__device__ __forceinline__ void level_rows_w(uint32_t tb, uint32_t R, int C, int c, int nthreads) {
    constexpr uint32_t SF = sizeof(TF), ST = sizeof(TS);
    const uint32_t cstride = 2u * (uint32_t)C;
    const uint32_t vbase = R + cstride * (uint32_t)(1 + W);
    const uint32_t vstride = SF * (uint32_t)C;
    for (int q = threadIdx.x; q < c; q += nthreads) {
        const uint32_t rq = R + 2u * (uint32_t)q;
        const uint32_t vq = vbase + SF * (uint32_t)q;
        const uint32_t r = lds_u16(rq);
        uint32_t ck[W];
        TF vk[W];
#pragma unroll
        for (int k = 0; k < W; ++k) ck[k] = lds_u16(rq + cstride * (uint32_t)(k + 1));
#pragma unroll
        for (int k = 0; k < W; ++k) vk[k] = lds<TF>(vq + vstride * (uint32_t)k);
        TF dg{};
        if (BACK) dg = lds<TF>(vq + vstride * (uint32_t)W);
        TS acc = lds<TS>(tb + ST * r);
        TS xk[W];
#pragma unroll
        for (int k = 0; k < W; ++k) xk[k] = lds<TS>(tb + ST * ck[k]);
#pragma unroll
        for (int k = 0; k < W; ++k) acc = sub_mul<TS, EXACT>(acc, Load<TS>::f(vk[k]), xk[k]);
        if (BACK) acc = div_diag(acc, Load<TS>::f(dg));
        sts(tb + ST * r, acc);
    }
}

// Any width w: the same row computation through generic pointers, the loads
// of four nonzeros at a time.
template <class TS, class TF, bool EXACT>
__device__ __forceinline__ void level_rows_any(TS* t, const unsigned char* R, int C, int c,
                                               int w, bool back, int nthreads) {
    const uint16_t* rr = reinterpret_cast<const uint16_t*>(R);
    const uint16_t* cc = rr + C;
    const TF* vv = reinterpret_cast<const TF*>(cc + (size_t)C * w);
    for (int q = threadIdx.x; q < c; q += nthreads) {
        const int r = rr[q];
        TS acc = t[r];
        for (int k0 = 0; k0 < w; k0 += 4) {
            int ci[4];
            TF vi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int o = (k0 + u < w ? k0 + u : k0) * C + q;
                ci[u] = cc[o];
                vi[u] = vv[o];
            }
            TS xi[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) xi[u] = t[ci[u]];
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (k0 + u < w) acc = sub_mul<TS, EXACT>(acc, Load<TS>::f(vi[u]), xi[u]);
        }
        if (back) acc = div_diag(acc, Load<TS>::f(vv[w * C + q]));
        t[r] = acc;
    }
}

// One level: the fixed-width row code for w = 2, 3, 4, else the generic one
// (t / t_s: the subdomain vector as generic pointer / shared address; R /
// R_s: the level record likewise).
template <class TS, class TF, bool EXACT>
__device__ __forceinline__ void level_rows(TS* t, uint32_t t_s, const unsigned char* R,
                                           uint32_t R_s, int C, int c, int w, bool back,
                                           int nthreads) {
    switch (w) {
    case 2:
        if (back) level_rows_w<2, true, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        else level_rows_w<2, false, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        return;
    case 3:
        if (back) level_rows_w<3, true, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        else level_rows_w<3, false, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        return;
    case 4:
        if (back) level_rows_w<4, true, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        else level_rows_w<4, false, TS, TF, EXACT>(t_s, R_s, C, c, nthreads);
        return;
    default:
        level_rows_any<TS, TF, EXACT>(t, R, C, c, w, back, nthreads);
    }
}

// Factored local CSR (FP64, reference layout) -> level records of type TF.
template <class TF>
__global__ void __launch_bounds__(256)
k_pack_rec(const SubInfo* __restrict__ info, const int* __restrict__ lrp,
           const int* __restrict__ lci, const int* __restrict__ ldiag,
           const double* __restrict__ lu, const uint16_t* __restrict__ perm_f,
           const uint16_t* __restrict__ perm_b, const int* __restrict__ lev_f,
           const int* __restrict__ lev_b, const long long* __restrict__ off_f,
           const long long* __restrict__ off_b, const int* __restrict__ rows_f,
           const int* __restrict__ rows_b, unsigned char* rec) {
    const SubInfo inf = info[blockIdx.x];
    const int* rp = lrp + inf.csr_row_off;
    const int* ci = lci + inf.csr_nz_off;
    const double* v = lu + inf.csr_nz_off;
    const int* dg = ldiag + inf.row_off;
    for (int l = 0; l < inf.nlev_f; ++l) {
        const int p0 = lev_f[inf.lev_off_f + l], c = lev_f[inf.lev_off_f + l + 1] - p0;
        const int C = rows_f[inf.lev_off_f + l];
        unsigned char* R = rec + off_f[inf.lev_off_f + l];
        uint16_t* rr = reinterpret_cast<uint16_t*>(R);
        uint16_t* cc = rr + C;
        TF* vv = reinterpret_cast<TF*>(cc + (size_t)C * inf.wl);
        for (int q = threadIdx.x; q < C; q += blockDim.x) {
            int k = 0;
            if (q < c) {
                const int r = perm_f[inf.row_off + p0 + q];
                rr[q] = (uint16_t)tslot(r, inf.tshift);
                for (int e = rp[r]; e < rp[r + 1] && k < inf.wl; ++e) {
                    const int col = ci[e];
                    if (col >= r) break;
                    cc[(size_t)k * C + q] = (uint16_t)tslot(col, inf.tshift);
                    vv[(size_t)k * C + q] = to_factor<TF>(v[e]);
                    ++k;
                }
            } else {
                rr[q] = 0;
            }
            for (; k < inf.wl; ++k) {
                cc[(size_t)k * C + q] = (uint16_t)tslot(inf.n, inf.tshift);
                vv[(size_t)k * C + q] = to_factor<TF>(0.0);
            }
        }
    }
    for (int l = 0; l < inf.nlev_b; ++l) {
        const int p0 = lev_b[inf.lev_off_b + l], c = lev_b[inf.lev_off_b + l + 1] - p0;
        const int C = rows_b[inf.lev_off_b + l];
        unsigned char* R = rec + off_b[inf.lev_off_b + l];
        uint16_t* rr = reinterpret_cast<uint16_t*>(R);
        uint16_t* cc = rr + C;
        TF* vv = reinterpret_cast<TF*>(cc + (size_t)C * inf.wu);
        TF* dd = vv + (size_t)C * inf.wu;
        for (int q = threadIdx.x; q < C; q += blockDim.x) {
            int k = 0;
            if (q < c) {
                const int r = perm_b[inf.row_off + p0 + q];
                rr[q] = (uint16_t)tslot(r, inf.tshift);
                for (int e = dg[r] + 1; e < rp[r + 1] && k < inf.wu; ++e) {
                    cc[(size_t)k * C + q] = (uint16_t)tslot(ci[e], inf.tshift);
                    vv[(size_t)k * C + q] = to_factor<TF>(v[e]);
                    ++k;
                }
                dd[q] = to_factor<TF>(v[dg[r]]);
            } else {
                rr[q] = 0;
                dd[q] = to_factor<TF>(1.0);
            }
            for (; k < inf.wu; ++k) {
                cc[(size_t)k * C + q] = (uint16_t)tslot(inf.n, inf.tshift);
                vv[(size_t)k * C + q] = to_factor<TF>(0.0);
            }
        }
    }
}

// ---- R right-hand sides at once (FP32 sweeps): the shared vector holds R
// interleaved floats per slot, so every level record is read once for all of
// them; the row arithmetic per right-hand side is the single-vector code's.
template <int R>
struct FVec;
template <>
struct FVec<2> {
    __device__ __forceinline__ static void ld(uint32_t a, float (&v)[2]) {
        asm volatile("ld.shared.v2.f32 {%0,%1}, [%2];" : "=f"(v[0]), "=f"(v[1]) : "r"(a) : "memory");
    }
    __device__ __forceinline__ static void st(uint32_t a, const float (&v)[2]) {
        asm volatile("st.shared.v2.f32 [%0], {%1,%2};" ::"r"(a), "f"(v[0]), "f"(v[1]) : "memory");
    }
};
template <>
struct FVec<4> {
    __device__ __forceinline__ static void ld(uint32_t a, float (&v)[4]) {
        asm volatile("ld.shared.v4.f32 {%0,%1,%2,%3}, [%4];"
                     : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3])
                     : "r"(a)
                     : "memory");
    }
    __device__ __forceinline__ static void st(uint32_t a, const float (&v)[4]) {
        asm volatile("st.shared.v4.f32 [%0], {%1,%2,%3,%4};" ::"r"(a), "f"(v[0]), "f"(v[1]),
                     "f"(v[2]), "f"(v[3])
                     : "memory");
    }
};

// W > 0: rows with W nonzeros per triangle; W = 0: any width w
template <int W, bool BACK, class TF, int R>
__device__ __forceinline__ void level_rows_mr(uint32_t tb, uint32_t Rr, int C, int c, int w,
                                              int nthreads) {
    constexpr uint32_t SF = sizeof(TF), ST = 4u * R;
    const int ww = W > 0 ? W : w;
    const uint32_t cstride = 2u * (uint32_t)C;
    const uint32_t vbase = Rr + cstride * (uint32_t)(1 + ww);
    const uint32_t vstride = SF * (uint32_t)C;
    for (int q = threadIdx.x; q < c; q += nthreads) {
        const uint32_t rq = Rr + 2u * (uint32_t)q;
        const uint32_t vq = vbase + SF * (uint32_t)q;
        const uint32_t r = lds_u16(rq);
        float acc[R];
        FVec<R>::ld(tb + ST * r, acc);
        if constexpr (W > 0) {
            uint32_t ck[W];
            TF vk[W];
#pragma unroll
            for (int k = 0; k < W; ++k) ck[k] = lds_u16(rq + cstride * (uint32_t)(k + 1));
#pragma unroll
            for (int k = 0; k < W; ++k) vk[k] = lds<TF>(vq + vstride * (uint32_t)k);
            float xk[W][R];
#pragma unroll
            for (int k = 0; k < W; ++k) FVec<R>::ld(tb + ST * ck[k], xk[k]);
#pragma unroll
            for (int k = 0; k < W; ++k) {
                const float v = Load<float>::f(vk[k]);
#pragma unroll
                for (int i = 0; i < R; ++i) acc[i] = fmaf(-v, xk[k][i], acc[i]);
            }
        } else {
            for (int k = 0; k < ww; ++k) {
                const uint32_t ci = lds_u16(rq + cstride * (uint32_t)(k + 1));
                const float v = Load<float>::f(lds<TF>(vq + vstride * (uint32_t)k));
                float xv[R];
                FVec<R>::ld(tb + ST * ci, xv);
#pragma unroll
                for (int i = 0; i < R; ++i) acc[i] = fmaf(-v, xv[i], acc[i]);
            }
        }
        if (BACK) {
            const float rd = 1.0f / Load<float>::f(lds<TF>(vq + vstride * (uint32_t)ww));
#pragma unroll
            for (int i = 0; i < R; ++i) acc[i] = acc[i] * rd;
        }
        FVec<R>::st(tb + ST * r, acc);
    }
}

// ---- the gather and the restricted scatter of the TMA-fed sweep.  Rows are
// spread over the threads (consecutive rows on consecutive lanes, so index
// loads, element copies and stores stay coalesced) and each thread keeps
// SW_ILP index loads in flight: a cold gather or scatter of ~9,000 rows
// costs two or three memory round trips.  With R right-hand sides, element
// i of row li sits at x[i * ldx + dof[li]] and in slot component i.
__device__ __forceinline__ void cp_async4(uint32_t dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async8(uint32_t dst, const void* src) {
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.wait_all;" ::: "memory");
}
template <class T>
__device__ __forceinline__ void cp_async_elt(uint32_t dst, const T* src) {
    if constexpr (sizeof(T) == 8) cp_async8(dst, src);
    else cp_async4(dst, src);
}

constexpr int SW_ILP = 16;

// input of the sweep's own type: every element copied global -> shared by
// cp.async (no register holds a value, so all of a thread's copies stay in
// flight); the caller waits with cp_async_wait_all
template <class T, int R>
__device__ __forceinline__ void gather_async(uint32_t t_s, const T* __restrict__ x,
                                             long long ldx, const int* __restrict__ dof, int n,
                                             int bs, int p) {
    constexpr int U = sizeof(T) == 8 ? SW_ILP / 2 : SW_ILP;
    for (int li = threadIdx.x; li < n; li += U * bs) {
        int d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) d[u] = li + u * bs < n ? __ldg(dof + li + u * bs) : -1;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (d[u] >= 0) {
                const uint32_t slot = t_s + (uint32_t)(sizeof(T) * R * tslot(li + u * bs, p));
#pragma unroll
                for (int i = 0; i < R; ++i)
                    cp_async_elt<T>(slot + (uint32_t)(sizeof(T) * i), x + i * ldx + d[u]);
            }
    }
}

// other input types convert through registers
template <class TS, class TI, int R>
__device__ __forceinline__ void gather_convert(TS* t, const TI* __restrict__ x, long long ldx,
                                               const int* __restrict__ dof, int n, int bs, int p) {
    // values in flight per thread (U x R inputs held in registers)
    constexpr int U = R > 1 ? 2 : (sizeof(TI) == 8 ? 4 : 8);
    for (int li = threadIdx.x; li < n; li += U * bs) {
        int d[U];
#pragma unroll
        for (int u = 0; u < U; ++u) d[u] = li + u * bs < n ? __ldg(dof + li + u * bs) : -1;
        TI v[U][R];
#pragma unroll
        for (int u = 0; u < U; ++u)
#pragma unroll
            for (int i = 0; i < R; ++i) v[u][i] = d[u] >= 0 ? x[i * ldx + d[u]] : (TI)0;
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (d[u] >= 0)
#pragma unroll
                for (int i = 0; i < R; ++i)
                    t[(size_t)R * tslot(li + u * bs, p) + i] = Load<TS>::f(v[u][i]);
    }
}

// y[i * ldy + og[q]] = t[tslot(ol[q])][i] (+ the coarse term), q < n_own
template <class TS, class TO, int R>
__device__ __forceinline__ void scatter_ilp(const TS* t, TO* __restrict__ y, long long ldy,
                                            const int* __restrict__ ol, const int* __restrict__ og,
                                            int n_own, int coarse, double zc, int bs, int p) {
    const CoarseAdd<TO> add(zc);
    constexpr int U = sizeof(TO) == 8 ? SW_ILP / 2 : SW_ILP;
    for (int q = threadIdx.x; q < n_own; q += U * bs) {
        int l[U], g[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool in = q + u * bs < n_own;
            l[u] = in ? __ldg(ol + q + u * bs) : -1;
            g[u] = in ? __ldg(og + q + u * bs) : 0;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (l[u] >= 0) {
#pragma unroll
                for (int i = 0; i < R; ++i) {
                    const TS v = t[(size_t)R * tslot(l[u], p) + i];
                    y[i * ldy + g[u]] = coarse ? add(v) : Store<TO>::f(v);
                }
            }
    }
}

// Static schedule of one subdomain's record stream through the ring: the
// stream (forward records, then backward, contiguous from `base` in the
// packed array) is cut into groups of whole levels, each copied by one
// cp.async.bulk into a fixed ring position and tracked by mbarrier
// (group % RING_NBAR).  Per level (int4): x = rows | padded rows << 16, y =
// the record's byte offset in the ring, z = the group whose copy the level
// waits for (its first level; -1 otherwise), w = the groups that may have
// been issued once the level is done.  Per group (int2): x = stream offset,
// y = bytes / 16 | ring position / 16 << 16.
struct RingSub {
    long long base;
    int meta_off, grp_off, ngrp, ninit;
};
constexpr int RING_LOG_NBAR = 5;
constexpr int RING_NBAR = 1 << RING_LOG_NBAR;

struct RecArgs {
    const SubInfo* info;
    const int* order;
    const int* dofs;
    const RingSub* ring;
    const int4* meta;
    const int2* grp;
    const unsigned char* rec;
    const int* ownloc;
    const int* owned;
    const double* a0inv;
    const double* r0;
    int nparts;
    int nc;
    int a0pre;       // 1: the coarse row a0inv[s] is prefetched into shared memory
    int ring_bytes;  // bytes of the record ring
    int t_len;       // slots of the subdomain vector region (largest tslot(n) + 1)
    int max_levels;  // largest nlev_f + nlev_b over the subdomains
    long long ldx, ldy;  // distance between right-hand sides (R > 1)
    int* err;
    // optional per-subdomain switches, one array of nparts per right-hand
    // side (0: skipped; a subdomain runs when any of its R switches is on)
    const int* sub_on;
    // persistent launch: CTAs take subdomains (in `order`) from work[0];
    // work[1] counts the CTAs that are done, and the last one resets both
    int persist;
    unsigned* work;
    // coarse restriction fused into the sweep (cooperative launch, all blocks
    // resident): each block writes r0[s] and counts itself in sync[0]; sync[1]
    // counts the blocks done with r0 (the last one resets both)
    int fuse;
    double* r0w;
    unsigned* sync;
    // bounded waits: cycle budget of the record and restriction waits, and
    // the test mode that makes one of them run out without any fault
    // (1: record group 0 is never copied; 2: no restriction is counted)
    long long wait_budget;
    int wait_test;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// The ring side of the level loop.  Set-up has checked that every group is
// issued (after the level its schedule names) before its first level waits
// for it, and that a group re-arms an mbarrier or overwrites ring bytes only
// after every thread has observed, and finished with, the group before it.
//
// A wait that gives up marks the thread (bad: it computes no more rows) and
// the block: the shared word fail takes the failing level + 1.  Every thread
// reads it when it next opens a group and acts only on a failure at an
// earlier level -- written before a barrier it has passed, so all threads
// see it and leave at the same level, while a failure being recorded at the
// current level by a faster thread is left for the next group -- and once
// more after the last level.
struct RecRing {
    const unsigned char* src;
    const int2* grp;       // shared memory
    volatile int* fail;    // shared memory
    uint32_t bars_s, ring_s;
    long long budget;
    int gbase;     // groups this CTA streamed for earlier subdomains: group j
                   // of this one uses mbarrier (gbase + j) % RING_NBAR with
                   // phase parity ((gbase + j) / RING_NBAR) & 1
    int issued;    // producer: groups issued
    int observed;  // groups this thread has seen complete
    bool producer, bad;
    int wait_test;

    __device__ __forceinline__ uint32_t bar(int j) const {
        return bars_s + 8u * (uint32_t)((gbase + j) & (RING_NBAR - 1));
    }
    __device__ __forceinline__ uint32_t parity(int j) const {
        return (uint32_t)((gbase + j) >> RING_LOG_NBAR) & 1u;
    }
    __device__ __forceinline__ void issue_to(int limit) {
        if (issued >= limit) return;
        fence_proxy_async();  // the ring bytes it overwrites were read by the generic proxy
        do {
            const int2 gi = grp[issued];
            const uint32_t bytes = ((uint32_t)gi.y & 0xffffu) << 4;
            const uint32_t pos = ((uint32_t)gi.y >> 16) << 4;
            if (!(wait_test == 1 && issued == 0)) {
                mbar_expect_tx(bar(issued), bytes);
                bulk_g2s_stream(ring_s + pos, src + (uint32_t)gi.x, bytes, bar(issued));
            }
        } while (++issued < limit);
    }
    // the first try costs one mbarrier probe; the bounded loop (which reads
    // the clock) runs only when the copy has not landed yet
    __device__ __forceinline__ void wait_group(int j, int level) {
        const uint32_t par = parity(j);
        if (mbar_try(bar(j), par) || mbar_wait(bar(j), par, budget)) {
            observed = j + 1;
        } else {
            bad = true;
            *fail = level + 1;
        }
    }
    // the block leaves after a wait gave up: the producer waits (full budget
    // each) for the copies it issued that it has not seen land, so none
    // lands after the block has left; if one still does not arrive -- only
    // possible when a copy never lands at all -- the error word says 2
    __device__ void drain(int* err) const {
        if (!producer) return;
        int code = 1;
        for (int k = observed; k < issued; ++k) {
            if (wait_test == 1 && k == 0) continue;
            if (!mbar_wait(bar(k), parity(k), WAIT_CYCLES)) code = 2;
        }
        atomicMax(err, code);
    }
};

// One sweep direction: levels [g0, g1), rows with W nonzeros per triangle
// (W = 0: any width w).  Per level: the wait for the level's group when it
// opens one, the rows, one barrier, then the producer issues the groups the
// schedule allows.  The next level's metadata loads while this one
// computes.  Returns false when the block leaves because a group did not
// arrive within the wait budget.
template <int W, bool BACK, class TS, class TF, bool EXACT, int R>
__device__ __forceinline__ bool level_loop(const int4* meta, int g0, int g1, int T, int w,
                                           RecRing& ring, TS* t, uint32_t t_s,
                                           unsigned char* ring_g, int NC, int* err) {
    if (g0 >= g1) return true;
    int4 md = meta[g0];
    for (int g = g0; g < g1; ++g) {
        int4 mn = md;
        if (g + 1 < T) mn = meta[g + 1];
        if (md.z >= 0) {
            const int f = *ring.fail;
            if (f != 0 && f <= g) {  // a wait at an earlier level gave up
                ring.drain(err);
                return false;
            }
            ring.wait_group(md.z, g);
        }
        if (!ring.bad) {
            const int c = md.x & 0xffff, C = (int)((unsigned)md.x >> 16);
            if constexpr (R > 1)
                level_rows_mr<W, BACK, TF, R>(t_s, ring.ring_s + (uint32_t)md.y, C, c, w, NC);
            else if constexpr (W > 0)
                level_rows_w<W, BACK, TS, TF, EXACT>(t_s, ring.ring_s + (uint32_t)md.y, C, c, NC);
            else
                level_rows_any<TS, TF, EXACT>(t, ring_g + md.y, C, c, w, BACK, NC);
        }
        __syncthreads();
        if (ring.producer) ring.issue_to(md.w);
        md = mn;
    }
    return true;
}

template <bool BACK, class TS, class TF, bool EXACT, int R>
__device__ __forceinline__ bool level_loop_w(const int4* meta, int g0, int g1, int T, int w,
                                             RecRing& ring, TS* t, uint32_t t_s,
                                             unsigned char* ring_g, int NC, int* err) {
    switch (w) {
    case 2: return level_loop<2, BACK, TS, TF, EXACT, R>(meta, g0, g1, T, w, ring, t, t_s, ring_g, NC, err);
    case 3: return level_loop<3, BACK, TS, TF, EXACT, R>(meta, g0, g1, T, w, ring, t, t_s, ring_g, NC, err);
    case 4: return level_loop<4, BACK, TS, TF, EXACT, R>(meta, g0, g1, T, w, ring, t, t_s, ring_g, NC, err);
    default: return level_loop<0, BACK, TS, TF, EXACT, R>(meta, g0, g1, T, w, ring, t, t_s, ring_g, NC, err);
    }
}

// The shared memory of one CTA of the sweep.
struct SweepSmem {
    unsigned char* raw;   // RING_NBAR mbarriers, then the ring
    unsigned char* ring;  // ring_bytes
    void* t;              // t_len slots of R elements
    int4* meta;           // max_levels
    int2* grp;            // max_levels
    double* a0row;        // nc (a0pre)
};

// One subdomain: stage its schedule, start its record stream, gather its
// right-hand side(s) (and, in the fused two-level mode, the coarse
// restrictions this block owes), run both sweeps, add the coarse term and
// write the owned rows.  Returns false when the block must leave (a bounded
// wait gave up; the error word is set).
template <class TI, class TO, class TS, class TF, bool EXACT, int R>
__device__ __forceinline__ bool sweep_one(const RecArgs& a, int s, const TI* __restrict__ x,
                                          TO* __restrict__ y, int mode, int coarse,
                                          const SweepSmem& sm, int& gbase, bool first) {
    __shared__ double s_zc;
    __shared__ double s_red[RC_MAXCH];
    __shared__ int s_ok;
    __shared__ int s_fail;
    const int NC = (int)blockDim.x;
    TS* t = reinterpret_cast<TS*>(sm.t);
    const SubInfo inf = a.info[s];
    const RingSub rs = a.ring[s];
    const int n = inf.n;
    const int nf = inf.nlev_f, T = inf.nlev_f + inf.nlev_b;
    // the schedule, staged once (the level loop touches global memory only
    // through the ring)
    for (int g = threadIdx.x; g < T; g += NC) sm.meta[g] = a.meta[rs.meta_off + g];
    for (int j = threadIdx.x; j < rs.ngrp; j += NC) sm.grp[j] = a.grp[rs.grp_off + j];

    RecRing ring;
    ring.src = a.rec + rs.base;
    ring.grp = sm.grp;
    ring.bars_s = smem_u32(sm.raw);
    ring.ring_s = smem_u32(sm.ring);
    ring.budget = a.wait_budget;
    ring.fail = &s_fail;
    ring.gbase = gbase;
    ring.issued = 0;
    ring.observed = 0;
    ring.bad = false;
    ring.wait_test = a.wait_test;
    // the producer is the block's last thread: levels rarely have rows for
    // it, so its copies overlap the other threads' work.  The mbarriers are
    // initialised with the CTA's first subdomain; later ones continue their
    // phases (every group of the previous subdomain was issued and observed).
    ring.producer = threadIdx.x == blockDim.x - 1;
    if (ring.producer) {
        if (first)
            for (int i = 0; i < RING_NBAR; ++i) mbar_init(ring.bars_s + 8u * (uint32_t)i, 1);
        fence_mbar_init();
        s_fail = 0;
    }
    gbase += rs.ngrp;
    __syncthreads();
    if (ring.producer) ring.issue_to(rs.ninit);
    // gather while the first records are in flight; with a coarse term the
    // subdomain's row of the coarse inverse comes into shared memory with it
    const int* dof = a.dofs + inf.row_off;
    const int tp = inf.tshift;
    if (coarse && a.a0pre && threadIdx.x < 32) {
        const double* row = a.a0inv + (size_t)s * a.nc;
        for (int q = threadIdx.x; q < a.nc; q += 32) cp_async8(smem_u32(sm.a0row + q), row + q);
    }
    if constexpr (std::is_same<TI, TS>::value) {
        gather_async<TS, R>(smem_u32(t), x, a.ldx, dof, n, NC, tp);
    } else {
        gather_convert<TS, TI, R>(t, x, a.ldx, dof, n, NC, tp);
    }
    cp_async_wait_all();
    if (threadIdx.x < R) t[(size_t)R * tslot(n, tp) + threadIdx.x] = (TS)0;
    if (coarse && a.fuse && (int)blockIdx.x >= (int)gridDim.x / 2) {
        // coarse restrictions (the order of k_restrict), published for the
        // other blocks before the level loop.  Blocks run largest subdomain
        // first, so the second half -- the smaller subdomains, with slack --
        // computes its own and its mirror block's, and the critical first
        // half computes none.
        const int mirror = (int)gridDim.x - 1 - (int)blockIdx.x;
        for (int pass = 0; pass < (mirror == (int)blockIdx.x ? 1 : 2); ++pass) {
            const int sr = pass == 0 ? s : a.order[mirror];
            const SubInfo ir = pass == 0 ? inf : a.info[sr];
            const double z = restrict_chunks<TI>(a.owned + ir.own_off, x, ir.n_own, s_red);
            if (threadIdx.x == 0) {
                a.r0w[sr] = ir.cscale * z;
                __threadfence();
                if (a.wait_test != 2) atomicAdd(&a.sync[0], 1u);
            }
        }
    }
    __syncthreads();

    // the level loop -- the latency chain of the sweep -- one direction at a
    // time, specialised on the row width
    const uint32_t t_s = smem_u32(t);
    if (!level_loop_w<false, TS, TF, EXACT, R>(sm.meta, 0, nf, T, inf.wl, ring, t, t_s, sm.ring,
                                               NC, a.err))
        return false;
    if (!level_loop_w<true, TS, TF, EXACT, R>(sm.meta, nf, T, T, inf.wu, ring, t, t_s, sm.ring,
                                              NC, a.err))
        return false;
    if (s_fail) {  // a wait in the last group gave up (read after the last level's barrier)
        ring.drain(a.err);
        return false;
    }

    if (coarse) {
        if (a.fuse) {
            // every block published its restriction before its level loop;
            // all blocks are resident (cooperative launch), so this bounded
            // wait ends as soon as the slowest block got there
            if (threadIdx.x == 0) {
                const long long t0 = clock64();
                int ok = 1;
                while (ld_acquire(&a.sync[0]) < gridDim.x) {
                    if (clock64() - t0 > a.wait_budget) {
                        ok = 0;
                        break;
                    }
                    __nanosleep(64);
                }
                s_ok = ok;
            }
            __syncthreads();
            if (!s_ok) {
                if (threadIdx.x == 0) atomicMax(a.err, 1);
                return false;
            }
        }
        if (threadIdx.x < 32) {
            const double* row = a.a0pre ? sm.a0row : a.a0inv + (size_t)s * a.nc;
            const double z = a.fuse ? coarse_dot_warp0<true>(row, a.r0, a.nc)
                                    : coarse_dot_warp0<false>(row, a.r0, a.nc);
            if (threadIdx.x == 0) {
                s_zc = inf.cscale * z;
                // the last block done with r0 resets the counters
                if (a.fuse && atomicAdd(&a.sync[1], 1u) == gridDim.x - 1) {
                    a.sync[0] = 0u;
                    a.sync[1] = 0u;
                }
            }
        }
        __syncthreads();
    }
    const double zc = coarse ? s_zc : 0.0;
    if (mode == 0) {
        scatter_ilp<TS, TO, R>(t, y, a.ldy, a.ownloc + inf.own_off, a.owned + inf.own_off,
                               inf.n_own, coarse, zc, NC, tp);
    } else {
        for (int li = threadIdx.x; li < n; li += NC)
#pragma unroll
            for (int i = 0; i < R; ++i)
                atomicAdd(&y[i * a.ldy + dof[li]], Store<TO>::f(t[(size_t)R * tslot(li, tp) + i]));
        if (coarse) {
            const int* og = a.owned + inf.own_off;
            for (int q = threadIdx.x; q < inf.n_own; q += NC)
                atomicAdd(&y[og[q]], Store<TO>::f(zc));
        }
    }
    return true;
}

// mode 0: RAS (owned rows written), 1: ASM (all rows added atomically).  One
// subdomain per CTA, or (PERSIST) CTAs looping over subdomains taken largest
// first from a work counter.
template <class TI, class TO, class TS, class TF, bool EXACT, int R, bool PERSIST>
__global__ void __launch_bounds__(SW_T, 2)
k_sweep_tma(RecArgs a, const TI* __restrict__ x, TO* __restrict__ y, int mode, int coarse,
            const int* __restrict__ active) {
    if (active && *active == 0) return;
    extern __shared__ __align__(128) unsigned char smraw[];
    constexpr uint32_t HDR = RING_NBAR * 8;
    SweepSmem sm;
    sm.raw = smraw;
    sm.ring = smraw + HDR;
    sm.t = sm.ring + a.ring_bytes;
    sm.meta = reinterpret_cast<int4*>(reinterpret_cast<unsigned char*>(sm.t) +
                                      (((size_t)a.t_len * R * sizeof(TS) + 15) & ~(size_t)15));
    sm.grp = reinterpret_cast<int2*>(sm.meta + a.max_levels);
    sm.a0row = reinterpret_cast<double*>(sm.grp + a.max_levels);
    auto on = [&](int s) {
        if (!a.sub_on) return true;
        bool v = false;
#pragma unroll
        for (int i = 0; i < R; ++i) v = v || a.sub_on[(size_t)i * a.nparts + s] != 0;
        return v;
    };
    int gbase = 0;  // record groups this CTA has streamed (mbarrier phases)
    if constexpr (!PERSIST) {
        const int s = a.order[blockIdx.x];
        if (!on(s)) return;  // subdomain not needed by this apply
        sweep_one<TI, TO, TS, TF, EXACT, R>(a, s, x, y, mode, coarse, sm, gbase, true);
    } else {
        __shared__ int s_next;
        bool first = true;
        for (;;) {
            __syncthreads();  // every thread has read the previous index
            if (threadIdx.x == 0) s_next = (int)atomicAdd(&a.work[0], 1u);
            __syncthreads();
            const int idx = s_next;
            if (idx >= a.nparts) break;
            const int s = a.order[idx];
            if (!on(s)) continue;
            if (!sweep_one<TI, TO, TS, TF, EXACT, R>(a, s, x, y, mode, coarse, sm, gbase, first))
                return;
            first = false;
        }
        if (threadIdx.x == 0 && atomicAdd(&a.work[1], 1u) == gridDim.x - 1) {
            a.work[0] = 0u;  // every CTA has taken its last index: the counters restart
            a.work[1] = 0u;
        }
    }
}

bool sweep_a0_prefetch(const sg_precond* pc);

RecArgs rec_args(sg_precond* pc, const RingPlan& plan, bool fuse) {
    RecArgs a;
    a.fuse = fuse ? 1 : 0;
    a.r0w = pc->r0.p;
    a.sync = pc->coarse_sync.p;
    a.info = pc->info.p;
    a.order = pc->order.p;
    a.dofs = pc->dofs.p;
    a.ring = reinterpret_cast<const RingSub*>(plan.sub_d.p);
    a.meta = reinterpret_cast<const int4*>(plan.meta_d.p);
    a.grp = reinterpret_cast<const int2*>(plan.grp_d.p);
    a.rec = pc->rec_d.p;
    a.ownloc = pc->ownloc_d.p;
    a.owned = pc->owned_d.p;
    a.a0inv = pc->a0inv.p;
    a.r0 = pc->r0.p;
    a.nparts = pc->nparts;
    a.nc = pc->nc;
    a.a0pre = sweep_a0_prefetch(pc) ? 1 : 0;
    a.ring_bytes = (int)plan.ring_bytes;
    a.t_len = pc->t_len;
    a.max_levels = pc->max_levels;
    a.ldx = 0;
    a.ldy = 0;
    a.err = pc->err_d.p;
    a.sub_on = pc->sub_on;
    a.persist = (plan.grid > 0 && !fuse) ? 1 : 0;
    a.work = plan.work.p;
    a.wait_test = pc->wait_test;
    a.wait_budget = pc->wait_test ? WAIT_TEST_CYCLES : WAIT_CYCLES;
    return a;
}

// two-level preconditioners with at most 1024 subdomains keep the
// subdomain's row of the coarse inverse in shared memory
bool sweep_a0_prefetch(const sg_precond* pc) {
    return (pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS) &&
           pc->nparts <= 1024;
}

// dynamic shared memory of the sweep: the mbarriers, the record ring, the
// subdomain vector (R elements per slot), per-level and per-group schedule
// entries, the coarse row
size_t sweep_smem_for(const sg_precond* pc, long long ring_bytes, int R) {
    const size_t ts = pc->opts.sweep_dtype == SG_FP64 ? 8 : 4;
    const size_t tbytes = ((size_t)pc->t_len * ts * R + 15) & ~(size_t)15;
    const size_t a0 = sweep_a0_prefetch(pc) ? (size_t)pc->nparts * 8 : 0;
    return RING_NBAR * 8 + (size_t)ring_bytes + tbytes + (size_t)pc->max_levels * (16 + 8) + a0;
}
size_t sweep_smem(const sg_precond* pc, const RingPlan& plan) {
    return sweep_smem_for(pc, plan.ring_bytes, plan.R);
}

template <class TI, class TO, class TS, class TF, bool EXACT, int R>
void launch_tma(sg_precond* pc, const RingPlan& plan, const TI* x, TO* y, int mode, bool coarse,
                const int* active, bool fuse = false, long long ldx = 0, long long ldy = 0) {
    const size_t smem = sweep_smem(pc, plan);
    const int nt = plan.threads > 0 ? plan.threads : SW_T;
    RecArgs a = rec_args(pc, plan, fuse);
    // persistent CTAs only for FP32 sweeps (the FP64 ones keep their
    // registers for the level loop)
    if (sizeof(TS) == 8) a.persist = 0;
    auto kern = k_sweep_tma<TI, TO, TS, TF, EXACT, R, false>;
    if constexpr (sizeof(TS) == 4) {
        if (a.persist) kern = k_sweep_tma<TI, TO, TS, TF, EXACT, R, true>;
    }
    SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    a.ldx = ldx;
    a.ldy = ldy;
    const int coarse_i = coarse ? 1 : 0;
    if (fuse) {
        // the blocks wait for one another's restriction: co-residency is
        // guaranteed by the cooperative launch (checked at set-up)
        cudaLaunchConfig_t cfg = {};
        cfg.gridDim = dim3(pc->nparts);
        cfg.blockDim = dim3(nt);
        cfg.dynamicSmemBytes = smem;
        cfg.stream = pc->ctx->stream;
        cudaLaunchAttribute at[1];
        at[0].id = cudaLaunchAttributeCooperative;
        at[0].val.cooperative = 1;
        cfg.attrs = at;
        cfg.numAttrs = 1;
        SG_CUDA(cudaLaunchKernelEx(&cfg, kern, a, x, y, mode, coarse_i, active));
    } else {
        const int grid = a.persist ? plan.grid : pc->nparts;
        kern<<<grid, nt, smem, pc->ctx->stream>>>(a, x, y, mode, coarse_i, active);
    }
    SG_CUDA(cudaGetLastError());
    count_launch(pc->ctx);
}

}  // namespace

// Builds the static ring schedule of every subdomain (see RingSub) into
// `plan` for a ring of ring_bytes and groups of at most gmax bytes (a larger
// level is a group of its own).  Groups are placed one after another and
// start over at the ring's beginning when they would cross its end.  Group
// j may be issued after the last level of every earlier group whose ring
// bytes it overwrites and of group j - RING_NBAR (its mbarrier's previous
// user); the schedule is feasible when that is always before group j's
// first level.  Returns false (plan unchanged) when it is not.
static bool ring_schedule(const sg_precond* pc, RingPlan& plan, long long ring_bytes,
                          long long gmax) {
    const long long sf = pc->opts.sweep_dtype == SG_FP64 ? 8
                         : (pc->opts.factor_dtype == SG_BF16 ? 2 : 4);
    std::vector<RingSub> subs((size_t)pc->nparts);
    std::vector<int> meta, grp;  // int4 / int2 entries as ints
    std::vector<long long> rel, gstart, gbytes, gpos;
    std::vector<int> B, cnt, padded, gfirst, glast, ia;
    for (int s = 0; s < pc->nparts; ++s) {
        const SubInfo& inf = pc->h_info[s];
        const int nf = inf.nlev_f, T = inf.nlev_f + inf.nlev_b;
        rel.resize(T);
        B.resize(T);
        cnt.resize(T);
        padded.resize(T);
        for (int g = 0; g < T; ++g) {
            if (g < nf) {
                const int i = inf.lev_off_f + g;
                rel[g] = pc->h_rec_off_f[i];
                padded[g] = pc->h_rec_rows_f[i];
                cnt[g] = pc->h_lev_ptr_f[i + 1] - pc->h_lev_ptr_f[i];
                B[g] = (int)(padded[g] * (2 + inf.wl * (2 + sf)));
            } else {
                const int i = inf.lev_off_b + (g - nf);
                rel[g] = pc->h_rec_off_b[i];
                padded[g] = pc->h_rec_rows_b[i];
                cnt[g] = pc->h_lev_ptr_b[i + 1] - pc->h_lev_ptr_b[i];
                B[g] = (int)(padded[g] * (2 + inf.wu * (2 + sf) + sf));
            }
        }
        RingSub& r = subs[s];
        r.base = T > 0 ? rel[0] : 0;
        r.meta_off = (int)(meta.size() / 4);
        r.grp_off = (int)(grp.size() / 2);
        for (int g = 0; g < T; ++g) rel[g] -= r.base;
        // groups of whole levels
        gfirst.clear();
        glast.clear();
        gstart.clear();
        gbytes.clear();
        for (int g = 0; g < T; ++g) {
            if (gfirst.empty() || gbytes.back() + B[g] > gmax) {
                gfirst.push_back(g);
                glast.push_back(g);
                gstart.push_back(rel[g]);
                gbytes.push_back(B[g]);
            } else {
                glast.back() = g;
                gbytes.back() = rel[g] + B[g] - gstart.back();
            }
        }
        const int G = (int)gfirst.size();
        gpos.assign(G, 0);
        long long pos = 0;
        for (int j = 0; j < G; ++j) {
            if (gbytes[j] > ring_bytes || gbytes[j] >= (1ll << 20)) return false;
            if (pos + gbytes[j] > ring_bytes) pos = 0;
            gpos[j] = pos;
            pos += gbytes[j];
        }
        ia.assign(G, -1);
        int run = -1;
        for (int j = 0; j < G; ++j) {
            int v = -1;
            for (int i = std::max(0, j - RING_NBAR); i < j; ++i)
                if (gpos[i] < gpos[j] + gbytes[j] && gpos[j] < gpos[i] + gbytes[i])
                    v = std::max(v, glast[i]);
            if (j >= RING_NBAR) v = std::max(v, glast[j - RING_NBAR]);
            run = std::max(run, v);
            if (run >= gfirst[j]) return false;  // would wait for a copy not yet issued
            ia[j] = run;
        }
        int ninit = 0;
        while (ninit < G && ia[ninit] < 0) ++ninit;
        r.ngrp = G;
        r.ninit = ninit;
        int jg = 0, ji = 0;
        for (int g = 0; g < T; ++g) {
            while (jg + 1 < G && gfirst[jg + 1] <= g) ++jg;
            while (ji < G && ia[ji] <= g) ++ji;
            meta.push_back(cnt[g] | (padded[g] << 16));
            meta.push_back((int)(gpos[jg] + rel[g] - gstart[jg]));
            meta.push_back(gfirst[jg] == g ? jg : -1);
            meta.push_back(ji);
        }
        for (int j = 0; j < G; ++j) {
            grp.push_back((int)gstart[j]);
            grp.push_back((int)((gbytes[j] >> 4) | ((gpos[j] >> 4) << 16)));
        }
    }
    plan.sub.assign(reinterpret_cast<const unsigned char*>(subs.data()),
                    reinterpret_cast<const unsigned char*>(subs.data() + subs.size()));
    plan.meta.swap(meta);
    plan.grp.swap(grp);
    plan.ring_bytes = ring_bytes;
    plan.gmax = gmax;
    return true;
}

static void ring_upload(sg_precond* pc, RingPlan& plan) {
    cudaStream_t st = pc->ctx->stream;
    plan.sub_d.upload(plan.sub, st);
    plan.meta_d.upload(plan.meta, st);
    plan.grp_d.upload(plan.grp, st);
}

// Resident CTAs per SM of the sweep kernel for the plan's shared memory and
// block size.
template <class K>
static int sweep_occupancy(sg_precond* pc, const RingPlan& plan, K kern) {
    const size_t smem = sweep_smem(pc, plan);
    const int nt = plan.threads > 0 ? plan.threads : SW_T;
    int per_sm = 0;
    SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem));
    return per_sm;
}

// Sizes a plan's ring (what the shared memory of the CTAs that must share an
// SM leaves) and lists the record-group sizes whose schedule is feasible
// for it (the schedule of the last one is left in `plan`).
static std::vector<long long> ring_size(sg_precond* pc, RingPlan& plan) {
    sg_ctx* ctx = pc->ctx;
    int max_smem = 0, sm_smem = 0;
    SG_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                   ctx->device));
    SG_CUDA(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                   ctx->device));
    const int static_smem = 1024;  // reduction scratch and the like
    // CTAs per SM needed to keep every subdomain resident at once (more
    // subdomains than that run persistent or in waves)
    int want = (pc->nparts + ctx->num_sms - 1) / ctx->num_sms;
    if (want > 4) want = 4;
    // group size: opts.reserved[3] when set, else timed among 8 and 16 KB
    // (never below the largest record)
    std::vector<long long> gcand;
    if (pc->opts.reserved[3] > 0) gcand.push_back(pc->opts.reserved[3]);
    else gcand = {8192, 16384};
    std::vector<long long> gok;
    for (int per_sm = want < 1 ? 1 : want; per_sm >= 1 && gok.empty(); --per_sm) {
        const long long budget = std::min<long long>((long long)sm_smem / per_sm - static_smem - 1024,
                                                     (long long)max_smem - static_smem);
        const long long ring = (budget - (long long)sweep_smem_for(pc, 0, plan.R)) & ~15ll;
        if (ring < pc->rec_stage_bytes) continue;
        for (long long target : gcand) {
            for (long long gmax : {target, target / 2, target / 4}) {
                if (gmax < pc->rec_stage_bytes) gmax = pc->rec_stage_bytes;
                if (ring_schedule(pc, plan, ring, gmax)) {
                    if (std::find(gok.begin(), gok.end(), gmax) == gok.end()) gok.push_back(gmax);
                    break;
                }
            }
        }
    }
    return gok;
}

void tune_plan(sg_precond* pc, RingPlan& plan, const std::vector<long long>& gmax_list);

// Packs the level records in the configured factor type, plans the
// one-vector ring and times its block size, record-group size and launch
// shape.
void rec_setup_device(sg_precond* pc) {
    if (!pc->use_rec) return;
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    if (pc->rec_stage_bytes % 16 != 0 || pc->rec_total % 16 != 0)
        fail(SG_ERR_INTERNAL, "level records are not 16-byte multiples");
    RingPlan& plan = pc->ring1;
    plan.R = 1;
    plan.ready = false;
    pc->ring4.ready = false;  // a new set-up plans the four-vector ring again when asked
    const std::vector<long long> gok = ring_size(pc, plan);
    if (gok.empty() || (pc->opts.reserved[0] & 1)) {
        pc->use_rec = false;
        return;
    }
    pc->rec_depth = 1;
    ring_upload(pc, plan);
    pc->rec_off_f_d.upload(pc->h_rec_off_f, st);
    pc->rec_off_b_d.upload(pc->h_rec_off_b, st);
    pc->rec_rows_f_d.upload(pc->h_rec_rows_f, st);
    pc->rec_rows_b_d.upload(pc->h_rec_rows_b, st);
    pc->rec_d.alloc((size_t)pc->rec_total);
    pc->err_d.alloc(1);
    pc->err_d.zero(st);
    const uint16_t* pf = pc->perm_f.p;
    const uint16_t* pb = pc->perm_b.p;
#define SG_PACK(TF)                                                                        \
    k_pack_rec<TF><<<pc->nparts, 256, 0, st>>>(                                            \
        pc->info.p, pc->lrp_d.p, pc->lci_d.p, pc->ldiag_d.p, pc->lu_d.p, pf, pb,            \
        pc->lev_ptr_f.p, pc->lev_ptr_b.p, pc->rec_off_f_d.p, pc->rec_off_b_d.p,             \
        pc->rec_rows_f_d.p, pc->rec_rows_b_d.p, pc->rec_d.p)
    if (pc->opts.sweep_dtype == SG_FP64) SG_PACK(double);
    else if (pc->opts.factor_dtype == SG_BF16) SG_PACK(uint16_t);
    else SG_PACK(float);
#undef SG_PACK
    SG_CUDA(cudaGetLastError());
    // block size (forced by opts.reserved[1], else timed), record-group size
    // and launch shape.  Levels of a 3D subdomain hold ~100+ rows, those of a
    // small 2D one ~20: a 512-thread block then idles at every level
    // barrier, while narrower blocks let more subdomains run at once.
    tune_plan(pc, plan, gok);
    pc->sweep_threads = plan.threads;
    // two-level: the coarse restriction runs inside the sweep when every
    // subdomain's CTA can be resident at once (a cooperative launch)
    pc->fuse_restrict = false;
    if (pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS) {
        int coop = 0, per_sm = 0;
        SG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
        if (pc->opts.sweep_dtype == SG_FP64)
            per_sm = sweep_occupancy(pc, plan, k_sweep_tma<double, double, double, double, false, 1, false>);
        else if (pc->opts.factor_dtype == SG_BF16)
            per_sm = sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, uint16_t, false, 1, false>);
        else
            per_sm = sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, float, false, 1, false>);
        if (coop && (long long)per_sm * ctx->num_sms >= pc->nparts && pc->opts.reserved[2] == 0) {
            pc->coarse_sync.alloc(2);
            pc->coarse_sync.zero(st);
            pc->fuse_restrict = true;
        }
    }
}

bool sweep_fuses_restrict(const sg_precond* pc) {
    return pc->use_rec && pc->rec_depth > 0 && pc->fuse_restrict && !pc->sub_on;
}

// Times the sweep (RAS mode, no coarse term, zero input; R interleaved
// vectors) for every record-group size in gmax_list, 128, 256, 384 and 512
// threads per CTA (or the forced block size) and, when there are more
// subdomains than resident CTAs, one CTA per subdomain against a persistent
// grid; keeps the fastest.
void tune_plan(sg_precond* pc, RingPlan& plan, const std::vector<long long>& gmax_list) {
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    const int R = plan.R;
    const size_t n = (size_t)std::max(pc->n, 1) * R;
    const bool f64 = pc->opts.sweep_dtype == SG_FP64;
    const bool bf16 = pc->opts.factor_dtype == SG_BF16;
    DBuf<double> x64, y64;
    DBuf<float> x32, y32;
    if (f64) {
        x64.alloc(n);
        y64.alloc(n);
        x64.zero(st);
    } else {
        x32.alloc(n);
        y32.alloc(n);
        x32.zero(st);
    }
    if (!plan.work.p) {
        plan.work.alloc(2);
        plan.work.zero(st);
    }
    const long long ld = pc->n;
    auto run = [&] {
        if (f64) launch_tma<double, double, double, double, false, 1>(pc, plan, x64.p, y64.p, 0, false, nullptr);
        else if (R == 4 && bf16) launch_tma<float, float, float, uint16_t, false, 4>(pc, plan, x32.p, y32.p, 0, false, nullptr, false, ld, ld);
        else if (R == 4) launch_tma<float, float, float, float, false, 4>(pc, plan, x32.p, y32.p, 0, false, nullptr, false, ld, ld);
        else if (bf16) launch_tma<float, float, float, uint16_t, false, 1>(pc, plan, x32.p, y32.p, 0, false, nullptr);
        else launch_tma<float, float, float, float, false, 1>(pc, plan, x32.p, y32.p, 0, false, nullptr);
    };
    auto occupancy = [&]() -> int {
        if (f64) return sweep_occupancy(pc, plan, k_sweep_tma<double, double, double, double, false, 1, false>);
        if (R == 4 && bf16) return sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, uint16_t, false, 4, false>);
        if (R == 4) return sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, float, false, 4, false>);
        if (bf16) return sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, uint16_t, false, 1, false>);
        return sweep_occupancy(pc, plan, k_sweep_tma<float, float, float, float, false, 1, false>);
    };
    cudaEvent_t e0, e1;
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    float best = -1.f;
    int best_nt = SW_T, best_grid = 0;
    long long best_g = gmax_list.front();
    // one- and two-warp CTAs (reserved[1] = 32 or 64) are not timed: on the
    // 2D subdomains of the batched workload (~20 rows per level) they
    // measured slower than 128 threads (the gather, scatter and record
    // stream lose more than the cheaper barrier gains)
    std::vector<int> threads = {512, 384, 256, 128};
    if (pc->opts.reserved[1] > 0) threads = {pc->opts.reserved[1]};
    for (long long gmax : gmax_list) {
        if (!ring_schedule(pc, plan, plan.ring_bytes, gmax)) continue;
        ring_upload(pc, plan);
        for (int nt : threads) {
            plan.threads = nt;
            plan.grid = 0;
            const int per_sm = occupancy();
            if (per_sm < 1) continue;
            const long long cap = (long long)per_sm * ctx->num_sms;
            // launch shape: opts.reserved[4] 1 forces one CTA per subdomain,
            // 2 a persistent grid of the resident CTAs, k > 2 a persistent
            // grid of k CTAs (at most the resident ones); 0 times one CTA per
            // subdomain against the persistent grid when there are more
            // subdomains than resident CTAs
            std::vector<int> grids = {0};
            const int shape = pc->opts.reserved[4];
            if (shape == 2) grids = {(int)std::min<long long>(cap, pc->nparts)};
            else if (shape > 2) grids = {(int)std::min<long long>(std::min<long long>(cap, shape), pc->nparts)};
            else if (shape == 0 && cap < pc->nparts) grids.push_back((int)cap);
            if (f64) grids = {0};  // FP64 sweeps run one CTA per subdomain
            for (int grid : grids) {
                plan.grid = grid;
                run();
                run();
                cudaEventRecord(e0, st);
                for (int r = 0; r < 5; ++r) run();
                cudaEventRecord(e1, st);
                cudaError_t e = cudaEventSynchronize(e1);
                float ms = 0.f;
                if (e == cudaSuccess) e = cudaEventElapsedTime(&ms, e0, e1);
                if (e != cudaSuccess) {
                    cudaEventDestroy(e0);
                    cudaEventDestroy(e1);
                    SG_CUDA(e);
                }
                if (best < 0.f || ms < best) {
                    best = ms;
                    best_nt = nt;
                    best_g = gmax;
                    best_grid = grid;
                }
            }
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (best < 0.f) fail(SG_ERR_INTERNAL, "no sweep configuration fits the GPU");
    plan.threads = best_nt;
    plan.grid = best_grid;
    if (!ring_schedule(pc, plan, plan.ring_bytes, best_g)) fail(SG_ERR_INTERNAL, "ring schedule lost");
    ring_upload(pc, plan);
    plan.ready = true;
}

template <class TI, class TO>
bool sweep_tma(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse, bool exact,
               const int* active) {
    if (!pc->use_rec || pc->rec_depth == 0) return false;
    const RingPlan& plan = pc->ring1;
    const bool fuse = coarse && sweep_fuses_restrict(pc);
    if (pc->opts.sweep_dtype == SG_FP64) {
        if (exact) launch_tma<TI, TO, double, double, true, 1>(pc, plan, x, y, mode, coarse, active, fuse);
        else launch_tma<TI, TO, double, double, false, 1>(pc, plan, x, y, mode, coarse, active, fuse);
    } else if (pc->opts.factor_dtype == SG_BF16) {
        launch_tma<TI, TO, float, uint16_t, false, 1>(pc, plan, x, y, mode, coarse, active, fuse);
    } else {
        launch_tma<TI, TO, float, float, false, 1>(pc, plan, x, y, mode, coarse, active, fuse);
    }
    return true;
}

// Plans (and times) the four-vector ring of a RAS preconditioner with FP32
// sweeps, once per set-up; call it outside stream capture.  False when the
// preconditioner has no such sweep.
bool sweep_plan4(sg_precond* pc) {
    if (!pc->use_rec || pc->rec_depth == 0 || pc->opts.sweep_dtype == SG_FP64) return false;
    if (pc->kind != SG_PC_RAS) return false;
    RingPlan& plan = pc->ring4;
    if (plan.ready) return true;
    plan.R = 4;
    const std::vector<long long> gok = ring_size(pc, plan);
    if (gok.empty()) return false;
    const int* keep = pc->sub_on;
    pc->sub_on = nullptr;
    tune_plan(pc, plan, gok);
    pc->sub_on = keep;
    return true;
}

// Four right-hand sides at once (RAS without a coarse term, FP32 sweeps): x
// and y hold them ld apart; sub_on (NULL or 4 x nparts switches) gates the
// subdomains.  Returns false, launching nothing, when the four-vector ring
// has not been planned (sweep_plan4).
template <class TI, class TO>
bool sweep_tma4(sg_precond* pc, const TI* x, TO* y, long long ld, const int* sub_on) {
    if (!pc->use_rec || pc->rec_depth == 0 || pc->opts.sweep_dtype == SG_FP64) return false;
    if (pc->kind != SG_PC_RAS || !pc->ring4.ready) return false;
    const RingPlan& plan = pc->ring4;
    const int* keep = pc->sub_on;
    pc->sub_on = sub_on;
    struct Restore {
        sg_precond* pc;
        const int* v;
        ~Restore() { pc->sub_on = v; }
    } restore{pc, keep};
    if (pc->opts.factor_dtype == SG_BF16)
        launch_tma<TI, TO, float, uint16_t, false, 4>(pc, plan, x, y, 0, false, nullptr, false, ld, ld);
    else
        launch_tma<TI, TO, float, float, false, 4>(pc, plan, x, y, 0, false, nullptr, false, ld, ld);
    return true;
}

int sweep_error(sg_precond* pc) {
    if (!pc->err_d.p) return 0;
    int e = 0;
    SG_CUDA(cudaMemcpyAsync(&e, pc->err_d.p, sizeof(int), cudaMemcpyDeviceToHost, pc->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(pc->ctx->stream));
    // reported once: clear the error word, the fused restriction's counters
    // and the persistent launches' work counters, which a sweep that gave up
    // may have left mid-count, so the next apply starts clean
    if (e) {
        pc->err_d.zero(pc->ctx->stream);
        if (pc->coarse_sync.p) pc->coarse_sync.zero(pc->ctx->stream);
        if (pc->ring1.work.p) pc->ring1.work.zero(pc->ctx->stream);
        if (pc->ring4.work.p) pc->ring4.work.zero(pc->ctx->stream);
        SG_CUDA(cudaStreamSynchronize(pc->ctx->stream));
    }
    return e;
}

bool sweep_wait_test_supported(const sg_precond* pc, int mode) {
    if (mode == 0) return true;
    if (!pc->use_rec || pc->rec_depth == 0) return false;
    if (mode == 1) return true;
    return mode == 2 && sweep_fuses_restrict(pc);
}

template bool sweep_tma<double, double>(sg_precond*, const double*, double*, int, bool, bool,
                                        const int*);
template bool sweep_tma<double, float>(sg_precond*, const double*, float*, int, bool, bool,
                                       const int*);
template bool sweep_tma<float, float>(sg_precond*, const float*, float*, int, bool, bool,
                                      const int*);
template bool sweep_tma4<double, float>(sg_precond*, const double*, float*, long long, const int*);
template bool sweep_tma4<float, float>(sg_precond*, const float*, float*, long long, const int*);

}  // namespace sg

namespace sg {

// Host check of the TMA-fed sweep's data -- what a debug build's bounds
// asserts in the kernel would test, done on the host so that no check can
// fault a GPU: the level records are read back and
//  * every row slot of a level is a real row of the subdomain and every
//    column slot a real row or the zero slot (all inside the shared vector);
//  * every column a row reads was computed by an earlier level of the same
//    sweep (forward: the lower triangle; backward: the upper), i.e. the level
//    schedule respects the factor's dependences;
//  * every level's record lies inside its group's ring bytes and inside the
//    ring, each group is issued before the level that waits for it, and no
//    group overwrites ring bytes or re-arms an mbarrier of a group that a
//    later level still reads; each group's stream bytes match its records'
//    packed offsets.
// plant = 1 (testing) first corrupts one column slot of the host copy.
// Returns the number of violations found (0: all hold).
static long long plan_check(sg_precond* pc, const RingPlan& plan, int plant);

long long sweep_check(sg_precond* pc, int plant) {
    if (!pc->use_rec || pc->rec_depth == 0) return 0;
    long long bad = plan_check(pc, pc->ring1, plant);
    if (pc->ring4.ready) bad += plan_check(pc, pc->ring4, 0);
    return bad;
}

static long long plan_check(sg_precond* pc, const RingPlan& plan, int plant) {
    cudaStream_t st = pc->ctx->stream;
    std::vector<unsigned char> rec((size_t)pc->rec_total);
    SG_CUDA(cudaMemcpyAsync(rec.data(), pc->rec_d.p, rec.size(), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    const long long sf = pc->opts.sweep_dtype == SG_FP64 ? 8
                         : (pc->opts.factor_dtype == SG_BF16 ? 2 : 4);
    const RingSub* subs = reinterpret_cast<const RingSub*>(plan.sub.data());
    const int* meta = plan.meta.data();
    const int* grp = plan.grp.data();
    long long bad = 0;
    bool planted = false;
    std::vector<char> done;
    std::vector<int> last_level, first_level;
    for (int s = 0; s < pc->nparts; ++s) {
        const SubInfo& inf = pc->h_info[s];
        const RingSub& r = subs[s];
        const int nf = inf.nlev_f, T = inf.nlev_f + inf.nlev_b, n = inf.n, p = inf.tshift;
        const int zero_slot = tslot(n, p);
        // slot -> is it a real row
        std::vector<char> real((size_t)zero_slot + 1, 0);
        for (int li = 0; li < n; ++li) real[tslot(li, p)] = 1;
        // ---- records: bounds and dependences
        for (int dir = 0; dir < 2; ++dir) {
            done.assign((size_t)zero_slot + 1, 0);
            const int w = dir == 0 ? inf.wl : inf.wu;
            const int nl = dir == 0 ? inf.nlev_f : inf.nlev_b;
            for (int l = 0; l < nl; ++l) {
                const int i = (dir == 0 ? inf.lev_off_f : inf.lev_off_b) + l;
                const int c = dir == 0 ? pc->h_lev_ptr_f[i + 1] - pc->h_lev_ptr_f[i]
                                       : pc->h_lev_ptr_b[i + 1] - pc->h_lev_ptr_b[i];
                const int C = dir == 0 ? pc->h_rec_rows_f[i] : pc->h_rec_rows_b[i];
                const long long off = dir == 0 ? pc->h_rec_off_f[i] : pc->h_rec_off_b[i];
                const long long bytes = (long long)C * (2 + w * (2 + sf) + (dir ? sf : 0));
                if (C % 8 || c > C || off < 0 || off + bytes > pc->rec_total) {
                    ++bad;
                    continue;
                }
                uint16_t* rows = reinterpret_cast<uint16_t*>(rec.data() + off);
                uint16_t* cols = rows + C;
                if (plant && !planted && l > 0 && c > 0 && w > 0) {
                    cols[0] = (uint16_t)rows[0];  // a row reading itself: not yet computed
                    planted = true;
                }
                for (int q = 0; q < c; ++q) {
                    const int rs = rows[q];
                    if (rs >= zero_slot || !real[rs]) {
                        ++bad;
                        continue;
                    }
                    for (int k = 0; k < w; ++k) {
                        const int cs = cols[(size_t)k * C + q];
                        if (cs > zero_slot) ++bad;
                        else if (cs != zero_slot && (!real[cs] || !done[cs])) ++bad;
                    }
                }
                for (int q = 0; q < c; ++q)
                    if (rows[q] < zero_slot) done[rows[q]] = 1;
            }
        }
        // ---- ring schedule: simulate the producer and the level loop
        const int G = r.ngrp;
        last_level.assign(G, -1);
        first_level.assign(G, -1);
        int cur = -1;
        for (int g = 0; g < T; ++g) {
            const int* m = meta + 4 * ((size_t)r.meta_off + g);
            if (m[2] >= 0) {
                if (m[2] != cur + 1) ++bad;  // groups open in order
                cur = m[2];
                first_level[cur] = g;
            }
            if (cur < 0 || cur >= G) {
                ++bad;
                break;
            }
            last_level[cur] = g;
        }
        int issued = r.ninit;
        if (issued > G) ++bad;
        for (int g = 0; g < T && cur >= 0; ++g) {
            const int* m = meta + 4 * ((size_t)r.meta_off + g);
            int j = 0;
            while (j + 1 < G && first_level[j + 1] >= 0 && first_level[j + 1] <= g) ++j;
            const int c = m[0] & 0xffff, C = (int)((unsigned)m[0] >> 16);
            const bool back = g >= nf;
            const int i = back ? inf.lev_off_b + (g - nf) : inf.lev_off_f + g;
            const long long B = (long long)C * (back ? 2 + inf.wu * (2 + sf) + sf : 2 + inf.wl * (2 + sf));
            const long long rel = (back ? pc->h_rec_off_b[i] : pc->h_rec_off_f[i]) - r.base;
            const int* gj = grp + 2 * ((size_t)r.grp_off + j);
            const long long gstart = (unsigned)gj[0];
            const long long gbytes = (long long)(((unsigned)gj[1] & 0xffffu) << 4);
            const long long gpos = (long long)(((unsigned)gj[1] >> 16) << 4);
            if (c != (back ? pc->h_lev_ptr_b[i + 1] - pc->h_lev_ptr_b[i]
                           : pc->h_lev_ptr_f[i + 1] - pc->h_lev_ptr_f[i]))
                ++bad;
            if (m[1] < gpos || m[1] + B > gpos + gbytes || m[1] + B > plan.ring_bytes) ++bad;
            if (rel - gstart != m[1] - gpos) ++bad;  // the ring copy holds this record
            if (m[2] >= 0 && m[2] >= issued) ++bad;  // waits for a copy not yet issued
            // issue after the level: what the new groups overwrite must be done
            for (int k = issued; k < m[3] && k < G; ++k) {
                const int* gk = grp + 2 * ((size_t)r.grp_off + k);
                const long long kb = (long long)(((unsigned)gk[1] & 0xffffu) << 4);
                const long long kp = (long long)(((unsigned)gk[1] >> 16) << 4);
                for (int q = 0; q < k; ++q) {
                    if (last_level[q] <= g) continue;  // finished: its bytes are free
                    const int* gq = grp + 2 * ((size_t)r.grp_off + q);
                    const long long qb = (long long)(((unsigned)gq[1] & 0xffffu) << 4);
                    const long long qp = (long long)(((unsigned)gq[1] >> 16) << 4);
                    if (kp < qp + qb && qp < kp + kb) ++bad;
                }
                if (k >= RING_NBAR && last_level[k - RING_NBAR] > g) ++bad;
            }
            if (m[3] > issued) issued = m[3];
        }
        if (issued != G && T > 0) ++bad;  // every group issued by the end
    }
    if (plant && !planted) ++bad;  // nothing to corrupt: report it as found
    return bad;
}

}  // namespace sg
