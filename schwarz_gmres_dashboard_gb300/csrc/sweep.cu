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
// distinct banks).  A subdomain's records are contiguous (forward levels,
// then backward), so the ring holds groups of K consecutive records: the
// block's last thread copies a whole group into one of NB shared-memory
// buffers with one cp.async.bulk, tracked by one mbarrier, NB - 1 groups
// ahead of the group being computed.  So a level costs shared-memory latency
// plus one barrier instead of a global-memory round trip, and the copy issue
// and the waits are paid once per K levels.  Every mbarrier wait is bounded
// (about one second of clock cycles); on expiry the CTA records an error
// word, waits (bounded again) for the copies it issued, and returns without
// touching the output.
#include <algorithm>

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

struct RecArgs {
    const SubInfo* info;
    const int* order;
    const int* dofs;
    const int* lev_f;
    const int* lev_b;
    const long long* off_f;
    const long long* off_b;
    const int* rows_f;
    const int* rows_b;
    const unsigned char* rec;
    const int* ownloc;
    const int* owned;
    const double* a0inv;
    const double* r0;
    int nc;
    int nbuf;     // record buffers in the ring
    int glev;     // consecutive levels per buffer
    int gbytes;   // buffer size
    int t_len;       // elements of the subdomain vector region (largest tslot(n) + 1)
    int max_levels;  // largest nlev_f + nlev_b over the subdomains
    int* err;
    const int* sub_on;  // optional per-subdomain switch (0: the subdomain is skipped)
    // coarse restriction fused into the sweep (cooperative launch, all blocks
    // resident): each block writes r0[s] and counts itself in sync[0]; sync[1]
    // counts the blocks done with r0 (the last one resets both)
    int fuse;
    double* r0w;
    unsigned* sync;
    // bounded waits: cycle budget of the record and restriction waits, and
    // the test mode that makes one of them run out without any fault
    // (1: no record group 0 is copied; 2: no restriction is counted)
    long long wait_budget;
    int wait_test;
};

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// mode 0: RAS (owned rows written), 1: ASM (all rows added atomically).
template <class TI, class TO, class TS, class TF, bool EXACT>
__global__ void __launch_bounds__(SW_T, 2)
k_sweep_tma(RecArgs a, const TI* __restrict__ x, TO* __restrict__ y, int mode, int coarse,
            const int* __restrict__ active) {
    if (active && *active == 0) return;
    extern __shared__ __align__(128) unsigned char smraw[];
    __shared__ double s_zc;
    __shared__ double s_red[RC_MAXCH];
    __shared__ int s_ok;
    const int NB = a.nbuf, K = a.glev;
    uint64_t* bars = reinterpret_cast<uint64_t*>(smraw);              // NB x 8 B
    const int NC = (int)blockDim.x;
    unsigned char* bufs = smraw + 128;                                 // NB x gbytes
    TS* t = reinterpret_cast<TS*>(bufs + (size_t)NB * a.gbytes);       // t_len
    const int s = a.order[blockIdx.x];
    if (a.sub_on && !a.sub_on[s]) return;  // subdomain not needed by this apply
    const SubInfo inf = a.info[s];
    const int n = inf.n;
    const int nf = inf.nlev_f, T = inf.nlev_f + inf.nlev_b;
    const int sf = (int)sizeof(TF);
    // per-level metadata of both sweeps, staged once: rows, padded rows,
    // record offset (so the level loop touches global memory only through TMA)
    long long* m_off = reinterpret_cast<long long*>(
        reinterpret_cast<unsigned char*>(t) + (((size_t)a.t_len * sizeof(TS) + 15) & ~(size_t)15));
    int* m_c = reinterpret_cast<int*>(m_off + a.max_levels);
    int* m_C = m_c + a.max_levels;
    for (int g = threadIdx.x; g < T; g += blockDim.x) {
        if (g < nf) {
            const int i = inf.lev_off_f + g;
            m_c[g] = a.lev_f[i + 1] - a.lev_f[i];
            m_C[g] = a.rows_f[i];
            m_off[g] = a.off_f[i];
        } else {
            const int i = inf.lev_off_b + (g - nf);
            m_c[g] = a.lev_b[i + 1] - a.lev_b[i];
            m_C[g] = a.rows_b[i];
            m_off[g] = a.off_b[i];
        }
    }
    __syncthreads();

    const uint32_t bytes_f = (uint32_t)(2 + inf.wl * (2 + sf));
    const uint32_t bytes_b = (uint32_t)(2 + inf.wu * (2 + sf) + sf);
    const int ngrp = (T + K - 1) / K;
    // copy the records of group q (levels qK .. qK+K-1, contiguous) into
    // buffer b with one bulk copy
    auto issue = [&](int q, int b) {
        const int g0 = q * K, g1 = (g0 + K < T ? g0 + K : T) - 1;
        const uint32_t bytes = (uint32_t)(m_off[g1] - m_off[g0]) +
                               (uint32_t)m_C[g1] * (g1 < nf ? bytes_f : bytes_b);
        const uint32_t bar = smem_u32(&bars[b]);
        mbar_expect_tx(bar, bytes);
        bulk_g2s_stream(smem_u32(bufs + (size_t)b * a.gbytes), a.rec + m_off[g0], bytes, bar);
    };

    // the producer is the block's last thread: levels rarely have rows for
    // it, so issuing the next copy overlaps the other threads' work (a
    // separate producer warp, signalled through per-buffer "empty"
    // mbarriers, measured slower at every block size)
    const bool producer = threadIdx.x == blockDim.x - 1;
    if (producer) {
        for (int i = 0; i < NB; ++i) mbar_init(smem_u32(&bars[i]), 1);
        fence_mbar_init();
        fence_proxy_async();
        for (int q = 0; q < ngrp && q < NB; ++q)
            if (!(a.wait_test == 1 && q == 0)) issue(q, q);
    }
    // gather while the first records are in flight
    const int* dof = a.dofs + inf.row_off;
    const int tp = inf.tshift;
    gather_rows<TS>(t, x, dof, n, NC, tp);
    if (threadIdx.x == 0) t[tslot(n, tp)] = (TS)0;
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

    // The level loop is the latency chain of the sweep.  Per level: the rows,
    // then one barrier.  Per group of K levels: every thread observes the
    // buffer's mbarrier (acquiring the bulk copy) at the first level, a
    // failed wait travels in that level's barrier, and after the group's last
    // level the producer refills the buffer with group q + NB.  Buffer and
    // phase advance without divisions; the next level's row counts load while
    // this level computes.
    const uint32_t bufs_s = smem_u32(bufs), t_s = smem_u32(t);
    int q = 0, b = 0, gstart = 0, gend = T < K ? T : K;
    uint32_t ph = 0;
    // level g's rows (c), padded rows (C) and record offset in its buffer
    // (roff) are in registers; the next level's load during this level and
    // are used after its barrier, so no shared-memory load heads a level
    int c = T > 0 ? m_c[0] : 0, C = T > 0 ? m_C[0] : 0;
    long long base_off = T > 0 ? m_off[0] : 0;
    uint32_t roff = 0;
    for (int g = 0; g < T; ++g) {
        bool ok = true;
        if (g == gstart) ok = mbar_wait(smem_u32(&bars[b]), ph, a.wait_budget);
        int cn = 0, Cn = 0;
        long long on = 0;
        if (g + 1 < T) {
            cn = m_c[g + 1];
            Cn = m_C[g + 1];
            on = m_off[g + 1];
        }
        if (ok) {
            const bool back = g >= nf;
            const uint32_t off = (uint32_t)b * (uint32_t)a.gbytes + roff;
            level_rows<TS, TF, EXACT>(t, t_s, bufs + off, bufs_s + off, C, c,
                                      back ? inf.wu : inf.wl, back, NC);
        }
        if (g == gstart) {
            if (__syncthreads_or(ok ? 0 : 1)) {
                // a record group did not arrive in time: report, drain the
                // copies that were issued (groups q .. q+NB-1; the earlier
                // ones have landed), leave y alone.  Each drain wait has the
                // full budget; if one still gives up, the block leaves with
                // that copy outstanding -- accepted only because such a copy
                // never arrives at all -- and the error word says 2.
                if (producer) {
                    int code = 1;
                    int b2 = b;
                    uint32_t p2 = ph;
                    for (int h = q; h < ngrp && h < q + NB; ++h) {
                        const bool issued = !(a.wait_test == 1 && h == 0);
                        if (issued && !mbar_wait(smem_u32(&bars[b2]), p2, WAIT_CYCLES)) code = 2;
                        if (++b2 == NB) {
                            b2 = 0;
                            p2 ^= 1u;
                        }
                    }
                    atomicMax(a.err, code);
                }
                return;
            }
        } else {
            __syncthreads();
        }
        if (g + 1 == gend) {
            // buffer b is free again: refill it with group q + NB
            if (producer && q + NB < ngrp) {
                fence_proxy_async();
                issue(q + NB, b);
            }
            ++q;
            if (++b == NB) {
                b = 0;
                ph ^= 1u;
            }
            gstart = gend;
            gend = gstart + K < T ? gstart + K : T;
            base_off = on;  // the next level opens the new group
        }
        roff = (uint32_t)(on - base_off);
        c = cn;
        C = Cn;
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
                return;
            }
        }
        if (threadIdx.x < 32) {
            const double z = a.fuse ? coarse_dot_warp0<true>(a.a0inv + (size_t)s * a.nc, a.r0, a.nc)
                                    : coarse_dot_warp0<false>(a.a0inv + (size_t)s * a.nc, a.r0, a.nc);
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
        scatter_owned<TS, TO>(t, y, a.ownloc + inf.own_off, a.owned + inf.own_off, inf.n_own,
                              coarse, zc, NC, tp);
    } else {
        for (int li = threadIdx.x; li < n; li += NC)
            atomicAdd(&y[dof[li]], Store<TO>::f(t[tslot(li, tp)]));
        if (coarse) {
            const int* og = a.owned + inf.own_off;
            for (int q = threadIdx.x; q < inf.n_own; q += NC)
                atomicAdd(&y[og[q]], Store<TO>::f(zc));
        }
    }
}

RecArgs rec_args(sg_precond* pc, bool fuse) {
    RecArgs a;
    a.fuse = fuse ? 1 : 0;
    a.r0w = pc->r0.p;
    a.sync = pc->coarse_sync.p;
    a.info = pc->info.p;
    a.order = pc->order.p;
    a.dofs = pc->dofs.p;
    a.lev_f = pc->lev_ptr_f.p;
    a.lev_b = pc->lev_ptr_b.p;
    a.off_f = pc->rec_off_f_d.p;
    a.off_b = pc->rec_off_b_d.p;
    a.rows_f = pc->rec_rows_f_d.p;
    a.rows_b = pc->rec_rows_b_d.p;
    a.rec = pc->rec_d.p;
    a.ownloc = pc->ownloc_d.p;
    a.owned = pc->owned_d.p;
    a.a0inv = pc->a0inv.p;
    a.r0 = pc->r0.p;
    a.nc = pc->nc;
    a.nbuf = pc->rec_depth;
    a.glev = pc->rec_glev;
    a.gbytes = (int)pc->rec_gbytes;
    a.t_len = pc->t_len;
    a.max_levels = pc->max_levels;
    a.err = pc->err_d.p;
    a.sub_on = pc->sub_on;
    a.wait_test = pc->wait_test;
    a.wait_budget = pc->wait_test ? WAIT_TEST_CYCLES : WAIT_CYCLES;
    return a;
}

// dynamic shared memory of the sweep: mbarriers, nbuf record buffers of
// gbytes, the subdomain vector, per-level metadata
size_t sweep_smem_for(const sg_precond* pc, int nbuf, long long gbytes) {
    const size_t ts = pc->opts.sweep_dtype == SG_FP64 ? 8 : 4;
    const size_t tbytes = ((size_t)pc->t_len * ts + 15) & ~(size_t)15;
    return 128 + (size_t)nbuf * (size_t)gbytes + tbytes + (size_t)pc->max_levels * 16;
}
size_t sweep_smem(const sg_precond* pc) {
    return sweep_smem_for(pc, pc->rec_depth, pc->rec_gbytes);
}

template <class TI, class TO, class TS, class TF, bool EXACT>
void launch_tma(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse, const int* active,
                bool fuse = false) {
    const size_t smem = sweep_smem(pc);
    const int nt = pc->sweep_threads > 0 ? pc->sweep_threads : SW_T;
    auto kern = k_sweep_tma<TI, TO, TS, TF, EXACT>;
    SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    RecArgs a = rec_args(pc, fuse);
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
        kern<<<pc->nparts, nt, smem, pc->ctx->stream>>>(a, x, y, mode, coarse_i, active);
    }
    SG_CUDA(cudaGetLastError());
    count_launch(pc->ctx);
}

}  // namespace

void tune_sweep_threads(sg_precond* pc);

// Largest byte span of K consecutive level records of one subdomain (its
// forward then backward records are contiguous in the packed array).
static long long rec_group_max(const sg_precond* pc, int K) {
    const long long sf = pc->opts.sweep_dtype == SG_FP64 ? 8
                         : (pc->opts.factor_dtype == SG_BF16 ? 2 : 4);
    long long mx = 0;
    std::vector<long long> offs;
    for (int s = 0; s < pc->nparts; ++s) {
        const SubInfo& inf = pc->h_info[s];
        const int T = inf.nlev_f + inf.nlev_b;
        if (T == 0) continue;
        offs.assign((size_t)T + 1, 0);
        for (int l = 0; l < inf.nlev_f; ++l) offs[l] = pc->h_rec_off_f[inf.lev_off_f + l];
        for (int l = 0; l < inf.nlev_b; ++l)
            offs[inf.nlev_f + l] = pc->h_rec_off_b[inf.lev_off_b + l];
        const long long last_rows = inf.nlev_b > 0
                                        ? pc->h_rec_rows_b[inf.lev_off_b + inf.nlev_b - 1]
                                        : pc->h_rec_rows_f[inf.lev_off_f + inf.nlev_f - 1];
        const long long last_bytes = inf.nlev_b > 0 ? last_rows * (2 + inf.wu * (2 + sf) + sf)
                                                    : last_rows * (2 + inf.wl * (2 + sf));
        offs[T] = offs[T - 1] + last_bytes;
        for (int g0 = 0; g0 < T; g0 += K) {
            const int g1 = g0 + K < T ? g0 + K : T;
            mx = std::max(mx, offs[g1] - offs[g0]);
        }
    }
    return mx;
}

// Packs the level records of the configured factor type and sizes the
// record ring so that as many subdomains as possible run at once.
void rec_setup_device(sg_precond* pc) {
    if (!pc->use_rec) return;
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    if (pc->rec_stage_bytes % 16 != 0 || pc->rec_total % 16 != 0)
        fail(SG_ERR_INTERNAL, "level records are not 16-byte multiples");
    int max_smem = 0;
    SG_CUDA(cudaDeviceGetAttribute(&max_smem, cudaDevAttrMaxSharedMemoryPerBlockOptin,
                                   ctx->device));
    int sm_smem = 0;
    SG_CUDA(cudaDeviceGetAttribute(&sm_smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor,
                                   ctx->device));
    const int static_smem = 1024;  // reduction scratch and the like
    // CTAs per SM needed to keep every subdomain resident at once
    const int want = (pc->nparts + ctx->num_sms - 1) / ctx->num_sms;
    // ring: nbuf buffers, each holding K consecutive level records (a
    // subdomain's records are contiguous: forward levels, then backward), so
    // one bulk copy and one mbarrier serve K levels.  Prefer K*(nbuf-1)
    // levels of lead (up to 8), then larger K, under the CTAs-per-SM budget.
    int nbuf = 0, glev = 1;
    long long gbytes = 0;
    for (int per_sm = want < 1 ? 1 : want; per_sm >= 1 && nbuf == 0; --per_sm) {
        const long long budget = (long long)sm_smem / per_sm - static_smem - 1024;
        int best = -1;
        for (int K : {8, 6, 4, 3, 2, 1}) {
            const long long g = (rec_group_max(pc, K) + 127) & ~127ll;
            for (int nb : {3, 2}) {
                const long long need = (long long)sweep_smem_for(pc, nb, g);
                if (need > budget || need > max_smem - static_smem) continue;
                const int lead = (nb - 1) * K;
                const int score = (lead < 8 ? lead : 8) * 10 + K;
                if (score > best) {
                    best = score;
                    nbuf = nb;
                    glev = K;
                    gbytes = g;
                }
            }
        }
    }
    // an mbarrier transaction count stays below 2^20 bytes
    if (nbuf == 0 || gbytes >= (1 << 20) || (pc->opts.reserved[0] & 1)) {
        pc->use_rec = false;
        return;
    }
    pc->rec_depth = nbuf;
    pc->rec_glev = glev;
    pc->rec_gbytes = gbytes;
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
    // threads per CTA: forced by opts.reserved[1], else timed.  Levels of a
    // 3D subdomain hold ~100+ rows, those of a small 2D one ~20: a 512-thread
    // block then idles at every level barrier, while narrower blocks let more
    // subdomains run at once on an SM.
    if (pc->opts.reserved[1] > 0) {
        pc->sweep_threads = pc->opts.reserved[1];
    } else {
        tune_sweep_threads(pc);
    }
    // two-level: the coarse restriction runs inside the sweep when every
    // subdomain's CTA can be resident at once (a cooperative launch)
    pc->fuse_restrict = false;
    if (pc->kind == SG_PC_TWOLEVEL_ASM || pc->kind == SG_PC_TWOLEVEL_RAS) {
        const size_t smem = sweep_smem(pc);
        const int nt = pc->sweep_threads > 0 ? pc->sweep_threads : SW_T;
        int coop = 0, per_sm = 0;
        SG_CUDA(cudaDeviceGetAttribute(&coop, cudaDevAttrCooperativeLaunch, ctx->device));
        auto occupancy = [&](auto kern) {
            SG_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         (int)smem));
            SG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, nt, smem));
        };
        if (pc->opts.sweep_dtype == SG_FP64)
            occupancy(k_sweep_tma<double, double, double, double, false>);
        else if (pc->opts.factor_dtype == SG_BF16)
            occupancy(k_sweep_tma<float, float, float, uint16_t, false>);
        else
            occupancy(k_sweep_tma<float, float, float, float, false>);
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

// Times the sweep (RAS mode, no coarse term, zero input) with 128, 256 and
// 512 threads per CTA and keeps the fastest.
void tune_sweep_threads(sg_precond* pc) {
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    const size_t n = (size_t)std::max(pc->n, 1);
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
    auto run = [&] {
        if (f64) launch_tma<double, double, double, double, false>(pc, x64.p, y64.p, 0, false, nullptr);
        else if (bf16) launch_tma<float, float, float, uint16_t, false>(pc, x32.p, y32.p, 0, false, nullptr);
        else launch_tma<float, float, float, float, false>(pc, x32.p, y32.p, 0, false, nullptr);
    };
    cudaEvent_t e0, e1;
    SG_CUDA(cudaEventCreate(&e0));
    SG_CUDA(cudaEventCreate(&e1));
    float best = 0.f;
    int best_nt = SW_T;
    for (int nt : {512, 256, 128}) {
        pc->sweep_threads = nt;
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
        if (nt == 512 || ms < best) {
            best = ms;
            best_nt = nt;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    pc->sweep_threads = best_nt;
}

template <class TI, class TO>
bool sweep_tma(sg_precond* pc, const TI* x, TO* y, int mode, bool coarse, bool exact,
               const int* active) {
    if (!pc->use_rec || pc->rec_depth == 0) return false;
    const bool fuse = coarse && sweep_fuses_restrict(pc);
    if (pc->opts.sweep_dtype == SG_FP64) {
        if (exact) launch_tma<TI, TO, double, double, true>(pc, x, y, mode, coarse, active, fuse);
        else launch_tma<TI, TO, double, double, false>(pc, x, y, mode, coarse, active, fuse);
    } else if (pc->opts.factor_dtype == SG_BF16) {
        launch_tma<TI, TO, float, uint16_t, false>(pc, x, y, mode, coarse, active, fuse);
    } else {
        launch_tma<TI, TO, float, float, false>(pc, x, y, mode, coarse, active, fuse);
    }
    return true;
}

int sweep_error(sg_precond* pc) {
    if (!pc->err_d.p) return 0;
    int e = 0;
    SG_CUDA(cudaMemcpyAsync(&e, pc->err_d.p, sizeof(int), cudaMemcpyDeviceToHost, pc->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(pc->ctx->stream));
    // reported once: clear the error word, and the fused restriction's
    // counters, which a sweep that gave up may have left mid-count, so the
    // next apply starts clean
    if (e) {
        pc->err_d.zero(pc->ctx->stream);
        if (pc->coarse_sync.p) pc->coarse_sync.zero(pc->ctx->stream);
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

}  // namespace sg
