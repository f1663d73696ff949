// dev_common.cuh -- device helpers shared by the kernels of libsgmres.
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sg_internal.h"

namespace sg {

// ----------------------------------------------------------------- arithmetic
// FP64 operations without multiply-add contraction: the reference's x86 build
// rounds every product and every sum, so these reproduce its results bit for
// bit where the operation order is also the same.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }

// acc - a*b: exact-order for double, fused for float
__device__ __forceinline__ double msub(double acc, double a, double b) {
    return __dsub_rn(acc, __dmul_rn(a, b));
}
__device__ __forceinline__ float msub(float acc, float a, float b) { return fmaf(-a, b, acc); }

// storage -> arithmetic conversions
__device__ __forceinline__ double to_d(double v) { return v; }
__device__ __forceinline__ double to_d(float v) { return (double)v; }
__device__ __forceinline__ float to_f(double v) { return (float)v; }
__device__ __forceinline__ float to_f(float v) { return v; }
__device__ __forceinline__ float bf16_to_f(uint16_t b) {
    return __uint_as_float(((unsigned)b) << 16);
}

// The backward sweep's division by the diagonal: FP64 divides (the
// reference's rounding); FP32 multiplies by the reciprocal, which depends
// only on the diagonal (loaded early), so it leaves the row's dependency
// chain -- one multiply instead of a division on it.
__device__ __forceinline__ double div_diag(double acc, double d) { return acc / d; }
__device__ __forceinline__ float div_diag(float acc, float d) { return acc * (1.0f / d); }

template <class TS>
struct Load;
template <>
struct Load<double> {
    __device__ __forceinline__ static double f(double v) { return v; }
    __device__ __forceinline__ static double f(float v) { return (double)v; }
    __device__ __forceinline__ static double f(uint16_t v) { return (double)bf16_to_f(v); }
};
template <>
struct Load<float> {
    __device__ __forceinline__ static float f(double v) { return (float)v; }
    __device__ __forceinline__ static float f(float v) { return v; }
    __device__ __forceinline__ static float f(uint16_t v) { return bf16_to_f(v); }
};

template <class TO>
struct Store;
template <>
struct Store<double> {
    __device__ __forceinline__ static double f(double v) { return v; }
    __device__ __forceinline__ static double f(float v) { return (double)v; }
};
template <>
struct Store<float> {
    __device__ __forceinline__ static float f(double v) { return (float)v; }
    __device__ __forceinline__ static float f(float v) { return v; }
};

// ---------------------------------------------------------- streaming loads
// Loads of data that a kernel streams once from HBM: the L2 fetches the whole
// aligned 256-byte block around the address (the neighbouring lanes' or the
// next step's data) instead of single sectors, and L1 keeps no copy.
// Measured on a 268 MB read: 5.8 TB/s against 4.9 TB/s with plain 16-byte
// loads.  ld_stream is coherent (safe on data the kernel itself writes
// later).
__device__ __forceinline__ float4 ld_stream(const float4* p) {
    float4 v;
    asm volatile("ld.global.L1::no_allocate.L2::256B.v4.f32 {%0,%1,%2,%3}, [%4];"
                 : "=f"(v.x), "=f"(v.y), "=f"(v.z), "=f"(v.w) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ double2 ld_stream(const double2* p) {
    double2 v;
    asm volatile("ld.global.L1::no_allocate.L2::256B.v2.f64 {%0,%1}, [%2];"
                 : "=d"(v.x), "=d"(v.y) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ float ld_stream(const float* p) {
    float v;
    asm volatile("ld.global.L1::no_allocate.L2::256B.f32 %0, [%1];" : "=f"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ double ld_stream(const double* p) {
    double v;
    asm volatile("ld.global.L1::no_allocate.L2::256B.f64 %0, [%1];" : "=d"(v) : "l"(p) : "memory");
    return v;
}

// Read-only streaming loads (data no thread writes during the kernel) with
// an L2 cache policy; policy_evict_first() marks data read once per solve
// step, which should not displace vectors that the next kernels re-read.
__device__ __forceinline__ uint64_t policy_evict_first() {
    uint64_t pol;
    asm("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(pol));
    return pol;
}
__device__ __forceinline__ float ldg_stream(const float* p, uint64_t pol) {
    float v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.f32 %0, [%1], %2;"
        : "=f"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ double ldg_stream(const double* p, uint64_t pol) {
    double v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.f64 %0, [%1], %2;"
        : "=d"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int ldg_stream(const int* p, uint64_t pol) {
    int v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.s32 %0, [%1], %2;"
        : "=r"(v) : "l"(p), "l"(pol));
    return v;
}
__device__ __forceinline__ int16_t ldg_stream(const int16_t* p, uint64_t pol) {
    unsigned short v;
    asm("ld.global.nc.L1::no_allocate.L2::cache_hint.L2::256B.u16 %0, [%1], %2;"
        : "=h"(v) : "l"(p), "l"(pol));
    return (int16_t)v;
}

// ----------------------------------------------------------------- reductions
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum `nv` per-thread values over the block into smem out[0..nv).  `red` is
// smem scratch of (blockDim.x/32) * nv doubles.  Fixed order: deterministic.
// The in-warp tree runs in T (FP32 values stay off GB300's narrow FP64
// pipe); the warp sums are combined in FP64.
template <int NVMAX, class T>
__device__ __forceinline__ void block_sum_multi(const T (&v)[NVMAX], int nv, double* red,
                                                double* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NVMAX; ++k) {
        if (k < nv) {
            const double s = (double)warp_sum(v[k]);
            if (lane == 0) red[warp * nv + k] = s;
        }
    }
    __syncthreads();
    for (int k = threadIdx.x; k < nv; k += blockDim.x) {
        double s = 0.0;
        for (int w = 0; w < nw; ++w) s += red[w * nv + k];
        out[k] = s;
    }
    __syncthreads();
}

// z = sum_q row[q] * r0[q] (the coarse term of a subdomain) summed by warp 0
// in an order that does not depend on the block size, so every sweep variant
// and block size gives the same bits: four lane-strided accumulators, then
// the shuffle tree.  Call from the threads of warp 0 only.
// (r0 through L2 when other blocks of the same launch wrote it)
template <bool CG = false>
__device__ __forceinline__ double coarse_dot_warp0(const double* __restrict__ row,
                                                   const double* __restrict__ r0, int nc) {
    const int lane = threadIdx.x & 31;
    auto ld = [&](int q) { return CG ? __ldcg(&r0[q]) : r0[q]; };
    double a0 = 0.0, a1 = 0.0, a2 = 0.0, a3 = 0.0;
    for (int q = lane; q < nc; q += 128) {
        a0 += row[q] * ld(q);
        if (q + 32 < nc) a1 += row[q + 32] * ld(q + 32);
        if (q + 64 < nc) a2 += row[q + 64] * ld(q + 64);
        if (q + 96 < nc) a3 += row[q + 96] * ld(q + 96);
    }
    return warp_sum((a0 + a1) + (a2 + a3));
}

// --------------------------------------------------------- coarse restriction
// sum_q x[owned[q]] over one subdomain's owned rows, in an order that does
// not depend on the block size: chunks of RC_CHUNK positions, each summed by
// one warp (lane l takes positions l, l+32, ... of the chunk into four
// accumulators in the input precision, combined pairwise, then the shuffle
// tree; FP64 from the warp sum on), chunk sums added in chunk order.  Every
// thread of the block calls it; the result is valid in thread 0.  red:
// shared scratch of RC_MAXCH doubles.
constexpr int RC_CHUNK = 1024;
constexpr int RC_MAXCH = 64;

template <class TI>
__device__ __forceinline__ double restrict_chunks(const int* __restrict__ owned,
                                                  const TI* __restrict__ x, int n_own,
                                                  double* red) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nch = (n_own + RC_CHUNK - 1) / RC_CHUNK;
    double total = 0.0;
    for (int c0 = 0; c0 < nch; c0 += RC_MAXCH) {
        const int cend = nch < c0 + RC_MAXCH ? nch : c0 + RC_MAXCH;
        for (int c = c0 + warp; c < cend; c += nw) {
            const int p0 = c * RC_CHUNK;
            TI a[4] = {(TI)0, (TI)0, (TI)0, (TI)0};
            for (int i0 = 0; i0 < RC_CHUNK / 32; i0 += 8) {
                int idx[8];
                TI v[8];
#pragma unroll
                for (int u = 0; u < 8; ++u) {
                    const int p = p0 + lane + 32 * (i0 + u);
                    idx[u] = p < n_own ? owned[p] : -1;
                }
#pragma unroll
                for (int u = 0; u < 8; ++u) v[u] = idx[u] >= 0 ? x[idx[u]] : (TI)0;
#pragma unroll
                for (int u = 0; u < 8; ++u) a[u & 3] += v[u];
            }
            const double sum = (double)warp_sum((a[0] + a[1]) + (a[2] + a[3]));
            if (lane == 0) red[c - c0] = sum;
        }
        __syncthreads();
        if (threadIdx.x == 0)
            for (int c = c0; c < cend; ++c) total += red[c - c0];
        __syncthreads();
    }
    return total;
}

// ------------------------------------------------------- subdomain gather/scatter
// Restriction x -> t over the n subdomain rows (t[tslot(li)] = x[dof[li]])
// and the restricted prolongation of the owned rows (y[og[q]] =
// t[tslot(ol[q])] (+ zc)); tslot with shift p (0: the identity).  `bs`
// threads of the block take part; each keeps eight independent index and
// value loads in flight, which the latency of a cold gather needs.
constexpr int SUB_ILP = 8;

template <class TS, class TI, int ILP = SUB_ILP>
__device__ __forceinline__ void gather_rows(TS* t, const TI* __restrict__ x,
                                            const int* __restrict__ dof, int n, int bs,
                                            int p = 0) {
    int li = threadIdx.x;
    for (; li + (ILP - 1) * bs < n; li += ILP * bs) {
        int d[ILP];
#pragma unroll
        for (int u = 0; u < ILP; ++u) d[u] = dof[li + u * bs];
        TI v[ILP];
#pragma unroll
        for (int u = 0; u < ILP; ++u) v[u] = x[d[u]];
#pragma unroll
        for (int u = 0; u < ILP; ++u) t[tslot(li + u * bs, p)] = Load<TS>::f(v[u]);
    }
    for (; li < n; li += bs) t[tslot(li, p)] = Load<TS>::f(x[dof[li]]);
}

// The coarse correction added to an owned row, in the precision of the
// output: FP64 output adds in FP64 with the reference's rounding; FP32 output
// adds (float)zc in FP32 (the sum is rounded to FP32 either way, and FP64
// arithmetic per row would run on GB300's narrow FP64 pipe).
template <class TO>
struct CoarseAdd;
template <>
struct CoarseAdd<double> {
    double z;
    __device__ __forceinline__ explicit CoarseAdd(double zc) : z(zc) {}
    template <class TS>
    __device__ __forceinline__ double operator()(TS v) const { return __dadd_rn((double)v, z); }
};
template <>
struct CoarseAdd<float> {
    float z;
    __device__ __forceinline__ explicit CoarseAdd(double zc) : z((float)zc) {}
    template <class TS>
    __device__ __forceinline__ float operator()(TS v) const { return Store<float>::f(v) + z; }
};

template <class TS, class TO>
__device__ __forceinline__ void scatter_owned(const TS* t, TO* __restrict__ y,
                                              const int* __restrict__ ol,
                                              const int* __restrict__ og, int n_own, int coarse,
                                              double zc, int bs, int p = 0) {
    const CoarseAdd<TO> add(zc);
    int q = threadIdx.x;
    for (; q + (SUB_ILP - 1) * bs < n_own; q += SUB_ILP * bs) {
        int l[SUB_ILP], g[SUB_ILP];
#pragma unroll
        for (int u = 0; u < SUB_ILP; ++u) {
            l[u] = ol[q + u * bs];
            g[u] = og[q + u * bs];
        }
#pragma unroll
        for (int u = 0; u < SUB_ILP; ++u) {
            const TS v = t[tslot(l[u], p)];
            y[g[u]] = coarse ? add(v) : Store<TO>::f(v);
        }
    }
    for (; q < n_own; q += bs) {
        const TS v = t[tslot(ol[q], p)];
        y[og[q]] = coarse ? add(v) : Store<TO>::f(v);
    }
}

// Grid-level completion of a reduction: every block stores its nv block sums
// (bsum, smem) into partials[block*nv + k]; the last block to arrive sums
// them in block order (deterministic) into smem `out` and returns true.  The
// arrival counter is reset by the last block, so consecutive kernels on one
// stream can share it.  No block waits for another.
struct NoPrefetch {
    __device__ __forceinline__ void operator()() const {}
};
// prefetch: run by the last block before it loads the partials (loads of
// what its epilogue needs, so both rounds of loads are in flight together;
// the results are visible to the block when this returns true)
template <class Prefetch = NoPrefetch>
__device__ __forceinline__ bool last_block_reduce(double* partials, unsigned* counter,
                                                  const double* bsum, int nv, double* out,
                                                  Prefetch prefetch = Prefetch()) {
    __shared__ unsigned s_ticket;
    for (int k = threadIdx.x; k < nv; k += blockDim.x)
        partials[(size_t)blockIdx.x * nv + k] = bsum[k];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(counter, 1u);
    __syncthreads();
    if (s_ticket != gridDim.x - 1) return false;
    __threadfence();
    prefetch();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nb = gridDim.x;
    // per lane the partials are added in block order, as a plain loop would;
    // the loads run ahead: sixteen per lane for one value per warp, else
    // four values k = k0 + nw * kk per warp with four partials each
    if (nv <= nw) {
        if (warp < nv) {
            double s = 0.0;
            for (int b0 = lane; b0 < nb; b0 += 32 * 16) {
                double v[16];
#pragma unroll
                for (int r = 0; r < 16; ++r) {
                    const int b = b0 + 32 * r;
                    v[r] = b < nb ? __ldcg(&partials[(size_t)b * nv + warp]) : 0.0;
                }
#pragma unroll
                for (int r = 0; r < 16; ++r)
                    if (b0 + 32 * r < nb) s += v[r];
            }
            s = warp_sum(s);
            if (lane == 0) out[warp] = s;
        }
    } else for (int k0 = warp; k0 < nv; k0 += 4 * nw) {
        double s[4] = {0.0, 0.0, 0.0, 0.0};
        for (int b0 = lane; b0 < nb; b0 += 32 * 4) {
            double v[4][4];
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int r = 0; r < 4; ++r) {
                    const int b = b0 + 32 * r, k = k0 + nw * kk;
                    v[kk][r] = (b < nb && k < nv) ? __ldcg(&partials[(size_t)b * nv + k]) : 0.0;
                }
#pragma unroll
            for (int kk = 0; kk < 4; ++kk)
#pragma unroll
                for (int r = 0; r < 4; ++r)
                    if (b0 + 32 * r < nb) s[kk] += v[kk][r];
        }
#pragma unroll
        for (int kk = 0; kk < 4; ++kk) {
            const double t = warp_sum(s[kk]);
            if (lane == 0 && k0 + nw * kk < nv) out[k0 + nw * kk] = t;
        }
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

}  // namespace sg
