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

// ----------------------------------------------------------------- reductions
template <class T>
__device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

// Sum `nv` per-thread values over the block into smem out[0..nv).  `red` is
// smem scratch of (blockDim.x/32) * nv doubles.  Fixed order: deterministic.
template <int NVMAX, class T>
__device__ __forceinline__ void block_sum_multi(const T (&v)[NVMAX], int nv, double* red,
                                                double* out) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int k = 0; k < NVMAX; ++k) {
        if (k < nv) {
            double s = warp_sum((double)v[k]);
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

// Grid-level completion of a reduction: every block stores its nv block sums
// (bsum, smem) into partials[block*nv + k]; the last block to arrive sums
// them in block order (deterministic) into smem `out` and returns true.  The
// arrival counter is reset by the last block, so consecutive kernels on one
// stream can share it.  No block waits for another.
__device__ __forceinline__ bool last_block_reduce(double* partials, unsigned* counter,
                                                  const double* bsum, int nv, double* out) {
    __shared__ unsigned s_ticket;
    for (int k = threadIdx.x; k < nv; k += blockDim.x)
        partials[(size_t)blockIdx.x * nv + k] = bsum[k];
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) s_ticket = atomicAdd(counter, 1u);
    __syncthreads();
    if (s_ticket != gridDim.x - 1) return false;
    __threadfence();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    const int nb = gridDim.x;
    for (int k = warp; k < nv; k += nw) {
        double s = 0.0;
#pragma unroll 8
        for (int b = lane; b < nb; b += 32) s += __ldcg(&partials[(size_t)b * nv + k]);
        s = warp_sum(s);
        if (lane == 0) out[k] = s;
    }
    __syncthreads();
    if (threadIdx.x == 0) *counter = 0u;
    return true;
}

}  // namespace sg
