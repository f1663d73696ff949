// learned.cu -- the learned coarse-correction stage (no counterpart in the
// reference).  Attached to a Schwarz preconditioner M it turns the apply into
//
//   z1 = M v                                  (two-level RAS etc.)
//   r1 = v - A z1                             (what M left unresolved)
//   s  = rms(R r1)
//   z  = z1 + s * c * P( CNN( [R r1 / s, f] ) )
//
//   R   restriction to the half-resolution grid (mean of the 2x2x2 children)
//   f   the coefficient feature: restricted log A_ii, standardised
//   CNN 4 layers of 3x3x3 convolutions, 16 channels, ReLU after layers 1-3,
//       BF16 weights and activations, FP32 accumulation, output channel 0
//   c   output scale (rms of the training targets)
//   P   cell-centred trilinear prolongation back to the fine grid
//
// The network is trained on (residual r, error e = A^{-1} r) pairs of plain
// solves to predict the error left after M, e1 = e - M r, in the energy norm
// of A: loss = ||e1/s - c P y||_A^2 / ||e1/s||_A^2 (the criterion a Galerkin
// coarse correction minimises; a coarse-MSE loss, also available, lets rough
// prediction errors blow up the fine-grid residual).  Scaling by s makes
// the stage positively homogeneous (FGMRES applies it to unnormalised
// vectors); the stage is nonlinear, so it runs inside FGMRES only.  A device
// monitor after every restart cycle switches the stage off for the rest of
// the solve when the cycle reduced the FP64 true residual by less than the
// stagnation ratio -- the plain preconditioner is the fallback.
//
// Every layer is an implicit GEMM on the tensor cores.  The forward layers
// and the input gradient run on tcgen05.mma (BF16 x BF16 -> FP32 in tensor
// memory): a CTA owns an 8 x 16 x 2 block of output voxels, TMA stages its
// 10 x 18 x 4 input halo (16 channels as two 8-channel planes) and a bulk copy
// the layer's weights, and one thread issues the MMAs straight from the
// shifted halo, one per (dy, dx) tap pair and halo slice (k_conv3d_tc).  The input
// gradient is the same kernel with flipped, transposed weights and the ReLU
// mask of the layer input in the epilogue.  The weight gradient (M = 16 input
// channels, below the 64 rows a tcgen05.mma needs; N = output channel, K =
// the tile's voxels) is an mma.sync kernel whose per-CTA partials a reduction
// kernel adds in a fixed order.  Channels are padded to 16 everywhere (layer
// 1 reads 2, layer 4 writes 1); padded weights stay 0.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <type_traits>
#include <vector>

#include "dev_common.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace sg {

constexpr int LC = 16;                    // channels (padded)
constexpr int LTAPS = 27;
constexpr int LAYER_W = LTAPS * LC * LC;  // weights of one layer, master layout [tap][ci][co]
constexpr int LAYER_P = LAYER_W + LC;     // + bias
constexpr int NLAYERS = 4;
constexpr int NET_PARAMS = NLAYERS * LAYER_P;
constexpr int LEARN_PARAMS = NET_PARAMS + 1;  // + output scale c

// device control block of one learned stage
struct LearnedCtl {
    float snorm;         // s of the current apply
    float out_scale;     // c
    int enabled;         // 0: the stage is skipped (fallback or switched off)
    int fallback_cycle;  // restart cycle after which the monitor switched it off (-1)
    double prev_rnorm;   // true residual at the previous cycle end
    double stag;         // stagnation ratio of the monitor (0: no monitor)
    unsigned long long applies;
    float pair_s;        // s of the last training pair
    float scratch_s;
};

namespace {

constexpr int CT = 256;  // threads of the weight-gradient kernel (8 warps)
constexpr int TB = 8;    // output tile edge
constexpr int HB = TB + 2;
constexpr int HALO_U32 = HB * HB * HB * 8;
constexpr int TILE_U32 = TB * TB * TB * 8;
constexpr int WGRAD_SMEM = (HALO_U32 + TILE_U32) * 4 + CT * 4;

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const uint32_t*>(&v);
}
__device__ __forceinline__ float bf_lo(uint32_t v) { return __uint_as_float(v << 16); }
__device__ __forceinline__ float bf_hi(uint32_t v) { return __uint_as_float(v & 0xffff0000u); }

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4],
                                         const uint32_t (&b)[2]) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
        "{%8,%9}, {%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

enum { EPI_RELU = 0, EPI_LINEAR_F32 = 1, EPI_MASK = 2 };

__device__ __forceinline__ bool skip(const int* enabled, const int* active) {
    return (active && *active == 0) || (enabled && *enabled == 0);
}

// Loads the 10x10x10 halo of the tile at (z0,y0,x0) of a [D][D][D][16] BF16
// volume (zero outside) into smem as uint32 channel pairs: halo[v*8 + pair].
__device__ __forceinline__ void load_halo(uint32_t* halo, const uint32_t* __restrict__ in, int D,
                                          int z0, int y0, int x0) {
    for (int q = threadIdx.x; q < HB * HB * HB * 2; q += blockDim.x) {
        const int v = q >> 1, half = q & 1;
        const int hz = v / (HB * HB), hy = (v / HB) % HB, hx = v % HB;
        const int z = z0 + hz - 1, y = y0 + hy - 1, x = x0 + hx - 1;
        uint4 val = make_uint4(0, 0, 0, 0);
        if (z >= 0 && z < D && y >= 0 && y < D && x >= 0 && x < D)
            val = reinterpret_cast<const uint4*>(in)[(((size_t)z * D + y) * D + x) * 2 + half];
        reinterpret_cast<uint4*>(halo)[q] = val;
    }
}

// ---- the convolution layers on the 5th-generation tensor cores
//
// One CTA computes an output tile of 8 (x) x 16 (y) x 2 (z) voxels as two
// GEMMs of M = 128 rows (the (y, x) positions of one z-plane), N = 16 output
// channels and K = 27 taps x 16 input channels, accumulated in tensor memory
// (two 128-lane x 16-column FP32 accumulators).  TMA copies the tile's
// 10 x 18 x 4 input halo into shared memory as two 8-channel planes (16 B
// per voxel each; the tensor map fills the voxels outside the volume with 0)
// and a bulk copy brings the layer's weights, already in the operand layout.
// With that layout the A operand of tap (dz, dy, dx) is the halo slice of
// its dz shifted by (dy, dx) -- eight consecutive x positions are one 8-row x
// 16-byte core matrix, the 16 rows of y are 8-row groups 18 x 16 B apart,
// the second channel half is the other plane -- so no operand is ever copied
// or re-laid out in shared memory, and one A tile serves every dz tap whose
// output plane lies in the tile: one tcgen05.mma of N = 16 or 32 per (dy,
// dx) pair and halo slice, 36 in all, each reading its 4 KB A tile once.
// One thread issues them and commits them to an mbarrier; each warp then
// reads its 32 accumulator lanes (tcgen05.ld) and runs the epilogue.
// (Two z-planes per CTA rather than four: 2.8 CTAs per SM at 48^3 instead
// of 1.4 balance the SMs better, measured 0.7 us faster per layer.)
constexpr int TC_TY = 16, TC_TZ = 2;
constexpr int TC_HX = TB + 2, TC_HY = TC_TY + 2, TC_HZ = TC_TZ + 2;
constexpr int TC_PLANE = TC_HX * TC_HY * TC_HZ * 16;  // one 8-channel half of the halo
constexpr int TC_WBYTES = LTAPS * LC * LC * 2;        // one layer's BF16 weights
constexpr int TC_OFF_W = 2 * TC_PLANE;
constexpr int TC_OFF_BAR = TC_OFF_W + TC_WBYTES;
constexpr int TC_SMEM = TC_OFF_BAR + 32 + 128;        // + barriers and words, + alignment slack
constexpr int TC_THREADS = 128;                       // warp w reads accumulator lanes 32w..32w+31
constexpr int TC_COLS = TC_TZ * LC;                   // tensor-memory columns (a power of 2, >= 32)
static_assert(TC_PLANE % 128 == 0 && TC_OFF_W % 128 == 0 && TC_OFF_BAR % 16 == 0,
              "TMA destinations and mbarriers must stay aligned");
static_assert(TC_COLS >= 32 && (TC_COLS & (TC_COLS - 1)) == 0,
              "tensor-memory allocation must be a power of two >= 32");

// instruction descriptor of tcgen05.mma kind::f16: FP32 accumulator (bits
// 4-5 = 1), BF16 A and B (bits 7-9, 10-12 = 1), both K-major (bits 15, 16 =
// 0), N >> 3 in bits 17-22, M >> 4 in bits 24-28
constexpr uint32_t tc_idesc(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
           ((uint32_t)(M >> 4) << 24);
}
// one MMA per (dy, dx) tap pair and halo slice covers the dz taps whose
// output planes lie in the tile: N = 16 output channels per tap (16 or 32)
constexpr uint32_t TC_IDESC16 = tc_idesc(128, LC);
constexpr uint32_t TC_IDESC32 = tc_idesc(128, 2 * LC);
static_assert(TC_TZ == 2, "the MMA order below initialises both planes' accumulators first");

// shared-memory operand descriptor, no swizzle, K-major: start address,
// byte offset between the two K-adjacent core matrices (lbo) and between
// M/N-adjacent 8-row groups (sbo), all in 16-byte units; bit 46 is the
// descriptor version of this architecture
__device__ __forceinline__ uint64_t tc_sdesc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}
__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// whole warp: allocate `cols` tensor-memory columns, address into smem slot
__device__ __forceinline__ void tc_alloc(uint32_t slot, uint32_t cols) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(slot),
                 "r"(cols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tc_dealloc(uint32_t taddr, uint32_t cols) {
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(taddr), "r"(cols)
                 : "memory");
}
// D[taddr] (+)= A * B^T, one thread
__device__ __forceinline__ void tc_mma(uint32_t taddr, uint64_t a, uint64_t b, uint32_t idesc,
                                       uint32_t accumulate) {
    asm volatile(
        "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
        " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(taddr),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}
// arrive on the mbarrier once every MMA this thread issued has completed
__device__ __forceinline__ void tc_commit(uint32_t bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
        : "memory");
}
// whole warp: 16 consecutive FP32 columns of this thread's accumulator lane
__device__ __forceinline__ void tc_ld16(uint32_t taddr, float (&v)[16]) {
    uint32_t r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
        "%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]),
          "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// conv3d 3x3x3, 16 -> 16 channels.  in_map: the BF16 [batch][D][D][D][16]
// input as a 5D tensor map (box 8 ch x 10 x 18 x 4 x 1).  w: the layer's
// weights in operand layout ([(dy, dx)][ci / 8][dz * 16 + co][ci % 8],
// 1,536 B per (dy, dx) pair).
// Grid: (D/8) x ceil(D/16) x (D/2) tiles x batch.  Epilogues:
//  RELU        out = relu(acc + bias) as BF16 [V][16]
//  LINEAR_F32  outf[v] = acc[ch 0] + bias[0] (FP32, one channel)
//  MASK        out = acc * (mask[v][ch] > 0) as BF16 (input gradient; no bias)
// A wait that runs out of its budget sets *err, drains what is in flight and
// leaves the tile's output unwritten.
__global__ void __launch_bounds__(TC_THREADS)
k_conv3d_tc(const __grid_constant__ CUtensorMap in_map, const uint8_t* __restrict__ w,
            const float* __restrict__ bias, int D, int epi, uint32_t* __restrict__ out,
            float* __restrict__ outf, const uint32_t* __restrict__ mask, const int* enabled,
            const int* active, int* err, int wait_test, const float* __restrict__ fin_rc,
            const float* __restrict__ fin_feat, const float* __restrict__ fin_s) {
    if (skip(enabled, active)) return;
    // wait_test 1 / 2 (testing of the give-up path): the copy barrier expects
    // 16 bytes nobody sends / the MMA barrier one arrival nobody makes, so
    // its wait runs out (short budget); the block then supplies what it
    // withheld and drains the real copies / MMAs with the full budget
    const bool t1 = wait_test == 1, t2 = wait_test == 2;
    extern __shared__ uint8_t tc_raw[];
    const uint32_t raw = smem_u32(tc_raw);
    const uint32_t base = (raw + 127u) & ~127u;
    uint8_t* sm = tc_raw + (base - raw);
    const uint32_t plane0 = base, wsm = base + TC_OFF_W;
    const uint32_t bar_in = base + TC_OFF_BAR, bar_mma = bar_in + 8;
    uint32_t* s_taddr = reinterpret_cast<uint32_t*>(sm + TC_OFF_BAR + 16);
    volatile int* s_bad = reinterpret_cast<volatile int*>(sm + TC_OFF_BAR + 20);

    const int ntx = D / TB, nty = (D + TC_TY - 1) / TC_TY, ntz = D / TC_TZ;
    int t = blockIdx.x;
    const int tx = t % ntx;
    t /= ntx;
    const int ty = t % nty;
    t /= nty;
    const int tz = t % ntz, b = t / ntz;
    const int x0 = tx * TB, y0 = ty * TC_TY, z0 = tz * TC_TZ;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

    // the copies go out first; the tensor-memory allocation and the block
    // barrier overlap their latency
    const bool fields = fin_rc != nullptr;
    if (threadIdx.x == 0) {
        *s_bad = 0;
        mbar_init(bar_in, 1);
        mbar_init(bar_mma, t2 ? 2 : 1);
        fence_mbar_init();
        mbar_expect_tx(bar_in, (fields ? 0 : 2 * TC_PLANE) + TC_WBYTES + (t1 ? 16 : 0));
        if (!fields) {
            tma_load_5d(plane0, &in_map, 0, x0 - 1, y0 - 1, z0 - 1, b, bar_in);
            tma_load_5d(plane0 + TC_PLANE, &in_map, 8, x0 - 1, y0 - 1, z0 - 1, b, bar_in);
        }
        bulk_g2s(wsm, w, TC_WBYTES, bar_in);
    }
    if (fields) {
        // the first layer of an apply packs its own input into the halo
        // planes: channel 0 = rc / s, channel 1 = the coefficient feature,
        // the rest 0 (one sample, read straight from rc and f), written by
        // the threads and fenced for the tensor cores' (async proxy) reads
        const float sv = *fin_s;
        const float inv = sv > 0.f ? 1.f / sv : 0.f;
        for (int q = threadIdx.x; q < TC_HX * TC_HY * TC_HZ; q += blockDim.x) {
            const int hx = q % TC_HX, hy = (q / TC_HX) % TC_HY, hz = q / (TC_HX * TC_HY);
            const int x = x0 - 1 + hx, y = y0 - 1 + hy, z = z0 - 1 + hz;
            uint32_t c01 = 0u;
            if (x >= 0 && x < D && y >= 0 && y < D && z >= 0 && z < D) {
                const size_t v = ((size_t)z * D + y) * D + x;
                c01 = pack_bf16(fin_rc[v] * inv, fin_feat[v]);
            }
            *reinterpret_cast<uint4*>(sm + (size_t)q * 16) = make_uint4(c01, 0u, 0u, 0u);
            *reinterpret_cast<uint4*>(sm + TC_PLANE + (size_t)q * 16) = make_uint4(0u, 0u, 0u, 0u);
        }
        fence_proxy_async();
    }
    if (warp == 0) {
        __syncwarp();
        tc_alloc(smem_u32(s_taddr), TC_COLS);
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t taddr = *s_taddr;

    if (threadIdx.x == 0) {
        int bad = 0;
        if (mbar_wait(bar_in, 0, t1 ? WAIT_TEST_CYCLES : WAIT_CYCLES)) {
            tc_fence_after();
            // halo slice h feeds output plane z = h - 1 - dz: the taps dz of
            // one (dy, dx) that land in the tile are adjacent rows of the
            // weight block and, with the planes' accumulators in descending
            // order (plane z at columns (TZ - 1 - z) * 16), adjacent columns
            // of tensor memory -- one MMA of N = 16 per tap.  Slice 1 goes
            // first: it writes both planes, so later MMAs all accumulate.
            constexpr int order[TC_TZ + 2] = {1, 0, 2, 3};
            for (int c = 0; c < 9; ++c) {
                const int dy = c / 3 - 1, dx = c % 3 - 1;
#pragma unroll
                for (int q = 0; q < TC_TZ + 2; ++q) {
                    const int h = order[q];
                    const int lo = h - TC_TZ + 1 > 0 ? h - TC_TZ + 1 : 0, hi = h < 2 ? h : 2;
                    const uint32_t a = plane0 + ((h * TC_HY + 1 + dy) * TC_HX + 1 + dx) * 16;
                    tc_mma(taddr + (uint32_t)((TC_TZ - 1 - (h - lo)) * LC),
                           tc_sdesc(a, TC_PLANE, TC_HX * 16),
                           tc_sdesc(wsm + c * 1536 + lo * 256, 768, 128),
                           hi > lo ? TC_IDESC32 : TC_IDESC16, (c > 0 || q > 0) ? 1u : 0u);
                }
            }
            tc_commit(bar_mma);
            if (!mbar_wait(bar_mma, 0, t2 ? WAIT_TEST_CYCLES : WAIT_CYCLES)) {
                bad = 2;
                if (t2) mbar_arrive(bar_mma);
                mbar_wait(bar_mma, 0, WAIT_CYCLES);  // let the MMAs finish before TMEM is freed
            }
        } else {
            bad = 1;
            if (t1) mbar_complete_tx(bar_in, 16);
            mbar_wait(bar_in, 0, WAIT_CYCLES);  // the copies may still land: wait once more
        }
        if (bad) {
            *s_bad = bad;
            atomicExch(err, bad);
        }
    }
    __syncthreads();
    tc_fence_after();
    if (*s_bad == 0) {
        const int m = warp * 32 + lane;  // accumulator lane = GEMM row = (y, x) in the z-plane
        const int yy = y0 + (m >> 3), xx = x0 + (m & 7);
        const size_t V = (size_t)D * D * D;
#pragma unroll 1
        for (int mt = 0; mt < TC_TZ; ++mt) {
            float acc[16];
            tc_ld16(taddr + ((uint32_t)(warp * 32) << 16) + (uint32_t)((TC_TZ - 1 - mt) * LC), acc);
            if (yy >= D) continue;
            const size_t v = (size_t)b * V + ((size_t)(z0 + mt) * D + yy) * D + xx;
            if (epi == EPI_LINEAR_F32) {
                outf[v] = acc[0] + bias[0];
                continue;
            }
            uint32_t pk[8];
            if (epi == EPI_RELU) {
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    pk[c] = pack_bf16(fmaxf(acc[2 * c] + bias[2 * c], 0.f),
                                      fmaxf(acc[2 * c + 1] + bias[2 * c + 1], 0.f));
            } else {
                const uint4 m0 = reinterpret_cast<const uint4*>(mask + v * 8)[0];
                const uint4 m1 = reinterpret_cast<const uint4*>(mask + v * 8)[1];
                const uint32_t mw[8] = {m0.x, m0.y, m0.z, m0.w, m1.x, m1.y, m1.z, m1.w};
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    pk[c] = pack_bf16(bf_lo(mw[c]) > 0.f ? acc[2 * c] : 0.f,
                                      bf_hi(mw[c]) > 0.f ? acc[2 * c + 1] : 0.f);
            }
            uint4* o = reinterpret_cast<uint4*>(out + v * 8);
            o[0] = make_uint4(pk[0], pk[1], pk[2], pk[3]);
            o[1] = make_uint4(pk[4], pk[5], pk[6], pk[7]);
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 0) {
        tc_fence_after();
        tc_dealloc(taddr, TC_COLS);
    }
}

// Weight-gradient partials of one tile: dW[tap][ci][co] = sum over the tile's
// voxels v of X[v + off(tap)][ci] * G[v][co]; dB[co] = sum_v G[v][co].
// mma with M = ci (16), N = co (2 x 8), K = voxels (16 per step).  Dynamic
// smem: halo | G tile | bias scratch.
__global__ void __launch_bounds__(CT)
k_conv3d_wgrad(const uint32_t* __restrict__ X, const uint32_t* __restrict__ G, int D,
               float* __restrict__ part) {
    extern __shared__ __align__(16) uint32_t wsm[];
    uint32_t* halo = wsm;
    uint32_t* gt = wsm + HALO_U32;
    float* bred = reinterpret_cast<float*>(wsm + HALO_U32 + TILE_U32);
    const int tiles = D / TB;
    const int nt3 = tiles * tiles * tiles;
    const int b = blockIdx.x / nt3;
    const int t = blockIdx.x % nt3;
    const int z0 = (t / (tiles * tiles)) * TB, y0 = ((t / tiles) % tiles) * TB, x0 = (t % tiles) * TB;
    const size_t V = (size_t)D * D * D;
    load_halo(halo, X + (size_t)b * V * 8, D, z0, y0, x0);
    for (int q = threadIdx.x; q < TB * TB * TB * 2; q += blockDim.x) {
        const int v = q >> 1, half = q & 1;
        const int vz = v / (TB * TB), vy = (v / TB) % TB, vx = v % TB;
        const size_t gv = ((size_t)(z0 + vz) * D + (y0 + vy)) * D + (x0 + vx);
        reinterpret_cast<uint4*>(gt)[q] =
            reinterpret_cast<const uint4*>(G)[((size_t)b * V + gv) * 2 + half];
    }
    __syncthreads();
    const unsigned short* hs = reinterpret_cast<const unsigned short*>(halo);
    const unsigned short* gs = reinterpret_cast<const unsigned short*>(gt);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int g = lane >> 2, tg = lane & 3;
    float* pb = part + (size_t)blockIdx.x * LAYER_P;
    for (int tap = warp; tap < LTAPS; tap += CT / 32) {
        const int dz = tap / 9 - 1, dy = (tap / 3) % 3 - 1, dx = tap % 3 - 1;
        float acc[2][4] = {{0.f, 0.f, 0.f, 0.f}, {0.f, 0.f, 0.f, 0.f}};
        for (int ks = 0; ks < TB * TB * TB / 16; ++ks) {
            // K index kk in [0,16): voxel 16 ks + kk of the tile; 16 voxels =
            // two x-runs of 8 (rows y = 2(ks%4), +1 of plane z = ks/4)
            const int vz = ks >> 2, vy = 2 * (ks & 3);
            const int base = (vz + 1 + dz) * HB * HB + (vy + 1 + dy) * HB + (1 + dx);
            const int k0 = 2 * tg;  // columns k0, k0+1 (first run), k0+8, k0+9 (second)
            const int ha = base + k0, hc = base + HB + k0;
            uint32_t af[4];
            af[0] = (uint32_t)hs[ha * 16 + g] | ((uint32_t)hs[(ha + 1) * 16 + g] << 16);
            af[1] = (uint32_t)hs[ha * 16 + g + 8] | ((uint32_t)hs[(ha + 1) * 16 + g + 8] << 16);
            af[2] = (uint32_t)hs[hc * 16 + g] | ((uint32_t)hs[(hc + 1) * 16 + g] << 16);
            af[3] = (uint32_t)hs[hc * 16 + g + 8] | ((uint32_t)hs[(hc + 1) * 16 + g + 8] << 16);
            const int va = 16 * ks + k0, vc = va + 8;
#pragma unroll
            for (int nt = 0; nt < 2; ++nt) {
                const int co = nt * 8 + g;
                uint32_t bf[2];
                bf[0] = (uint32_t)gs[va * 16 + co] | ((uint32_t)gs[(va + 1) * 16 + co] << 16);
                bf[1] = (uint32_t)gs[vc * 16 + co] | ((uint32_t)gs[(vc + 1) * 16 + co] << 16);
                mma_bf16(acc[nt], af, bf);
            }
        }
        // C: row = ci (g / g+8), column = co (nt*8 + 2tg, +1)
#pragma unroll
        for (int nt = 0; nt < 2; ++nt)
#pragma unroll
            for (int e = 0; e < 4; ++e) {
                const int ci = g + (e >= 2 ? 8 : 0);
                const int co = nt * 8 + 2 * tg + (e & 1);
                pb[(tap * LC + ci) * LC + co] = acc[nt][e];
            }
    }
    // bias gradient: 16 sums over the tile's 512 voxels (16 slices of 32)
    {
        const int co = threadIdx.x & 15, slice = threadIdx.x >> 4;
        float s = 0.f;
        for (int v = slice * 32; v < slice * 32 + 32; ++v)
            s += __uint_as_float((uint32_t)gs[v * 16 + co] << 16);
        bred[threadIdx.x] = s;
    }
    __syncthreads();
    if (threadIdx.x < LC) {
        float s = 0.f;
        for (int sl = 0; sl < CT / 16; ++sl) s += bred[sl * 16 + threadIdx.x];
        pb[LAYER_W + threadIdx.x] = s;
    }
}

// grad[i] = mask[i] * sum over CTAs of part[cta][i] (CTA order)
__global__ void k_wgrad_reduce(const float* __restrict__ part, int nblk,
                               const float* __restrict__ pmask, float* __restrict__ grad) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= LAYER_P) return;
    float s = 0.f;
    for (int c = 0; c < nblk; ++c) s += part[(size_t)c * LAYER_P + i];
    grad[i] = s * pmask[i];
}

// master FP32 [layer][tap][ci][co] -> the BF16 weights of the forward layers
// and the flipped, transposed weights of the input gradient (tap 26 - t,
// input and output channels swapped), both in the operand layout of
// k_conv3d_tc: per (dy, dx) pair c a 48 x 16 block -- rows dz-tap x output
// channel, columns input channel -- as two 8-input-channel halves of 48 rows
// of 8 channels ([c][k / 8][dz * 16 + n][k % 8], 1,536 bytes per pair)
__global__ void k_prep_weights(const float* __restrict__ master, __nv_bfloat16* __restrict__ wf,
                               __nv_bfloat16* __restrict__ wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= NLAYERS * LAYER_W) return;
    const int l = i / LAYER_W, r = i % LAYER_W;
    const int tap = r / (LC * LC), ci = (r / LC) % LC, co = r % LC;
    const __nv_bfloat16 v = __float2bfloat16_rn(master[(size_t)l * LAYER_P + r]);
    const size_t lb = (size_t)l * LAYER_W;
    const int tt = LTAPS - 1 - tap;
    wf[lb + (tap % 9) * 768 + (ci / 8) * 384 + ((tap / 9) * LC + co) * 8 + ci % 8] = v;
    wt[lb + (tt % 9) * 768 + (co / 8) * 384 + ((tt / 9) * LC + ci) * 8 + co % 8] = v;
}

// Adam (Kingma & Ba 2015) on the network parameters; padded entries stay 0
__global__ void k_adam(float* __restrict__ p, const float* __restrict__ grad,
                       float* __restrict__ m1, float* __restrict__ m2,
                       const float* __restrict__ pmask, int count, float lr, float b1, float b2,
                       float eps, float c1, float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= count) return;
    const float gr = grad[i];
    const float a = b1 * m1[i] + (1.f - b1) * gr;
    const float v = b2 * m2[i] + (1.f - b2) * gr * gr;
    m1[i] = a;
    m2[i] = v;
    p[i] = (p[i] - lr * (a / c1) / (sqrtf(v / c2) + eps)) * pmask[i];
}

// MSE over `count` outputs: loss += sum (Y - T)^2 / count (block sums added
// atomically -- reporting only); G[v] = (2 (Y - T) / count, 0, ..., 0) as BF16
__global__ void k_loss_grad(const float* __restrict__ Y, const float* __restrict__ T, size_t count,
                            uint32_t* __restrict__ G, float* __restrict__ loss) {
    float s = 0.f;
    const float inv = 1.f / (float)count;
    for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < count;
         i += (size_t)gridDim.x * blockDim.x) {
        const float d = Y[i] - T[i];
        s += d * d;
        if (G) {
            uint4* g4 = reinterpret_cast<uint4*>(G + i * 8);
            g4[0] = make_uint4(pack_bf16(2.f * d * inv, 0.f), 0u, 0u, 0u);
            g4[1] = make_uint4(0u, 0u, 0u, 0u);
        }
    }
    s = warp_sum(s);
    __shared__ float red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        atomicAdd(loss, t * inv);
    }
}

// rc[c] = mean over the 8 children f of c of (v[f] - az[f]) (az == nullptr:
// of v[f]), az = A z from the SpMV kernels; s_out = sqrt(mean rc^2).  TA:
// arithmetic of the residual rows.  A thread per coarse cell adds its
// children in the order x bit, y bit, z bit.
template <class TA, class TI, class TZ>
__global__ void __launch_bounds__(256)
k_resid_restrict(const TI* __restrict__ v, const TZ* __restrict__ az, int nx, int ny, int nz,
                 float* __restrict__ rc, double* partials, unsigned* counter, float* s_out,
                 const int* enabled, const int* active) {
    if (skip(enabled, active)) return;
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const int nc = cx * cy * cz;
    double ss = 0.0;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        const int i = c % cx, j = (c / cx) % cy, k = c / (cx * cy);
        TA r[8];
#pragma unroll
        for (int o = 0; o < 8; ++o) {
            const int f = ((2 * k + (o >> 2)) * ny + 2 * j + ((o >> 1) & 1)) * nx + 2 * i + (o & 1);
            r[o] = az ? (TA)v[f] - (TA)az[f] : (TA)v[f];
        }
        TA s = 0;
#pragma unroll
        for (int o = 0; o < 8; ++o) s += r[o];
        const float m = (float)(s * (TA)0.125);
        rc[c] = m;
        ss += (double)m * m;
    }
    __shared__ double red[8];
    __shared__ double bs[1], tot[1];
    double v1[1] = {ss};
    block_sum_multi<1>(v1, 1, red, bs);
    if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0)
        *s_out = (float)sqrt(tot[0] / (double)nc);
}

// packed inputs of a batch of stored samples (idx[b] = sample of batch entry
// b; idx == nullptr: entry b is sample b); targets scaled by inv_c
__global__ void k_pack_batch(const float* __restrict__ in, const float* __restrict__ feat,
                             const float* __restrict__ tgt, const int* __restrict__ idx, int batch,
                             int nc, float inv_c, uint32_t* __restrict__ X, float* __restrict__ T) {
    const size_t total = (size_t)batch * nc;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < total;
         q += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(q / nc), c = (int)(q % nc);
        const size_t src = (size_t)(idx ? idx[b] : b) * nc + c;
        uint4* x4 = reinterpret_cast<uint4*>(X + q * 8);
        x4[0] = make_uint4(pack_bf16(in[src], feat[src]), 0u, 0u, 0u);
        x4[1] = make_uint4(0u, 0u, 0u, 0u);
        if (T && tgt) T[q] = tgt[src] * inv_c;
    }
}

// cell-centred trilinear stencil along one axis: fine index fc -> coarse
// cells c = fc/2 (weight 3/4) and its neighbour towards fc (weight 1/4,
// clamped to the grid)
__device__ __forceinline__ void tri_axis(int fc, int nc, int (&id)[2]) {
    const int c = fc >> 1;
    const int o = (fc & 1) ? c + 1 : c - 1;
    id[0] = c;
    id[1] = o < 0 ? 0 : (o >= nc ? nc - 1 : o);
}

// z[f] += s * c * trilinear(Y)[f]
template <class TO>
__global__ void k_prolong_add(const float* __restrict__ Y, int nx, int ny, int nz,
                              LearnedCtl* ctl, const int* active, TO* __restrict__ z) {
    if (skip(&ctl->enabled, active)) return;
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const float sc = ctl->snorm * ctl->out_scale;
    const int n = nx * ny * nz;  // < 2^31 (checked at create)
    if (blockIdx.x == 0 && threadIdx.x == 0) ctl->applies += 1;
    const float w[2] = {0.75f, 0.25f};
    for (int f = blockIdx.x * blockDim.x + threadIdx.x; f < n; f += gridDim.x * blockDim.x) {
        const int fxy = f % (nx * ny);
        const int fx = fxy % nx, fy = fxy / nx, fz = f / (nx * ny);
        int ia[2], ja[2], ka[2];
        tri_axis(fx, cx, ia);
        tri_axis(fy, cy, ja);
        tri_axis(fz, cz, ka);
        float acc = 0.f;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int bb = 0; bb < 2; ++bb) {
                const float* row = Y + ((size_t)ka[a] * cy + ja[bb]) * cx;
                acc += w[a] * w[bb] * (0.75f * row[ia[0]] + 0.25f * row[ia[1]]);
            }
        z[f] = z[f] + (TO)(sc * acc);
    }
}

// training pair: in[slot] = rc / s, tgt[slot] = ec / s, feat[slot] = f
__global__ void k_store_pair(const float* __restrict__ rc, const float* __restrict__ ec,
                             const float* __restrict__ f, int nc, const LearnedCtl* ctl,
                             float* __restrict__ in, float* __restrict__ tgt,
                             float* __restrict__ feat) {
    const float s = ctl->pair_s;
    const float inv = s > 0.f ? 1.f / s : 0.f;
    for (int c = blockIdx.x * blockDim.x + threadIdx.x; c < nc; c += gridDim.x * blockDim.x) {
        in[c] = rc[c] * inv;
        tgt[c] = ec[c] * inv;
        feat[c] = f[c];
    }
}

// out = a - b (FP64)
__global__ void k_sub64(const double* __restrict__ a, const double* __restrict__ b, int n,
                        double* __restrict__ out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = a[i] - b[i];
}

// energy loss, step 1: u[b][f] = err[idx[b]][f] - c * P(Y[b])[f]
__global__ void k_energy_u(const float* __restrict__ err, const int* __restrict__ idx, int batch,
                           const float* __restrict__ Y, int nx, int ny, int nz, float c,
                           float* __restrict__ u) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const size_t n = (size_t)nx * ny * nz, ncc = (size_t)cx * cy * cz;
    const float w[2] = {0.75f, 0.25f};
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < n * batch;
         q += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(q / n);
        const size_t f = q % n;
        const int fx = (int)(f % nx), fy = (int)((f / nx) % ny), fz = (int)(f / ((size_t)nx * ny));
        int ia[2], ja[2], ka[2];
        tri_axis(fx, cx, ia);
        tri_axis(fy, cy, ja);
        tri_axis(fz, cz, ka);
        const float* Yb = Y + (size_t)b * ncc;
        float acc = 0.f;
#pragma unroll
        for (int a = 0; a < 2; ++a)
#pragma unroll
            for (int bb = 0; bb < 2; ++bb) {
                const float* row = Yb + ((size_t)ka[a] * cy + ja[bb]) * cx;
                acc += w[a] * w[bb] * (0.75f * row[ia[0]] + 0.25f * row[ia[1]]);
            }
        u[q] = err[(size_t)idx[b] * n + f] - c * acc;
    }
}

// energy loss, step 2: w[b] = A_{field(b)} u[b] (shared pattern, per-field
// FP32 values); loss += u.w / (energy_b * batch) (block sums added
// atomically -- reporting only).  blockIdx.y = batch entry.
__global__ void __launch_bounds__(256)
k_energy_spmv(const int* __restrict__ rp, const int* __restrict__ ci,
              const float* __restrict__ fvals, long long nnz, const int* __restrict__ sfield,
              const int* __restrict__ idx, const float* __restrict__ energy, int n, int batch,
              const float* __restrict__ u, float* __restrict__ w, float* __restrict__ loss) {
    const int b = blockIdx.y;
    const int smp = idx[b];
    const float* val = fvals + (size_t)sfield[smp] * nnz;
    const float* ub = u + (size_t)b * n;
    float* wb = w + (size_t)b * n;
    float s = 0.f;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        float acc = 0.f;
        for (int q = rp[i]; q < rp[i + 1]; ++q) acc += val[q] * ub[ci[q]];
        wb[i] = acc;
        s += acc * ub[i];
    }
    s = warp_sum(s);
    __shared__ float red[8];
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        float t = 0.f;
        for (int k = 0; k < (int)(blockDim.x >> 5); ++k) t += red[k];
        const float e = energy[smp];
        if (e > 0.f) atomicAdd(loss, t / (e * (float)batch));
    }
}

// adjoint of the trilinear prolongation along one axis: the fine points that
// coarse cell c contributes to, with their weights (returns the count)
__device__ __forceinline__ int tri_axis_t(int c, int nc, int (&f)[4], float (&wt)[4]) {
    int k = 0;
    f[k] = 2 * c;     wt[k++] = c == 0 ? 1.f : 0.75f;
    f[k] = 2 * c + 1; wt[k++] = c == nc - 1 ? 1.f : 0.75f;
    if (c >= 1) { f[k] = 2 * c - 1; wt[k++] = 0.25f; }
    if (c <= nc - 2) { f[k] = 2 * c + 2; wt[k++] = 0.25f; }
    return k;
}

// energy loss, step 3: G[b][c] = (-2 c / (energy_b * batch)) (P^T w_b)[c] in
// channel 0 (BF16), channels 1-15 zero
__global__ void k_energy_grad(const float* __restrict__ w, const int* __restrict__ idx,
                              const float* __restrict__ energy, int batch, int nx, int ny, int nz,
                              float c, uint32_t* __restrict__ G) {
    const int cx = nx / 2, cy = ny / 2, cz = nz / 2;
    const size_t n = (size_t)nx * ny * nz, ncc = (size_t)cx * cy * cz;
    for (size_t q = blockIdx.x * (size_t)blockDim.x + threadIdx.x; q < ncc * batch;
         q += (size_t)gridDim.x * blockDim.x) {
        const int b = (int)(q / ncc);
        const size_t cc = q % ncc;
        const int i = (int)(cc % cx), j = (int)((cc / cx) % cy), k = (int)(cc / ((size_t)cx * cy));
        int fi[4], fj[4], fk[4];
        float wi[4], wj[4], wk[4];
        const int ni = tri_axis_t(i, cx, fi, wi);
        const int nj = tri_axis_t(j, cy, fj, wj);
        const int nk = tri_axis_t(k, cz, fk, wk);
        const float* wb = w + (size_t)b * n;
        float acc = 0.f;
        for (int a = 0; a < nk; ++a)
            for (int bb = 0; bb < nj; ++bb) {
                const float* row = wb + ((size_t)fk[a] * ny + fj[bb]) * nx;
                float r = 0.f;
                for (int cc2 = 0; cc2 < ni; ++cc2) r += wi[cc2] * row[fi[cc2]];
                acc += wk[a] * wj[bb] * r;
            }
        const float e = energy[idx[b]];
        const float g = e > 0.f ? -2.f * c * acc / (e * (float)batch) : 0.f;
        uint4* g4 = reinterpret_cast<uint4*>(G + q * 8);
        g4[0] = make_uint4(pack_bf16(g, 0.f), 0u, 0u, 0u);
        g4[1] = make_uint4(0u, 0u, 0u, 0u);
    }
}

// FP32 copy of v * inv into out (the fine training target)
__global__ void k_scale_store(const double* __restrict__ v, int n, const LearnedCtl* ctl,
                              float* __restrict__ out) {
    const float s = ctl->pair_s;
    const double inv = s > 0.f ? 1.0 / (double)s : 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        out[i] = (float)(v[i] * inv);
}

// energy of the stored FP32 target: e^T A e with the field's FP32 values, in FP64
__global__ void __launch_bounds__(256)
k_energy_norm(const int* __restrict__ rp, const int* __restrict__ ci, const float* __restrict__ val,
              const float* __restrict__ e, int n, double* partials, unsigned* counter,
              float* __restrict__ out) {
    double s = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        double acc = 0.0;
        for (int q = rp[i]; q < rp[i + 1]; ++q) acc += (double)val[q] * (double)e[ci[q]];
        s += acc * (double)e[i];
    }
    __shared__ double red[8];
    __shared__ double bs[1], tot[1];
    double v1[1] = {s};
    block_sum_multi<1>(v1, 1, red, bs);
    if (last_block_reduce(partials, counter, bs, 1, tot) && threadIdx.x == 0) *out = (float)tot[0];
}

// solve start: stage on (unless switched off), monitor reference = initial residual
__global__ void k_learned_begin(LearnedCtl* ctl, const SolveState* st, int on) {
    ctl->enabled = on;
    ctl->fallback_cycle = -1;
    ctl->prev_rnorm = st->rnorm;
}

// after every restart cycle: switch the stage off when the cycle reduced the
// FP64 true residual by less than the stagnation ratio (or it is not finite)
__global__ void k_learned_monitor(LearnedCtl* ctl, const SolveState* st) {
    if (!ctl->enabled || (st->done && st->converged)) return;
    const double cur = st->rnorm;
    if (ctl->stag > 0.0 && !(cur <= ctl->stag * ctl->prev_rnorm)) {
        ctl->enabled = 0;
        ctl->fallback_cycle = st->cycles;
    }
    ctl->prev_rnorm = cur;
}

}  // namespace

// ============================================================ host side
struct LearnedImpl {
    sg_ctx* ctx = nullptr;
    uint64_t gen = 0;  // object generation, renewed by sg_learned_set_matrix
    int nx = 0, ny = 0, nz = 0, cx = 0, cy = 0, cz = 0;
    int nc = 0;  // coarse cells
    const sg_csr* A = nullptr;
    sg_precond* attached = nullptr;
    bool on = true;
    DBuf<float> master, grad, m1, m2, pmask;  // NET_PARAMS each
    DBuf<__nv_bfloat16> wf, wt;              // NLAYERS * LAYER_W
    DBuf<LearnedCtl> ctl;
    DBuf<float> feat;                        // coefficient feature of A
    DBuf<double> partials;
    DBuf<unsigned> counter;
    DBuf<int> cerr;  // set by a convolution whose bounded wait ran out
    int wait_test = 0;  // testing: 1 / 2 make the convolutions' copy / MMA waits give up
    DBuf<float> az32;   // A z of the stage's residual (FP32 values)
    DBuf<double> az64;  // the same for the FP64 training pairs
    // inference scratch (one sample)
    DBuf<float> rc, ec, yout;
    DBuf<uint32_t> act[4];
    // training pairs: coarse input, feature and target, fine energy target,
    // its energy, and the field (matrix) it came from
    DBuf<double> r64, e64, z64, t64;
    DBuf<float> s_in, s_tgt, s_feat, s_err, s_energy;
    DBuf<int> s_field;
    int nsamples = 0, cap = 0;
    std::vector<int> h_field;
    // fields of the stored pairs: one sparsity pattern, FP32 values per field
    DBuf<int> f_rp, f_ci;
    DBuf<float> f_vals;
    long long f_nnz = 0;
    int nfields = 0, fcap = 0;
    bool cur_registered = false;  // the current matrix is already a field
    // training scratch
    int tb = 0;
    DBuf<uint32_t> tact[4], tg[2];
    DBuf<float> ty, tt, tpart, tloss, tu, tw;
    DBuf<int> tidx;
    long long adam_t = 0;
    float out_scale = 1.f;
    int loss_kind = 0;  // 0 energy norm of A, 1 coarse mean squared error
};

}  // namespace sg

struct sg_learned : sg::LearnedImpl {};

namespace sg {

namespace {

int kblocks(sg_ctx* ctx, size_t n) {
    const size_t b = (n + 255) / 256;
    return (int)std::min<size_t>(std::max<size_t>(b, 1), (size_t)ctx->num_sms * 8);
}

void prep_weights(sg_learned* L) {
    k_prep_weights<<<(NLAYERS * LAYER_W + 255) / 256, 256, 0, L->ctx->stream>>>(L->master.p, L->wf.p,
                                                                             L->wt.p);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

// cuTensorMapEncodeTiled through the runtime's driver entry point (the
// library does not link the driver API)
PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q{};
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) != cudaSuccess ||
            q != cudaDriverEntryPointSuccess)
            p = nullptr;
        return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }();
    if (!fn) fail(SG_ERR_CUDA, "the driver provides no cuTensorMapEncodeTiled");
    return fn;
}

// the 5D tensor map of a BF16 [batch][D][D][D][16] activation volume whose
// box is one 8-channel half of a k_conv3d_tc halo
CUtensorMap halo_map(const uint32_t* in, int D, int batch) {
    CUtensorMap m;
    const cuuint64_t d = (cuuint64_t)D;
    const cuuint64_t dims[5] = {LC, d, d, d, (cuuint64_t)batch};
    const cuuint64_t strides[4] = {LC * 2, LC * 2 * d, LC * 2 * d * d, LC * 2 * d * d * d};
    const cuuint32_t box[5] = {8, TC_HX, TC_HY, TC_HZ, 1};
    const cuuint32_t estr[5] = {1, 1, 1, 1, 1};
    const CUresult r = tensor_map_encoder()(
        &m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 5, const_cast<uint32_t*>(in), dims, strides, box, estr,
        CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
        CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
    if (r != CUDA_SUCCESS) fail(SG_ERR_CUDA, "tensor map encoding failed (CUresult %d)", (int)r);
    return m;
}

// fin_*: the first layer of an inference apply reads its input from rc, f
// and s directly (one sample; `in` then only names a buffer for the map)
void conv(sg_learned* L, const uint32_t* in, int l, bool transposed, int epi, int batch,
          uint32_t* out, float* outf, const uint32_t* mask, const int* enabled, const int* active,
          const float* fin_rc = nullptr, const float* fin_feat = nullptr,
          const float* fin_s = nullptr) {
    const int D = L->cx;
    const int tiles = (D / TB) * ((D + TC_TY - 1) / TC_TY) * (D / TC_TZ);
    const __nv_bfloat16* w = (transposed ? L->wt.p : L->wf.p) + (size_t)l * LAYER_W;
    k_conv3d_tc<<<tiles * batch, TC_THREADS, TC_SMEM, L->ctx->stream>>>(
        halo_map(in, D, batch), reinterpret_cast<const uint8_t*>(w),
        L->master.p + (size_t)l * LAYER_P + LAYER_W, D, epi, out, outf, mask, enabled, active,
        L->cerr.p, L->wait_test, fin_rc, fin_feat, fin_s);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

void forward(sg_learned* L, const uint32_t* X0, uint32_t* A1, uint32_t* A2, uint32_t* A3,
             float* Y, int batch, const int* enabled, const int* active) {
    conv(L, X0, 0, false, EPI_RELU, batch, A1, nullptr, nullptr, enabled, active);
    conv(L, A1, 1, false, EPI_RELU, batch, A2, nullptr, nullptr, enabled, active);
    conv(L, A2, 2, false, EPI_RELU, batch, A3, nullptr, nullptr, enabled, active);
    conv(L, A3, 3, false, EPI_LINEAR_F32, batch, nullptr, Y, nullptr, enabled, active);
}

void wgrad(sg_learned* L, const uint32_t* X, const uint32_t* G, int l, int batch) {
    const int tiles = L->cx / TB;
    const int nblk = tiles * tiles * tiles * batch;
    k_conv3d_wgrad<<<nblk, CT, WGRAD_SMEM, L->ctx->stream>>>(X, G, L->cx, L->tpart.p);
    SG_CUDA(cudaGetLastError());
    k_wgrad_reduce<<<(LAYER_P + 255) / 256, 256, 0, L->ctx->stream>>>(
        L->tpart.p, nblk, L->pmask.p + (size_t)l * LAYER_P, L->grad.p + (size_t)l * LAYER_P);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
    count_launch(L->ctx);
}

void ensure_train(sg_learned* L, int batch) {
    if (L->tb >= batch) return;
    const size_t V = (size_t)L->nc;
    for (int i = 0; i < 4; ++i) L->tact[i].alloc(V * 8 * batch);
    for (int i = 0; i < 2; ++i) L->tg[i].alloc(V * 8 * batch);
    L->ty.alloc(V * batch);
    L->tt.alloc(V * batch);
    const int tiles = L->cx / TB;
    L->tpart.alloc((size_t)tiles * tiles * tiles * batch * LAYER_P);
    L->tloss.alloc(1);
    L->tidx.alloc(batch);
    if (L->loss_kind == 0) {
        const size_t n = (size_t)L->nx * L->ny * L->nz;
        L->tu.alloc(n * batch);
        L->tw.alloc(n * batch);
    }
    L->tb = batch;
}

// forward, loss and (with_grad) the parameter gradient of the packed batch in
// tact[0]; the loss is added to tloss.  energy: samples idx[0..batch) (device)
// of the stored pairs; otherwise targets tt (coarse mean squared error).
void loss_grad(sg_learned* L, int batch, bool with_grad, bool energy, const int* idx) {
    const size_t V = (size_t)L->nc;
    uint32_t *X0 = L->tact[0].p, *A1 = L->tact[1].p, *A2 = L->tact[2].p, *A3 = L->tact[3].p;
    forward(L, X0, A1, A2, A3, L->ty.p, batch, nullptr, nullptr);
    uint32_t* G = L->tg[0].p;
    uint32_t* H = L->tg[1].p;
    if (energy) {
        const int n = L->nx * L->ny * L->nz;
        if (L->tu.n < (size_t)n * batch) L->tu.alloc((size_t)n * batch);
        if (L->tw.n < (size_t)n * batch) L->tw.alloc((size_t)n * batch);
        cudaStream_t st = L->ctx->stream;
        k_energy_u<<<kblocks(L->ctx, (size_t)n * batch), 256, 0, st>>>(
            L->s_err.p, idx, batch, L->ty.p, L->nx, L->ny, L->nz, L->out_scale, L->tu.p);
        SG_CUDA(cudaGetLastError());
        const dim3 g((unsigned)std::min<long long>((n + 255) / 256, 1024), (unsigned)batch);
        k_energy_spmv<<<g, 256, 0, st>>>(L->f_rp.p, L->f_ci.p, L->f_vals.p, L->f_nnz, L->s_field.p,
                                         idx, L->s_energy.p, n, batch, L->tu.p, L->tw.p,
                                         L->tloss.p);
        SG_CUDA(cudaGetLastError());
        count_launch(L->ctx);
        count_launch(L->ctx);
        if (!with_grad) return;
        k_energy_grad<<<kblocks(L->ctx, V * batch), 256, 0, st>>>(
            L->tw.p, idx, L->s_energy.p, batch, L->nx, L->ny, L->nz, L->out_scale, G);
        SG_CUDA(cudaGetLastError());
        count_launch(L->ctx);
    } else {
        k_loss_grad<<<kblocks(L->ctx, V * batch), 256, 0, L->ctx->stream>>>(
            L->ty.p, L->tt.p, V * batch, with_grad ? G : nullptr, L->tloss.p);
        SG_CUDA(cudaGetLastError());
        count_launch(L->ctx);
        if (!with_grad) return;
    }
    // layer 4 (input A3), 3 (A2), 2 (A1), 1 (X0); the input gradient of a
    // layer is masked by the ReLU of its input (the previous layer's output)
    wgrad(L, A3, G, 3, batch);
    conv(L, G, 3, true, EPI_MASK, batch, H, nullptr, A3, nullptr, nullptr);
    wgrad(L, A2, H, 2, batch);
    conv(L, H, 2, true, EPI_MASK, batch, G, nullptr, A2, nullptr, nullptr);
    wgrad(L, A1, G, 1, batch);
    conv(L, G, 1, true, EPI_MASK, batch, H, nullptr, A1, nullptr, nullptr);
    wgrad(L, X0, H, 0, batch);
}

void adam_step(sg_learned* L, float lr) {
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    L->adam_t += 1;
    const float c1 = 1.f - (float)std::pow((double)b1, (double)L->adam_t);
    const float c2 = 1.f - (float)std::pow((double)b2, (double)L->adam_t);
    k_adam<<<(NET_PARAMS + 255) / 256, 256, 0, L->ctx->stream>>>(
        L->master.p, L->grad.p, L->m1.p, L->m2.p, L->pmask.p, NET_PARAMS, lr, b1, b2, eps, c1, c2);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
    prep_weights(L);
}

void grow_samples(sg_learned* L, int need) {
    if (need <= L->cap) return;
    const int ncap = std::max(need, std::max(16, 2 * L->cap));
    const size_t nc = (size_t)L->nc;
    auto grow = [&](DBuf<float>& b) {
        DBuf<float> nb;
        nb.alloc((size_t)ncap * nc);
        if (L->nsamples > 0)
            SG_CUDA(cudaMemcpyAsync(nb.p, b.p, sizeof(float) * nc * L->nsamples,
                                    cudaMemcpyDeviceToDevice, L->ctx->stream));
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
        std::swap(nb.p, b.p);
        std::swap(nb.n, b.n);
    };
    grow(L->s_in);
    grow(L->s_tgt);
    grow(L->s_feat);
    {
        const size_t n = (size_t)L->nx * L->ny * L->nz;
        DBuf<float> nb;
        nb.alloc((size_t)ncap * n);
        if (L->nsamples > 0)
            SG_CUDA(cudaMemcpyAsync(nb.p, L->s_err.p, sizeof(float) * n * L->nsamples,
                                    cudaMemcpyDeviceToDevice, L->ctx->stream));
        DBuf<float> ne;
        ne.alloc((size_t)ncap);
        DBuf<int> nf;
        nf.alloc((size_t)ncap);
        if (L->nsamples > 0) {
            SG_CUDA(cudaMemcpyAsync(ne.p, L->s_energy.p, sizeof(float) * L->nsamples,
                                    cudaMemcpyDeviceToDevice, L->ctx->stream));
            SG_CUDA(cudaMemcpyAsync(nf.p, L->s_field.p, sizeof(int) * L->nsamples,
                                    cudaMemcpyDeviceToDevice, L->ctx->stream));
        }
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
        std::swap(nb.p, L->s_err.p);
        std::swap(nb.n, L->s_err.n);
        std::swap(ne.p, L->s_energy.p);
        std::swap(ne.n, L->s_energy.n);
        std::swap(nf.p, L->s_field.p);
        std::swap(nf.n, L->s_field.n);
    }
    L->cap = ncap;
}

// the current matrix becomes a field of the stored pairs (FP32 values; the
// first field fixes the sparsity pattern every later one must share)
void register_field(sg_learned* L) {
    if (L->cur_registered) return;
    const sg_csr* A = L->A;
    sg_ctx* ctx = L->ctx;
    if (L->nfields == 0) {
        L->f_rp.upload(A->h_rp, ctx->stream);
        L->f_ci.upload(A->h_ci, ctx->stream);
        L->f_nnz = A->nnz;
    } else {
        std::vector<int> rp(A->nrows + 1), ci((size_t)A->nnz);
        if (A->nnz != L->f_nnz)
            fail(SG_ERR_INVALID_ARG, "pairs of one learned stage must share the sparsity pattern");
        SG_CUDA(cudaMemcpy(rp.data(), L->f_rp.p, sizeof(int) * rp.size(), cudaMemcpyDeviceToHost));
        SG_CUDA(cudaMemcpy(ci.data(), L->f_ci.p, sizeof(int) * ci.size(), cudaMemcpyDeviceToHost));
        if (rp != A->h_rp || ci != A->h_ci)
            fail(SG_ERR_INVALID_ARG, "pairs of one learned stage must share the sparsity pattern");
    }
    if (L->nfields + 1 > L->fcap) {
        const int ncap = std::max(4, 2 * L->fcap);
        DBuf<float> nb;
        nb.alloc((size_t)ncap * L->f_nnz);
        if (L->nfields > 0)
            SG_CUDA(cudaMemcpyAsync(nb.p, L->f_vals.p, sizeof(float) * L->f_nnz * L->nfields,
                                    cudaMemcpyDeviceToDevice, ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        std::swap(nb.p, L->f_vals.p);
        std::swap(nb.n, L->f_vals.n);
        L->fcap = ncap;
    }
    SG_CUDA(cudaMemcpyAsync(L->f_vals.p + (size_t)L->nfields * L->f_nnz, A->val32.p,
                            sizeof(float) * L->f_nnz, cudaMemcpyDeviceToDevice, ctx->stream));
    L->nfields += 1;
    L->cur_registered = true;
}

// restricted residual of v - A z (z may be null) into rc, s into *s_out: the
// matrix-level SpMV (the format tuned for A; TV = float: the FP32 values)
// into a fine scratch vector, then the restriction.  `active` gates the
// SpMV as it gates the solver's own; `enabled` gates the restriction and
// the rest of the stage.
template <class TA, class TI, class TO, class TV>
void resid_restrict(sg_learned* L, const TI* v, const TO* z, float* rc, float* s_out,
                    const int* enabled, const int* active) {
    const sg_csr* A = L->A;
    TV* az = nullptr;
    if (z) {
        const size_t n = (size_t)L->nx * L->ny * L->nz;
        if constexpr (std::is_same<TV, float>::value) {
            if (L->az32.n < n) L->az32.alloc(n);
            az = L->az32.p;
        } else {
            if (L->az64.n < n) L->az64.alloc(n);
            az = L->az64.p;
        }
        launch_spmv_a<TV, TO, TV>(L->ctx, A, z, az, nullptr, active);
    }
    const int grid = std::min(kblocks(L->ctx, (size_t)L->nc), 4096);  // 4096 partial sums
    k_resid_restrict<TA, TI, TV><<<grid, 256, 0, L->ctx->stream>>>(
        v, az, L->nx, L->ny, L->nz, rc, L->partials.p, L->counter.p, s_out, enabled, active);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

void check_ready(const sg_learned* L) {
    if (!L->A) fail(SG_ERR_NOT_SETUP, "learned stage has no matrix (sg_learned_set_matrix)");
}

void check_conv(sg_learned* L) {
    if (learned_error(L))
        fail(SG_ERR_DEVICE_TIMEOUT, "a learned-stage convolution gave up waiting for its tile");
}

}  // namespace

// ---------------------------------------------------------------- hooks
int learned_error(sg_learned* L) {
    if (!L || !L->cerr.p) return 0;
    int e = 0;
    SG_CUDA(cudaMemcpyAsync(&e, L->cerr.p, sizeof(int), cudaMemcpyDeviceToHost, L->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
    if (e) {  // reported once
        L->cerr.zero(L->ctx->stream);
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
    }
    return e;
}

template <class TI, class TO>
void learned_apply(sg_learned* L, const TI* x, TO* y, int n, const int* active) {
    check_ready(L);
    if ((long long)L->nx * L->ny * L->nz != (long long)n)
        fail(SG_ERR_INVALID_ARG, "learned stage grid %dx%dx%d does not match n = %d", L->nx, L->ny,
             L->nz, n);
    LearnedCtl* c = L->ctl.p;
    const int* en = &c->enabled;
    resid_restrict<float, TI, TO, float>(L, x, y, L->rc.p, &c->snorm, en, active);
    // the first layer packs its input from rc, f and s itself
    conv(L, L->act[0].p, 0, false, EPI_RELU, 1, L->act[1].p, nullptr, nullptr, en, active, L->rc.p,
         L->feat.p, &c->snorm);
    conv(L, L->act[1].p, 1, false, EPI_RELU, 1, L->act[2].p, nullptr, nullptr, en, active);
    conv(L, L->act[2].p, 2, false, EPI_RELU, 1, L->act[3].p, nullptr, nullptr, en, active);
    conv(L, L->act[3].p, 3, false, EPI_LINEAR_F32, 1, nullptr, L->yout.p, nullptr, en, active);
    // one fine cell per thread: each thread's eight loads of Y in flight at once
    k_prolong_add<TO><<<(n + 255) / 256, 256, 0, L->ctx->stream>>>(L->yout.p, L->nx, L->ny, L->nz,
                                                                   c, active, y);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

template void learned_apply<double, double>(sg_learned*, const double*, double*, int, const int*);
template void learned_apply<double, float>(sg_learned*, const double*, float*, int, const int*);
template void learned_apply<float, float>(sg_learned*, const float*, float*, int, const int*);

void learned_detach(sg_learned* L) {
    if (L) L->attached = nullptr;
}

uint64_t learned_gen(const sg_learned* L) { return L ? L->gen : 0; }

void learned_begin(sg_learned* L, SolveState* st) {
    check_ready(L);
    k_learned_begin<<<1, 1, 0, L->ctx->stream>>>(L->ctl.p, st, L->on ? 1 : 0);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

void learned_monitor(sg_learned* L, SolveState* st) {
    k_learned_monitor<<<1, 1, 0, L->ctx->stream>>>(L->ctl.p, st);
    SG_CUDA(cudaGetLastError());
    count_launch(L->ctx);
}

}  // namespace sg

using namespace sg;

namespace {
template <class F>
sg_status lguard(F&& f) {
    try {
        f();
        sg::set_last_error("");
        return SG_OK;
    } catch (const sg::Error& e) {
        sg::set_last_error(e.msg.c_str());
        return e.status;
    } catch (const std::exception& e) {
        sg::set_last_error(e.what());
        return SG_ERR_INTERNAL;
    }
}

void write_ctl(sg_learned* L, const LearnedCtl& h) {
    SG_CUDA(cudaMemcpyAsync(L->ctl.p, &h, sizeof(h), cudaMemcpyHostToDevice, L->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
}

LearnedCtl read_ctl(sg_learned* L) {
    LearnedCtl h{};
    SG_CUDA(cudaMemcpyAsync(&h, L->ctl.p, sizeof(h), cudaMemcpyDeviceToHost, L->ctx->stream));
    SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
    return h;
}

uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
double unit(uint64_t& s) { return (double)(splitmix(s) >> 11) * (1.0 / 9007199254740992.0); }

void split_pairs(const float* x, size_t V, std::vector<float>& in, std::vector<float>& ft) {
    in.resize(V);
    ft.resize(V);
    for (size_t q = 0; q < V; ++q) {
        in[q] = x[2 * q];
        ft[q] = x[2 * q + 1];
    }
}
}  // namespace

extern "C" {

int sg_learned_num_params(void) { return LEARN_PARAMS; }

sg_status sg_learned_create(sg_ctx* ctx, int nx, int ny, int nz, sg_learned** out) {
    return lguard([&] {
        SG_CHECK_ARG(ctx && out, "NULL argument");
        *out = nullptr;
        SG_CHECK_ARG(nx == ny && ny == nz, "the learned stage needs a cubic grid (got %dx%dx%d)",
                     nx, ny, nz);
        SG_CHECK_ARG(nx > 0 && nx % (2 * TB) == 0,
                     "grid edge must be a positive multiple of %d (got %d)", 2 * TB, nx);
        SG_CHECK_ARG((long long)nx * ny * nz < (1ll << 31), "grid too large");
        // the restriction keeps four fine grid lines per block in shared memory
        SG_CUDA(cudaSetDevice(ctx->device));
        auto* L = new sg_learned();
        L->gen = next_object_gen();
        try {
            L->ctx = ctx;
            L->nx = nx; L->ny = ny; L->nz = nz;
            L->cx = nx / 2; L->cy = ny / 2; L->cz = nz / 2;
            L->nc = L->cx * L->cy * L->cz;
            L->master.alloc(NET_PARAMS);
            L->grad.alloc(NET_PARAMS);
            L->m1.alloc(NET_PARAMS);
            L->m2.alloc(NET_PARAMS);
            L->pmask.alloc(NET_PARAMS);
            L->wf.alloc((size_t)NLAYERS * LAYER_W);
            L->wt.alloc((size_t)NLAYERS * LAYER_W);
            // real parameters: layer 1 reads channels 0-1, layer 4 writes channel 0
            std::vector<float> mask(NET_PARAMS, 1.f);
            for (int l = 0; l < NLAYERS; ++l)
                for (int i = 0; i < LAYER_P; ++i) {
                    float& m = mask[(size_t)l * LAYER_P + i];
                    if (i < LAYER_W) {
                        const int ci = (i / LC) % LC, co = i % LC;
                        if (l == 0 && ci >= 2) m = 0.f;
                        if (l == NLAYERS - 1 && co >= 1) m = 0.f;
                    } else if (l == NLAYERS - 1 && i - LAYER_W >= 1) {
                        m = 0.f;
                    }
                }
            L->pmask.upload(mask, ctx->stream);
            L->master.zero(ctx->stream);
            L->grad.zero(ctx->stream);
            L->m1.zero(ctx->stream);
            L->m2.zero(ctx->stream);
            L->ctl.alloc(1);
            LearnedCtl h{};
            h.out_scale = 1.f;
            h.enabled = 1;
            h.fallback_cycle = -1;
            L->ctl.upload(&h, 1, ctx->stream);
            L->partials.alloc(4096);
            L->counter.alloc(1);
            L->counter.zero(ctx->stream);
            L->cerr.alloc(1);
            L->cerr.zero(ctx->stream);
            SG_CUDA(cudaFuncSetAttribute(k_conv3d_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         TC_SMEM));
            L->rc.alloc(L->nc);
            L->ec.alloc(L->nc);
            L->yout.alloc(L->nc);
            for (int i = 0; i < 4; ++i) L->act[i].alloc((size_t)L->nc * 8);
            L->feat.alloc(L->nc);
            L->feat.zero(ctx->stream);
            SG_CUDA(cudaFuncSetAttribute(k_conv3d_wgrad, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         WGRAD_SMEM));
            prep_weights(L);
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
        } catch (...) {
            delete L;
            throw;
        }
        *out = L;
    });
}

sg_status sg_learned_destroy(sg_learned* L) {
    return lguard([&] {
        if (!L) return;
        cudaSetDevice(L->ctx->device);
        if (L->attached) {
            L->attached->learned = nullptr;
            L->attached->gen = next_object_gen();
        }
        delete L;
    });
}

sg_status sg_learned_set_matrix(sg_learned* L, const sg_csr* A) {
    return lguard([&] {
        SG_CHECK_ARG(L && A, "NULL argument");
        L->gen = next_object_gen();
        SG_CHECK_ARG(A->ctx == L->ctx, "matrix belongs to a different context");
        SG_CHECK_ARG(A->nrows == A->ncols &&
                         (long long)L->nx * L->ny * L->nz == (long long)A->nrows,
                     "matrix of %d rows does not match the %dx%dx%d grid", A->nrows, L->nx, L->ny,
                     L->nz);
        // coefficient feature: log A_ii restricted to the coarse cells, standardised
        std::vector<double> ld(A->nrows, 0.0);
        for (int i = 0; i < A->nrows; ++i) {
            double d = 0.0;
            for (int q = A->h_rp[i]; q < A->h_rp[i + 1]; ++q)
                if (A->h_ci[q] == i) d += A->h_val[q];
            if (!(d > 0.0)) fail(SG_ERR_INVALID_ARG, "row %d has a non-positive diagonal", i);
            ld[i] = std::log(d);
        }
        std::vector<float> c((size_t)L->nc);
        std::vector<double> cd((size_t)L->nc);
        double mean = 0.0;
        for (int k = 0; k < L->cz; ++k)
            for (int j = 0; j < L->cy; ++j)
                for (int i = 0; i < L->cx; ++i) {
                    double s = 0.0;
                    for (int o = 0; o < 8; ++o) {
                        const int fx = 2 * i + (o & 1), fy = 2 * j + ((o >> 1) & 1),
                                  fz = 2 * k + (o >> 2);
                        s += ld[((size_t)fz * L->ny + fy) * L->nx + fx];
                    }
                    cd[((size_t)k * L->cy + j) * L->cx + i] = s / 8.0;
                    mean += s / 8.0;
                }
        mean /= (double)cd.size();
        double var = 0.0;
        for (double v : cd) var += (v - mean) * (v - mean);
        var /= (double)cd.size();
        const double inv = var > 1e-24 ? 1.0 / std::sqrt(var) : 0.0;
        for (size_t q = 0; q < cd.size(); ++q) c[q] = (float)((cd[q] - mean) * inv);
        const_cast<sg_csr*>(A)->ensure_fp32();
        L->feat.upload(c, L->ctx->stream);
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
        L->A = A;
        L->cur_registered = false;
    });
}

sg_status sg_learned_init_weights(sg_learned* L, uint64_t seed) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        // He-uniform over the real fan-in; the last layer starts 10x smaller so
        // the untrained stage adds little
        std::vector<float> w(NET_PARAMS, 0.f);
        uint64_t s = seed;
        for (int l = 0; l < NLAYERS; ++l) {
            const int fan_in = LTAPS * (l == 0 ? 2 : LC);
            double bound = std::sqrt(6.0 / fan_in);
            if (l == NLAYERS - 1) bound *= 0.1;
            for (int i = 0; i < LAYER_W; ++i) {
                const int ci = (i / LC) % LC, co = i % LC;
                const double u = unit(s);
                if ((l == 0 && ci >= 2) || (l == NLAYERS - 1 && co >= 1)) continue;
                w[(size_t)l * LAYER_P + i] = (float)((2.0 * u - 1.0) * bound);
            }
        }
        L->master.upload(w, L->ctx->stream);
        L->m1.zero(L->ctx->stream);
        L->m2.zero(L->ctx->stream);
        L->adam_t = 0;
        prep_weights(L);
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
    });
}

sg_status sg_learned_set_weights(sg_learned* L, const float* w, int count) {
    return lguard([&] {
        SG_CHECK_ARG(L && w, "NULL argument");
        SG_CHECK_ARG(count == LEARN_PARAMS, "expected %d parameters (got %d)", LEARN_PARAMS, count);
        SG_CHECK_ARG(std::isfinite(w[NET_PARAMS]) && w[NET_PARAMS] > 0.f,
                     "output scale must be positive");
        std::vector<float> mask(NET_PARAMS);
        SG_CUDA(cudaMemcpy(mask.data(), L->pmask.p, sizeof(float) * NET_PARAMS,
                           cudaMemcpyDeviceToHost));
        std::vector<float> h(w, w + NET_PARAMS);
        for (int i = 0; i < NET_PARAMS; ++i) {
            SG_CHECK_ARG(std::isfinite(h[i]), "parameter %d is not finite", i);
            h[i] *= mask[i];
        }
        L->master.upload(h, L->ctx->stream);
        L->out_scale = w[NET_PARAMS];
        LearnedCtl c = read_ctl(L);
        c.out_scale = L->out_scale;
        write_ctl(L, c);
        L->m1.zero(L->ctx->stream);
        L->m2.zero(L->ctx->stream);
        L->adam_t = 0;
        prep_weights(L);
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
    });
}

sg_status sg_learned_get_weights(sg_learned* L, float* w, int count) {
    return lguard([&] {
        SG_CHECK_ARG(L && w, "NULL argument");
        SG_CHECK_ARG(count == LEARN_PARAMS, "expected %d parameters (got %d)", LEARN_PARAMS, count);
        SG_CUDA(cudaMemcpyAsync(w, L->master.p, sizeof(float) * NET_PARAMS, cudaMemcpyDeviceToHost,
                                L->ctx->stream));
        SG_CUDA(cudaStreamSynchronize(L->ctx->stream));
        w[NET_PARAMS] = L->out_scale;
    });
}

sg_status sg_learned_add_pair(sg_learned* L, sg_precond* pc, const double* r, const double* e,
                              int n, sg_mem mem) {
    return lguard([&] {
        SG_CHECK_ARG(L && pc && r && e, "NULL argument");
        check_ready(L);
        SG_CHECK_ARG(pc->ctx == L->ctx, "preconditioner belongs to a different context");
        if (!pc->is_setup) fail(SG_ERR_NOT_SETUP, "preconditioner used before setup");
        SG_CHECK_ARG(n == L->A->nrows && pc->n == n, "n (%d) does not match the grid", n);
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        const double* dr = r;
        const double* de = e;
        if (mem == SG_MEM_HOST) {
            L->r64.upload(r, n, ctx->stream);
            L->e64.upload(e, n, ctx->stream);
            dr = L->r64.p;
            de = L->e64.p;
        }
        if (L->z64.n < (size_t)n) L->z64.alloc(n);
        if (L->t64.n < (size_t)n) L->t64.alloc(n);
        // z1 = M r (the plain preconditioner); r1 = r - A z1; e1 = e - z1
        precond_apply_device<double, double>(pc, dr, L->z64.p, nullptr, false);
        LearnedCtl* c = L->ctl.p;
        resid_restrict<double, double, double, double>(L, dr, L->z64.p, L->rc.p,
                                                       &c->pair_s, nullptr, nullptr);
        k_sub64<<<kblocks(ctx, n), 256, 0, ctx->stream>>>(de, L->z64.p, n, L->t64.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        resid_restrict<double, double, double, double>(L, L->t64.p,
                                                       static_cast<const double*>(nullptr), L->ec.p,
                                                       &c->scratch_s, nullptr, nullptr);
        grow_samples(L, L->nsamples + 1);
        register_field(L);
        const int field = L->nfields - 1;
        const size_t off = (size_t)L->nsamples * L->nc;
        k_store_pair<<<kblocks(ctx, (size_t)L->nc), 256, 0, ctx->stream>>>(
            L->rc.p, L->ec.p, L->feat.p, L->nc, c, L->s_in.p + off, L->s_tgt.p + off,
            L->s_feat.p + off);
        SG_CUDA(cudaGetLastError());
        // fine energy target (e - M r) / s and its energy in the field's A
        float* err = L->s_err.p + (size_t)L->nsamples * n;
        k_scale_store<<<kblocks(ctx, n), 256, 0, ctx->stream>>>(L->t64.p, n, c, err);
        SG_CUDA(cudaGetLastError());
        k_energy_norm<<<std::min(kblocks(ctx, n), 4096), 256, 0, ctx->stream>>>(
            L->f_rp.p, L->f_ci.p, L->f_vals.p + (size_t)field * L->f_nnz, err, n, L->partials.p,
            L->counter.p, L->s_energy.p + L->nsamples);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        count_launch(ctx);
        count_launch(ctx);
        SG_CUDA(cudaMemcpyAsync(L->s_field.p + L->nsamples, &field, sizeof(int),
                                cudaMemcpyHostToDevice, ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        if (sweep_error(pc))
            fail(SG_ERR_DEVICE_TIMEOUT, "a subdomain sweep gave up waiting for its factor records");
        L->nsamples += 1;
    });
}

sg_status sg_learned_num_samples(sg_learned* L, int* count) {
    return lguard([&] {
        SG_CHECK_ARG(L && count, "NULL argument");
        *count = L->nsamples;
    });
}

sg_status sg_learned_clear_samples(sg_learned* L) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        L->nsamples = 0;
        L->nfields = 0;
        L->cur_registered = false;
    });
}

sg_status sg_learned_get_sample_fine(sg_learned* L, int i, float* err, float* energy, int* field) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        SG_CHECK_ARG(i >= 0 && i < L->nsamples, "sample %d out of range [0,%d)", i, L->nsamples);
        const size_t n = (size_t)L->nx * L->ny * L->nz;
        if (err)
            SG_CUDA(cudaMemcpy(err, L->s_err.p + (size_t)i * n, sizeof(float) * n,
                               cudaMemcpyDeviceToHost));
        if (energy)
            SG_CUDA(cudaMemcpy(energy, L->s_energy.p + i, sizeof(float), cudaMemcpyDeviceToHost));
        if (field) SG_CUDA(cudaMemcpy(field, L->s_field.p + i, sizeof(int), cudaMemcpyDeviceToHost));
    });
}

sg_status sg_learned_set_loss(sg_learned* L, int kind) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        SG_CHECK_ARG(kind == 0 || kind == 1, "loss kind must be 0 (energy) or 1 (coarse MSE)");
        L->loss_kind = kind;
    });
}

sg_status sg_learned_sample_gradient(sg_learned* L, int first, int count, float* grad,
                                     double* loss) {
    return lguard([&] {
        SG_CHECK_ARG(L && grad && loss, "NULL argument");
        SG_CHECK_ARG(first >= 0 && count >= 1 && count <= 64 && first + count <= L->nsamples,
                     "samples [%d,%d) out of range [0,%d) or more than 64", first, first + count,
                     L->nsamples);
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        ensure_train(L, count);
        std::vector<int> idx(count);
        for (int i = 0; i < count; ++i) idx[i] = first + i;
        L->tidx.upload(idx, ctx->stream);
        k_pack_batch<<<kblocks(ctx, (size_t)count * L->nc), 256, 0, ctx->stream>>>(
            L->s_in.p, L->s_feat.p, L->s_tgt.p, L->tidx.p, count, L->nc, 1.f / L->out_scale,
            L->tact[0].p, L->tt.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        L->tloss.zero(ctx->stream);
        loss_grad(L, count, true, L->loss_kind == 0, L->tidx.p);
        float l = 0.f;
        SG_CUDA(cudaMemcpyAsync(&l, L->tloss.p, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(cudaMemcpyAsync(grad, L->grad.p, sizeof(float) * NET_PARAMS, cudaMemcpyDeviceToHost,
                                ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        check_conv(L);
        *loss = l;
    });
}

sg_status sg_learned_get_sample(sg_learned* L, int i, float* input, float* feature,
                                float* target) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        SG_CHECK_ARG(i >= 0 && i < L->nsamples, "sample %d out of range [0,%d)", i, L->nsamples);
        const size_t off = (size_t)i * L->nc, bytes = sizeof(float) * L->nc;
        if (input) SG_CUDA(cudaMemcpy(input, L->s_in.p + off, bytes, cudaMemcpyDeviceToHost));
        if (feature) SG_CUDA(cudaMemcpy(feature, L->s_feat.p + off, bytes, cudaMemcpyDeviceToHost));
        if (target) SG_CUDA(cudaMemcpy(target, L->s_tgt.p + off, bytes, cudaMemcpyDeviceToHost));
    });
}

sg_status sg_learned_train(sg_learned* L, int first, int count, int epochs, int batch, double lr,
                           uint64_t seed, double* epoch_loss) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        SG_CHECK_ARG(first >= 0 && count >= 1 && first + count <= L->nsamples,
                     "samples [%d,%d) out of range [0,%d)", first, first + count, L->nsamples);
        SG_CHECK_ARG(epochs >= 0 && batch >= 1 && batch <= 64, "bad epochs/batch");
        SG_CHECK_ARG(lr > 0 && std::isfinite(lr), "learning rate must be positive");
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        ensure_train(L, batch);
        // output scale: rms of the training targets
        {
            std::vector<float> t((size_t)count * L->nc);
            SG_CUDA(cudaMemcpy(t.data(), L->s_tgt.p + (size_t)first * L->nc,
                               sizeof(float) * t.size(), cudaMemcpyDeviceToHost));
            double ss = 0.0;
            for (float v : t) ss += (double)v * v;
            const double rms = std::sqrt(ss / (double)t.size());
            L->out_scale = rms > 0 && std::isfinite(rms) ? (float)rms : 1.f;
            LearnedCtl c = read_ctl(L);
            c.out_scale = L->out_scale;
            write_ctl(L, c);
        }
        const float inv_c = 1.f / L->out_scale;
        uint64_t s = seed;
        std::vector<int> perm(count);
        DBuf<int> dperm;
        dperm.alloc(count);
        for (int ep = 0; ep < epochs; ++ep) {
            for (int i = 0; i < count; ++i) perm[i] = first + i;
            for (int i = count - 1; i > 0; --i) {
                const int j = (int)(splitmix(s) % (uint64_t)(i + 1));
                std::swap(perm[i], perm[j]);
            }
            dperm.upload(perm, ctx->stream);
            L->tloss.zero(ctx->stream);
            int nb = 0;
            for (int b0 = 0; b0 < count; b0 += batch, ++nb) {
                const int bs = std::min(batch, count - b0);
                k_pack_batch<<<kblocks(ctx, (size_t)bs * L->nc), 256, 0, ctx->stream>>>(
                    L->s_in.p, L->s_feat.p, L->s_tgt.p, dperm.p + b0, bs, L->nc, inv_c,
                    L->tact[0].p, L->tt.p);
                SG_CUDA(cudaGetLastError());
                count_launch(ctx);
                loss_grad(L, bs, true, L->loss_kind == 0, dperm.p + b0);
                adam_step(L, (float)lr);
            }
            float lsum = 0.f;
            SG_CUDA(cudaMemcpyAsync(&lsum, L->tloss.p, sizeof(float), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
            if (epoch_loss) epoch_loss[ep] = (double)lsum / nb;
            check_conv(L);
            if (!std::isfinite(lsum)) fail(SG_ERR_NONFINITE, "training loss is not finite");
        }
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

sg_status sg_learned_eval(sg_learned* L, int first, int count, double* loss) {
    return lguard([&] {
        SG_CHECK_ARG(L && loss, "NULL argument");
        SG_CHECK_ARG(first >= 0 && count >= 1 && first + count <= L->nsamples,
                     "samples [%d,%d) out of range [0,%d)", first, first + count, L->nsamples);
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        const int batch = L->tb > 0 ? std::min(L->tb, 8) : 8;
        ensure_train(L, batch);
        const float inv_c = 1.f / L->out_scale;
        std::vector<int> idx(count);
        for (int i = 0; i < count; ++i) idx[i] = first + i;
        DBuf<int> didx;
        didx.upload(idx, ctx->stream);
        double total = 0.0;
        for (int b0 = 0; b0 < count; b0 += batch) {
            const int bs = std::min(batch, count - b0);
            L->tloss.zero(ctx->stream);
            k_pack_batch<<<kblocks(ctx, (size_t)bs * L->nc), 256, 0, ctx->stream>>>(
                L->s_in.p, L->s_feat.p, L->s_tgt.p, didx.p + b0, bs, L->nc, inv_c, L->tact[0].p,
                L->tt.p);
            SG_CUDA(cudaGetLastError());
            count_launch(ctx);
            loss_grad(L, bs, false, L->loss_kind == 0, didx.p + b0);
            float l = 0.f;
            SG_CUDA(cudaMemcpyAsync(&l, L->tloss.p, sizeof(float), cudaMemcpyDeviceToHost,
                                    ctx->stream));
            SG_CUDA(cudaStreamSynchronize(ctx->stream));
            total += (double)l * bs;
        }
        check_conv(L);
        *loss = total / count;
    });
}

sg_status sg_learned_forward(sg_learned* L, const float* x, int batch, float* y) {
    return lguard([&] {
        SG_CHECK_ARG(L && x && y, "NULL argument");
        SG_CHECK_ARG(batch >= 1 && batch <= 64, "batch must be in [1,64]");
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        ensure_train(L, batch);
        const size_t V = (size_t)L->nc * batch;
        std::vector<float> in, ft;
        split_pairs(x, V, in, ft);
        DBuf<float> din, dft;
        din.upload(in, ctx->stream);
        dft.upload(ft, ctx->stream);
        k_pack_batch<<<kblocks(ctx, V), 256, 0, ctx->stream>>>(din.p, dft.p, nullptr, nullptr, batch,
                                                              L->nc, 1.f, L->tact[0].p, nullptr);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        forward(L, L->tact[0].p, L->tact[1].p, L->tact[2].p, L->tact[3].p, L->ty.p, batch, nullptr,
                nullptr);
        SG_CUDA(cudaMemcpyAsync(y, L->ty.p, sizeof(float) * V, cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        check_conv(L);
    });
}

sg_status sg_learned_gradient(sg_learned* L, const float* x, const float* t, int batch,
                              float* grad, double* loss) {
    return lguard([&] {
        SG_CHECK_ARG(L && x && t && grad && loss, "NULL argument");
        SG_CHECK_ARG(batch >= 1 && batch <= 64, "batch must be in [1,64]");
        sg_ctx* ctx = L->ctx;
        SG_CUDA(cudaSetDevice(ctx->device));
        ensure_train(L, batch);
        const size_t V = (size_t)L->nc * batch;
        std::vector<float> in, ft;
        split_pairs(x, V, in, ft);
        DBuf<float> din, dft, dt;
        din.upload(in, ctx->stream);
        dft.upload(ft, ctx->stream);
        dt.upload(t, V, ctx->stream);
        k_pack_batch<<<kblocks(ctx, V), 256, 0, ctx->stream>>>(din.p, dft.p, dt.p, nullptr, batch,
                                                              L->nc, 1.f, L->tact[0].p, L->tt.p);
        SG_CUDA(cudaGetLastError());
        count_launch(ctx);
        L->tloss.zero(ctx->stream);
        loss_grad(L, batch, true, false, nullptr);
        float l = 0.f;
        SG_CUDA(cudaMemcpyAsync(&l, L->tloss.p, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream));
        SG_CUDA(cudaMemcpyAsync(grad, L->grad.p, sizeof(float) * NET_PARAMS, cudaMemcpyDeviceToHost,
                                ctx->stream));
        SG_CUDA(cudaStreamSynchronize(ctx->stream));
        check_conv(L);
        *loss = l;
    });
}

sg_status sg_learned_set_enabled(sg_learned* L, int on) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        L->on = on != 0;
        LearnedCtl c = read_ctl(L);
        c.enabled = L->on ? 1 : 0;
        write_ctl(L, c);
    });
}

sg_status sg_learned_set_wait_test(sg_learned* L, int mode) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        SG_CHECK_ARG(mode >= 0 && mode <= 2, "wait test mode must be 0, 1 or 2 (got %d)", mode);
        L->wait_test = mode;
    });
}

sg_status sg_learned_get_state(sg_learned* L, int* enabled, int* fallback_cycle,
                               long long* applies) {
    return lguard([&] {
        SG_CHECK_ARG(L, "NULL argument");
        const LearnedCtl c = read_ctl(L);
        if (enabled) *enabled = c.enabled;
        if (fallback_cycle) *fallback_cycle = c.fallback_cycle;
        if (applies) *applies = (long long)c.applies;
    });
}

sg_status sg_precond_set_learned(sg_precond* pc, sg_learned* L, double stagnation) {
    return lguard([&] {
        SG_CHECK_ARG(pc, "NULL argument");
        pc->gen = next_object_gen();
        if (!L) {
            if (pc->learned) pc->learned->attached = nullptr;
            pc->learned = nullptr;
            return;
        }
        SG_CHECK_ARG(L->ctx == pc->ctx, "learned stage belongs to a different context");
        SG_CHECK_ARG(pc->kind >= SG_PC_ASM && pc->kind <= SG_PC_TWOLEVEL_RAS,
                     "the learned stage attaches to Schwarz preconditioners");
        SG_CHECK_ARG(stagnation >= 0.0 && std::isfinite(stagnation),
                     "stagnation ratio must be >= 0");
        check_ready(L);
        if (pc->is_setup)
            SG_CHECK_ARG(pc->n == L->A->nrows, "preconditioner size %d != grid size %d", pc->n,
                         L->A->nrows);
        if (L->attached && L->attached != pc) {
            L->attached->learned = nullptr;
            L->attached->gen = next_object_gen();
        }
        if (pc->learned && pc->learned != L) pc->learned->attached = nullptr;
        L->attached = pc;
        pc->learned = L;
        LearnedCtl c = read_ctl(L);
        c.stag = stagnation;
        write_ctl(L, c);
    });
}

}  // extern "C"
