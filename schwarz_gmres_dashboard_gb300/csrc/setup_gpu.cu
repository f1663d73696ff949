// setup_gpu.cu -- the integer set-up of the Schwarz preconditioners on the
// device: the same decomposition (src/decomp/domain_decomp.h:61-93), owned-
// local map (src/precond/ras.h:34-41), local CSR structure of A[dofs,dofs]
// (src/core/sparse_matrix.h:53-83), ILU(0) diagonal positions
// (src/precond/ilu0.h:19-29), level schedules and slot layouts as the host
// set-up of setup.cpp, bit for bit, from the matrix already in HBM.
//
//  1. owned lists: rows sorted by part, stable (an LSD radix sort, 8 bits per
//     pass; inside a block one warp places 32 rows at a time, ranks from
//     __match_any_sync, so equal parts keep row order);
//  2. overlap: each subdomain marks its rows in a bitmap over the row range
//     its overlap can reach (owned rows +- overlap x the matrix half
//     bandwidths); layer k marks the neighbours of the rows layer k-1 added;
//     a subdomain's sorted row list is its bitmap read in order, and a row's
//     local index is the popcount below it (word prefix + in-word count);
//  3. local CSR: per local row the entries whose column is in the bitmap,
//     local column = its rank, in the original (sorted) order, plus the
//     global entry index, the diagonal position and the row's widths;
//  4. level schedules: one block per subdomain relaxes the level recurrence
//     to its (unique) fixed point in shared memory, then one warp places the
//     rows by level, stably;
//  5. slot layout: per candidate shift the warp-exact bank-conflict cost of
//     the sweep's shared-memory loads (distinct slots per bank, as the host
//     counts them).
// The host finishes with schwarz_finish (O(parts + levels) work).  When the
// bitmaps would take too much memory (a matrix whose bandwidth makes every
// subdomain's range close to n, with many subdomains) the caller falls back
// to the host set-up.
#include <algorithm>
#include <climits>
#include <cmath>
#include <vector>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

void schwarz_finish(sg_precond* pc, const std::vector<int>& perm_f_all,
                    const std::vector<int>& perm_b_all);

namespace {

constexpr int ST = 256;

__device__ __forceinline__ int upper_bound_dev(const int* a, int n, int v) {
    // first index i in [0, n) with a[i] > v (a ascending)
    int lo = 0, hi = n;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (a[mid] <= v) lo = mid + 1;
        else hi = mid;
    }
    return lo;
}
// segment of x in the ascending offsets ptr[0..P] (ptr[s] <= x < ptr[s+1])
__device__ __forceinline__ int segment_of(const int* ptr, int P, int x) {
    return upper_bound_dev(ptr, P + 1, x) - 1;
}

// ------------------------------------------------------------ device scan
// exclusive prefix sums of int counts (long long results), in three steps:
// per-block sums, a one-block scan of those, per-block add
constexpr int SC_T = 1024, SC_I = 4, SC_B = SC_T * SC_I;

__global__ void __launch_bounds__(SC_T) k_scan_blocks(const int* in, long long n, long long* out,
                                                     long long* bsum) {
    __shared__ long long ws[SC_T / 32];
    const long long base = (long long)blockIdx.x * SC_B + (long long)threadIdx.x * SC_I;
    long long v[SC_I], run = 0;
#pragma unroll
    for (int k = 0; k < SC_I; ++k) {
        v[k] = base + k < n ? in[base + k] : 0;
        run += v[k];
    }
    // inclusive scan of the per-thread totals across the block
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < SC_T / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SC_T / 32) ws[lane] = w;
    }
    __syncthreads();
    long long excl = x - run + (warp > 0 ? ws[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < SC_I; ++k) {
        if (base + k < n) out[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SC_T - 1) bsum[blockIdx.x] = excl;
}

// one block: exclusive scan of the nb block sums in place (nb <= SC_B)
__global__ void __launch_bounds__(SC_T) k_scan_sums(long long* bsum, int nb, long long* total) {
    __shared__ long long ws[SC_T / 32];
    const int base = threadIdx.x * SC_I;
    long long v[SC_I], run = 0;
#pragma unroll
    for (int k = 0; k < SC_I; ++k) {
        v[k] = base + k < nb ? bsum[base + k] : 0;
        run += v[k];
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    long long x = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const long long y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    if (warp == 0) {
        long long w = lane < SC_T / 32 ? ws[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const long long y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < SC_T / 32) ws[lane] = w;
    }
    __syncthreads();
    long long excl = x - run + (warp > 0 ? ws[warp - 1] : 0);
#pragma unroll
    for (int k = 0; k < SC_I; ++k) {
        if (base + k < nb) bsum[base + k] = excl;
        excl += v[k];
    }
    if (threadIdx.x == SC_T - 1) *total = excl;
}

__global__ void k_scan_add(long long* out, long long n, const long long* bsum) {
    const long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) out[i] += bsum[i / SC_B];
}

// ------------------------------------------------------------ owned lists
constexpr int RS_CH = 4096;  // rows per radix-sort block

__global__ void k_count_parts(const int* part, int n, int* cnt) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        atomicAdd(&cnt[part[i]], 1);
}

__global__ void __launch_bounds__(256) k_rs_hist(const int* key, int n, int shift, int nb,
                                                 int* hist) {
    __shared__ int h[256];
    h[threadIdx.x] = 0;
    __syncthreads();
    const int end = min(n, (blockIdx.x + 1) * RS_CH);
    for (int i = blockIdx.x * RS_CH + threadIdx.x; i < end; i += 256)
        atomicAdd(&h[(key[i] >> shift) & 255], 1);
    __syncthreads();
    hist[threadIdx.x * nb + blockIdx.x] = h[threadIdx.x];  // digit-major
}

// one warp per block, rows in order, 32 at a time: equal digits keep order
__global__ void __launch_bounds__(32) k_rs_scatter(const int* key, const int* val, int n,
                                                   int shift, int nb, const long long* off,
                                                   int* key_out, int* val_out) {
    __shared__ long long cnt[256];
    const int lane = threadIdx.x;
    for (int d = lane; d < 256; d += 32) cnt[d] = off[(size_t)d * nb + blockIdx.x];
    __syncwarp();
    const int end = min(n, (blockIdx.x + 1) * RS_CH);
    const unsigned lt = (1u << lane) - 1u;
    for (int i0 = blockIdx.x * RS_CH; i0 < end; i0 += 32) {
        const int i = i0 + lane;
        const bool valid = i < end;
        const int k = valid ? key[i] : 0;
        const int d = valid ? (k >> shift) & 255 : 256 + lane;
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt);
        const long long base = valid ? cnt[d] : 0;
        __syncwarp();
        if (valid) {
            key_out[base + rank] = k;
            val_out[base + rank] = val[i];
            if (lane == __ffs(peers) - 1) cnt[d] = base + __popc(peers);
        }
        __syncwarp();
    }
}

__global__ void k_iota(int* v, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) v[i] = i;
}

// half bandwidths of A: max(i - first column), max(last column - i)
__global__ void k_bandwidth(const int* rp, const int* ci, int n, int* bw) {
    int lo = 0, hi = 0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        if (rp[i + 1] > rp[i]) {
            lo = max(lo, i - ci[rp[i]]);
            hi = max(hi, ci[rp[i + 1] - 1] - i);
        }
    }
    atomicMax(&bw[0], lo);
    atomicMax(&bw[1], hi);
}

// first and last owned row of every subdomain (the owned lists ascend)
__global__ void k_owned_ends(const int* owned, const int* optr, int P, int* ends) {
    const int s = blockIdx.x * blockDim.x + threadIdx.x;
    if (s >= P) return;
    ends[2 * s] = owned[optr[s]];
    ends[2 * s + 1] = owned[optr[s + 1] - 1];
}

// ------------------------------------------------------------ overlap bitmaps
struct Bits {
    const int* lo;       // [P] first row of the range
    const int* woff;     // [P+1] first word
    unsigned* w;         // the bitmaps
    int P;
};

__device__ __forceinline__ bool bits_set(const Bits& b, int s, int r, int* bad) {
    const int x = r - b.lo[s];
    const int wi = b.woff[s] + (x >> 5);
    if (x < 0 || wi >= b.woff[s + 1]) {
        atomicExch(bad, 1);  // outside the range the bandwidth bound promised
        return false;
    }
    atomicOr(&b.w[wi], 1u << (x & 31));
    return true;
}

// layer 0: every owned row
__global__ void k_mark_owned(const int* owned, const int* part, int n, Bits b, int* bad) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = owned[q];
        bits_set(b, part[r], r, bad);
    }
}

// layer 1: the neighbours of every owned row
__global__ void k_expand_owned(const int* owned, const int* part, int n, const int* rp,
                               const int* ci, Bits b, int* bad) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = owned[q], s = part[r];
        for (int e = rp[r]; e < rp[r + 1]; ++e) bits_set(b, s, ci[e], bad);
    }
}

// layers >= 2: the neighbours of the rows the previous layer added
// (frontier bits f = current & ~before, computed before this kernel)
__global__ void k_expand_bits(const unsigned* f, int nw, const int* rp, const int* ci, Bits b,
                              int* bad) {
    for (int wi = blockIdx.x * blockDim.x + threadIdx.x; wi < nw; wi += gridDim.x * blockDim.x) {
        unsigned m = f[wi];
        if (!m) continue;
        const int s = segment_of(b.woff, b.P, wi);
        const int r0 = b.lo[s] + 32 * (wi - b.woff[s]);
        while (m) {
            const int bit = __ffs(m) - 1;
            m &= m - 1;
            const int r = r0 + bit;
            for (int e = rp[r]; e < rp[r + 1]; ++e) bits_set(b, s, ci[e], bad);
        }
    }
}

__global__ void k_andnot(const unsigned* a, const unsigned* b, unsigned* f, int nw) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nw; i += gridDim.x * blockDim.x)
        f[i] = a[i] & ~b[i];
}

// per subdomain (one block each): exclusive prefix of the words' popcounts
// (wpre) and the subdomain's row count
__global__ void __launch_bounds__(ST) k_word_prefix(const unsigned* w, const int* woff,
                                                    int* wpre, int* count) {
    __shared__ int ws[ST / 32];
    __shared__ int carry;
    const int s = blockIdx.x, w0 = woff[s], w1 = woff[s + 1];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    for (int b0 = w0; b0 < w1; b0 += ST) {
        const int i = b0 + threadIdx.x;
        const int v = i < w1 ? __popc(w[i]) : 0;
        int x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        int pre = 0;
        for (int k = 0; k < warp; ++k) pre += ws[k];
        const int c0 = carry;
        if (i < w1) wpre[i] = c0 + pre + x - v;
        __syncthreads();
        if (threadIdx.x == ST - 1) carry = c0 + pre + x;
        __syncthreads();
    }
    if (threadIdx.x == 0) count[s] = carry;
}

// local index of row r in subdomain s (r must be a member)
__device__ __forceinline__ int rank_in(const Bits& b, const int* wpre, int s, int r) {
    const int x = r - b.lo[s];
    const int wi = b.woff[s] + (x >> 5);
    return wpre[wi] + __popc(b.w[wi] & ((1u << (x & 31)) - 1u));
}
__device__ __forceinline__ bool member(const Bits& b, int s, int r) {
    const int x = r - b.lo[s];
    if (x < 0) return false;
    const int wi = b.woff[s] + (x >> 5);
    if (wi >= b.woff[s + 1]) return false;
    return (b.w[wi] >> (x & 31)) & 1u;
}

// the sorted row list of every subdomain
__global__ void k_fill_sub(Bits b, const int* wpre, const int* sub_ptr, int nw, int* sub) {
    for (int wi = blockIdx.x * blockDim.x + threadIdx.x; wi < nw; wi += gridDim.x * blockDim.x) {
        unsigned m = b.w[wi];
        if (!m) continue;
        const int s = segment_of(b.woff, b.P, wi);
        const int r0 = b.lo[s] + 32 * (wi - b.woff[s]);
        int pos = sub_ptr[s] + wpre[wi];
        while (m) {
            const int bit = __ffs(m) - 1;
            m &= m - 1;
            sub[pos++] = r0 + bit;
        }
    }
}

// owned-local map: position of every owned row in its subdomain's list
__global__ void k_fill_ownloc(const int* owned, const int* part, int n, Bits b, const int* wpre,
                              int* ownloc) {
    for (int q = blockIdx.x * blockDim.x + threadIdx.x; q < n; q += gridDim.x * blockDim.x) {
        const int r = owned[q];
        ownloc[q] = rank_in(b, wpre, part[r], r);
    }
}

// ------------------------------------------------------------ local CSR
__global__ void k_local_count(const int* sub, const int* sub_ptr, int P, int nsub,
                              const int* rp, const int* ci, Bits b, int* cnt) {
    for (int L = blockIdx.x * blockDim.x + threadIdx.x; L < nsub; L += gridDim.x * blockDim.x) {
        const int s = segment_of(sub_ptr, P, L);
        const int g = sub[L];
        int c = 0;
        for (int e = rp[g]; e < rp[g + 1]; ++e) c += member(b, s, ci[e]) ? 1 : 0;
        cnt[L] = c;
    }
}

struct LocalOut {
    int* lrp;        // concatenated: n_s + 1 entries per subdomain, local offsets
    int* lci;
    int* lmap;
    int* ldiag;      // [nsub] entry of the diagonal within its subdomain (-1: none)
    int* wl;         // [P] widest lower / upper triangle of a row
    int* wu;
    int* miss;       // [P] first local row without a diagonal (INT_MAX: none)
};

__global__ void k_local_fill(const int* sub, const int* sub_ptr, int P, int nsub, const int* rp,
                             const int* ci, Bits b, const int* wpre, const long long* G,
                             LocalOut o) {
    for (int L = blockIdx.x * blockDim.x + threadIdx.x; L < nsub; L += gridDim.x * blockDim.x) {
        const int s = segment_of(sub_ptr, P, L);
        const int li = L - sub_ptr[s];
        const long long nz0 = G[sub_ptr[s]];
        const long long base = G[L];
        const int g = sub[L];
        int k = 0, dg = -1, lower = 0;
        for (int e = rp[g]; e < rp[g + 1]; ++e) {
            const int c = ci[e];
            if (!member(b, s, c)) continue;
            const int lj = rank_in(b, wpre, s, c);
            o.lci[base + k] = lj;
            o.lmap[base + k] = e;
            if (lj == li && dg < 0) dg = k;
            if (lj < li && lower == k) ++lower;  // leading entries left of the diagonal
            ++k;
        }
        o.lrp[L + s] = (int)(base - nz0);
        if (L + 1 == sub_ptr[s + 1]) o.lrp[L + 1 + s] = (int)(base + k - nz0);
        o.ldiag[L] = dg >= 0 ? (int)(base - nz0) + dg : -1;
        atomicMax(&o.wl[s], lower);
        if (dg >= 0) atomicMax(&o.wu[s], k - (dg + 1));
        else atomicMin(&o.miss[s], li);
    }
}

// ------------------------------------------------------------ level schedules
struct LevArgs {
    const int* sub_ptr;
    const int* lrp;     // concatenated local row pointers
    const int* lci;
    const int* ldiag;
    const long long* nz0;  // [P] first entry of every subdomain
    int* lev_lo;
    int* lev_up;
    int* nlev;          // [2P]: forward, backward level counts
    int P;
    int* bad;           // set when a relaxation did not settle (never, for a valid CSR)
};

// One block per subdomain: the forward and backward levels (levels_lower /
// levels_upper of setup.cpp) as the fixed point of
//   lev(i) = max(lev(c) + 1 over the row's lower (upper) columns c), 0 if none,
// relaxed in place by all threads until a pass changes nothing.  The fixed
// point of this recurrence over a DAG is unique (the longest path into the
// row), so the result is the serial loop's whatever the update order; a pass
// propagates at least one more level, and in natural order usually many.
// Levels live in shared memory when the subdomain fits (else in global).
constexpr int LV_T = 256;

__device__ __forceinline__ int lev_pass(const int* rp, const int* ci, const int* dg, int ns,
                                        int* lev, bool back) {
    int changed = 0;
    for (int i = threadIdx.x; i < ns; i += LV_T) {
        const int r = back ? ns - 1 - i : i;
        int l = 0;
        if (!back) {
            for (int e = rp[r]; e < rp[r + 1]; ++e) {
                const int c = ci[e];
                if (c >= r) break;
                l = max(l, ((volatile int*)lev)[c] + 1);
            }
        } else {
            // a repeated diagonal entry (c == r) counts as level 0 + 1: the
            // serial loop reads the row's own level before writing it
            for (int e = dg[r] + 1; e < rp[r + 1]; ++e) {
                const int c = ci[e];
                l = max(l, c == r ? 1 : ((volatile int*)lev)[c] + 1);
            }
        }
        if (l != ((volatile int*)lev)[r]) {
            ((volatile int*)lev)[r] = l;
            changed = 1;
        }
    }
    return __syncthreads_or(changed);
}

__global__ void __launch_bounds__(LV_T) k_levels(LevArgs a, int smem_rows) {
    extern __shared__ int slev[];
    const int s = blockIdx.x;
    const int r0 = a.sub_ptr[s], ns = a.sub_ptr[s + 1] - r0;
    const int* rp = a.lrp + r0 + s;
    const int* ci = a.lci + a.nz0[s];
    const int* dg = a.ldiag + r0;
    for (int dir = 0; dir < 2; ++dir) {
        int* out = (dir ? a.lev_up : a.lev_lo) + r0;
        int* lev = ns <= smem_rows ? slev : out;  // out is zero on entry
        if (lev == slev)
            for (int i = threadIdx.x; i < ns; i += LV_T) slev[i] = 0;
        __syncthreads();
        // the fixed point needs at most (longest path + 1) <= ns + 1 passes;
        // the bound makes any error in the recurrence end with a status
        // instead of a loop that never ends
        int pass = 0;
        while (lev_pass(rp, ci, dg, ns, lev, dir == 1)) {
            if (++pass > ns + 1) {
                if (threadIdx.x == 0) atomicExch(a.bad, 1);
                break;
            }
        }
        int nl = 0;
        for (int i = threadIdx.x; i < ns; i += LV_T) {
            const int l = lev[i];
            nl = max(nl, l + 1);
            if (lev == slev) out[i] = l;
        }
        nl = __reduce_max_sync(0xffffffffu, nl);
        __shared__ int s_nl[LV_T / 32];
        if ((threadIdx.x & 31) == 0) s_nl[threadIdx.x >> 5] = nl;
        __syncthreads();
        if (threadIdx.x == 0) {
            int m = 0;
            for (int w = 0; w < LV_T / 32; ++w) m = max(m, s_nl[w]);
            a.nlev[dir * a.P + s] = m;
        }
        __syncthreads();
    }
}

// One block per subdomain and direction: rows placed by level, stable
// (level_order of setup.cpp).  All threads count per level; warp 0 places
// the rows 32 at a time in row order (equal levels ranked by
// __match_any_sync), advancing per-level cursors.  ptr (nlev + 1 entries,
// zero on entry) is in global memory; the cursors in shared memory when
// they fit.
__global__ void __launch_bounds__(LV_T) k_level_order(const int* sub_ptr, const int* lev_lo,
                                                      const int* lev_up, const int* lev_off_f,
                                                      const int* lev_off_b, const int* nlev,
                                                      int P, int* ptr_f, int* ptr_b, int* perm_f,
                                                      int* perm_b, int smem_levels) {
    extern __shared__ int scur[];
    const int t = blockIdx.x;
    const int s = t % P;
    const bool back = t >= P;
    const int r0 = sub_ptr[s], ns = sub_ptr[s + 1] - r0;
    const int* lev = (back ? lev_up : lev_lo) + r0;
    int* ptr = back ? ptr_b + lev_off_b[s] : ptr_f + lev_off_f[s];
    int* perm = (back ? perm_b : perm_f) + r0;
    const int nl = nlev[t];
    for (int i = threadIdx.x; i < ns; i += LV_T) atomicAdd(&ptr[lev[i] + 1], 1);
    __syncthreads();
    if (threadIdx.x == 0)
        for (int l = 0; l < nl; ++l) ptr[l + 1] += ptr[l];
    __syncthreads();
    int* cur = nl <= smem_levels ? scur : nullptr;
    if (threadIdx.x < 32) {
        const int lane = threadIdx.x;
        if (cur)
            for (int l = lane; l < nl; l += 32) cur[l] = ptr[l];
        __syncwarp();
        const unsigned lt = (1u << lane) - 1u;
        for (int i0 = 0; i0 < ns; i0 += 32) {
            const int i = i0 + lane;
            const bool valid = i < ns;
            const int l = valid ? lev[i] : -1 - lane;
            const unsigned peers = __match_any_sync(0xffffffffu, l);
            int base = 0;
            if (valid) base = cur ? cur[l] : ptr[l];
            __syncwarp();
            if (valid) {
                perm[base + __popc(peers & lt)] = i;
                if (lane == __ffs(peers) - 1) {
                    if (cur) cur[l] = base + __popc(peers);
                    else ptr[l] = base + __popc(peers);
                }
            }
            __syncwarp();
        }
        if (!cur) {
            // the cursors ran in ptr: each advanced to the next level's start
            __syncwarp();
            if (lane == 0) {
                for (int l = nl; l > 0; --l) ptr[l] = ptr[l - 1];
                ptr[0] = 0;
            }
        }
    }
}

// ------------------------------------------------------------ slot layout
struct BankArgs {
    const int* sub_ptr;
    const int* lrp;
    const int* lci;
    const int* ldiag;
    const long long* nz0;
    const int* perm_f;
    const int* perm_b;
    const int* ptr_f;
    const int* ptr_b;
    const int* lev_off_f;
    const int* lev_off_b;
    const int* nlev;
    const int* wl;
    const int* wu;
    long long* cost;   // [P][3] for shifts 0, 5, 4
    int P;
    int words;         // 4-byte banks per element
};

__device__ __forceinline__ int tslot_dev(int r, int p) { return p ? r + (r >> p) : r; }

// the largest number of distinct slots that share a bank among the m < 32
// lanes' slots (the host's load_cost)
__device__ __forceinline__ int warp_load_cost(int slot, bool valid, int words) {
    const int lane = threadIdx.x & 31;
    const unsigned ps = __match_any_sync(0xffffffffu, valid ? slot : -1 - lane);
    const bool first = valid && lane == __ffs(ps) - 1;
    const int bank = (int)(((long long)slot * words) % 32) / words;
    const unsigned pb = __match_any_sync(0xffffffffu, first ? bank : 32 + lane);
    int c = first ? __popc(pb) : 0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c = max(c, __shfl_xor_sync(0xffffffffu, c, o));
    return c;
}

// one warp per (subdomain, shift candidate)
__global__ void k_bank_cost(BankArgs a) {
    const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (wid >= 3 * a.P) return;
    const int s = wid / 3, cand = wid % 3;
    const int p = cand == 0 ? 0 : (cand == 1 ? 5 : 4);
    const int r0 = a.sub_ptr[s], ns = a.sub_ptr[s + 1] - r0;
    const int* rp = a.lrp + r0 + s;
    const int* ci = a.lci + a.nz0[s];
    const int* dg = a.ldiag + r0;
    long long cost = 0;
    for (int pass = 0; pass < 2; ++pass) {
        const int* perm = (pass ? a.perm_b : a.perm_f) + r0;
        const int* ptr = pass ? a.ptr_b + a.lev_off_b[s] : a.ptr_f + a.lev_off_f[s];
        const int nl = a.nlev[pass * a.P + s];
        const int w = pass ? a.wu[s] : a.wl[s];
        for (int l = 0; l < nl; ++l) {
            for (int q0 = ptr[l]; q0 < ptr[l + 1]; q0 += 32) {
                const int m = min(32, ptr[l + 1] - q0);
                const bool valid = lane < m;
                const int r = valid ? perm[q0 + lane] : 0;
                cost += warp_load_cost(tslot_dev(r, p), valid, a.words);
                for (int k = 0; k < w; ++k) {
                    int col = ns;
                    if (valid) {
                        if (pass == 0) {
                            const int e = rp[r] + k;
                            if (e < rp[r + 1] && ci[e] < r) col = ci[e];
                        } else {
                            const int e = dg[r] + 1 + k;
                            if (e < rp[r + 1]) col = ci[e];
                        }
                    }
                    cost += warp_load_cost(tslot_dev(col, p), valid, a.words);
                }
            }
        }
    }
    if (lane == 0) a.cost[wid] = cost;
}

int grid_for(const sg_ctx* ctx, long long n) {
    const long long need = (n + ST - 1) / ST;
    const long long cap = (long long)ctx->num_sms * 8;
    return (int)std::max(1ll, std::min(need, cap));
}

// exclusive scan of n int counts into out (long long); returns the total
// (n <= SC_B * SC_B, checked by the caller)
long long device_scan(const int* in, long long n, long long* out, DBuf<long long>& scratch,
                      cudaStream_t st) {
    const long long nb = (n + SC_B - 1) / SC_B;
    if (scratch.n < (size_t)nb + 1) scratch.alloc((size_t)nb + 1);
    if (n > 0) {
        k_scan_blocks<<<(unsigned)nb, SC_T, 0, st>>>(in, n, out, scratch.p);
        k_scan_sums<<<1, SC_T, 0, st>>>(scratch.p, (int)nb, scratch.p + nb);
        k_scan_add<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(out, n, scratch.p);
        SG_CUDA(cudaGetLastError());
    }
    long long total = 0;
    if (n > 0)
        SG_CUDA(cudaMemcpyAsync(&total, scratch.p + nb, sizeof(long long), cudaMemcpyDeviceToHost, st));
    SG_CUDA(cudaStreamSynchronize(st));
    return total;
}

template <class T>
void download(std::vector<T>& h, const T* d, size_t n, cudaStream_t st) {
    h.resize(n);
    if (n) SG_CUDA(cudaMemcpyAsync(h.data(), d, n * sizeof(T), cudaMemcpyDeviceToHost, st));
}

}  // namespace

// The device set-up; false (pc untouched) when it does not apply: then the
// caller runs the host set-up.  Same checks and messages as the host path.
bool build_schwarz_device(sg_precond* pc, const sg_csr* A, const int* part_in, int nparts,
                          int overlap) {
    sg_ctx* ctx = pc->ctx;
    cudaStream_t st = ctx->stream;
    const int n = A->nrows;
    SG_CHECK_ARG(nparts >= 1, "nparts must be >= 1 (got %d)", nparts);
    SG_CHECK_ARG(overlap >= 0, "overlap must be >= 0 (got %d)", overlap);
    SG_CHECK_ARG(A->nrows == A->ncols, "Schwarz/ILU preconditioners need a square matrix");
    SG_CHECK_ARG(A->sorted, "ILU(0) needs column indices sorted within each row");
    for (int i = 0; i < n; ++i)
        SG_CHECK_ARG(part_in[i] >= 0 && part_in[i] < nparts,
                     "partition[%d] = %d is outside [0,%d)", i, part_in[i], nparts);
    // (the radix sort scans 256 counts per 4096 rows; the scan covers SC_B^2)
    if (n < 1 || (long long)n / 16 > (long long)SC_B * SC_B) return false;
    const int P = nparts;
    DBuf<int> d_part, d_cnt, d_optr, d_owned, d_key2, d_val2, d_hist, d_bw, d_ends;
    DBuf<long long> d_off, scan_scratch;
    d_part.upload(part_in, (size_t)n, st);
    // ---- owned lists
    d_cnt.alloc((size_t)P);
    d_cnt.zero(st);
    k_count_parts<<<grid_for(ctx, n), ST, 0, st>>>(d_part.p, n, d_cnt.p);
    SG_CUDA(cudaGetLastError());
    std::vector<int> cnt;
    download(cnt, d_cnt.p, (size_t)P, st);
    SG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> optr((size_t)P + 1, 0);
    for (int s = 0; s < P; ++s) optr[s + 1] = optr[s] + cnt[s];
    for (int s = 0; s < P; ++s)
        if (cnt[s] == 0) fail(SG_ERR_INVALID_ARG, "subdomain %d owns no rows", s);
    d_optr.upload(optr, st);
    {
        const int nb = (n + RS_CH - 1) / RS_CH;
        DBuf<int> k0, v0;
        k0.alloc((size_t)n);
        v0.alloc((size_t)n);
        d_key2.alloc((size_t)n);
        d_val2.alloc((size_t)n);
        SG_CUDA(cudaMemcpyAsync(k0.p, d_part.p, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
        k_iota<<<grid_for(ctx, n), ST, 0, st>>>(v0.p, n);
        d_hist.alloc((size_t)256 * nb);
        d_off.alloc((size_t)256 * nb);
        int* kin = k0.p;
        int* vin = v0.p;
        int* kout = d_key2.p;
        int* vout = d_val2.p;
        for (int shift = 0; shift == 0 || ((P - 1) >> shift) > 0; shift += 8) {
            k_rs_hist<<<nb, 256, 0, st>>>(kin, n, shift, nb, d_hist.p);
            SG_CUDA(cudaGetLastError());
            device_scan(d_hist.p, (long long)256 * nb, d_off.p, scan_scratch, st);
            k_rs_scatter<<<nb, 32, 0, st>>>(kin, vin, n, shift, nb, d_off.p, kout, vout);
            SG_CUDA(cudaGetLastError());
            std::swap(kin, kout);
            std::swap(vin, vout);
        }
        d_owned.alloc((size_t)n);
        SG_CUDA(cudaMemcpyAsync(d_owned.p, vin, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
    }
    // ---- bitmap ranges from the half bandwidths
    d_bw.alloc(2);
    d_bw.zero(st);
    k_bandwidth<<<grid_for(ctx, n), ST, 0, st>>>(A->rp.p, A->ci.p, n, d_bw.p);
    d_ends.alloc((size_t)2 * P);
    k_owned_ends<<<(P + 255) / 256, 256, 0, st>>>(d_owned.p, d_optr.p, P, d_ends.p);
    SG_CUDA(cudaGetLastError());
    std::vector<int> bw, ends;
    download(bw, d_bw.p, 2, st);
    download(ends, d_ends.p, (size_t)2 * P, st);
    SG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> lo((size_t)P), woff((size_t)P + 1, 0);
    for (int s = 0; s < P; ++s) {
        const long long l = std::max(0ll, (long long)ends[2 * s] - (long long)overlap * bw[0]);
        const long long h = std::min((long long)n - 1, (long long)ends[2 * s + 1] + (long long)overlap * bw[1]);
        lo[s] = (int)l;
        const long long words = (h - l) / 32 + 1;
        if ((long long)woff[s] + words > INT_MAX / 2) return false;
        woff[s + 1] = woff[s] + (int)words;
    }
    const long long nw = woff[P];
    // bitmaps: one (overlap <= 1) or three (frontiers of later layers) copies
    size_t free_b = 0, total_b = 0;
    SG_CUDA(cudaMemGetInfo(&free_b, &total_b));
    const long long bytes = nw * 4 * (overlap >= 2 ? 3 : 1);
    if (bytes > (long long)(free_b / 4) || bytes > (4ll << 30)) return false;
    DBuf<int> d_lo, d_woff, d_bad, d_wpre, d_scount, d_sptr;
    DBuf<unsigned> d_bm, d_old, d_front;
    d_lo.upload(lo, st);
    d_woff.upload(woff, st);
    d_bm.alloc((size_t)nw);
    d_bm.zero(st);
    d_bad.alloc(1);
    d_bad.zero(st);
    Bits b{d_lo.p, d_woff.p, d_bm.p, P};
    k_mark_owned<<<grid_for(ctx, n), ST, 0, st>>>(d_owned.p, d_part.p, n, b, d_bad.p);
    if (overlap >= 2) {
        d_old.alloc((size_t)nw);
        d_front.alloc((size_t)nw);
        SG_CUDA(cudaMemcpyAsync(d_old.p, d_bm.p, sizeof(unsigned) * nw, cudaMemcpyDeviceToDevice, st));
    }
    if (overlap >= 1)
        k_expand_owned<<<grid_for(ctx, n), ST, 0, st>>>(d_owned.p, d_part.p, n, A->rp.p, A->ci.p,
                                                         b, d_bad.p);
    for (int layer = 2; layer <= overlap; ++layer) {
        k_andnot<<<grid_for(ctx, nw), ST, 0, st>>>(d_bm.p, d_old.p, d_front.p, (int)nw);
        SG_CUDA(cudaMemcpyAsync(d_old.p, d_bm.p, sizeof(unsigned) * nw, cudaMemcpyDeviceToDevice, st));
        k_expand_bits<<<grid_for(ctx, nw), ST, 0, st>>>(d_front.p, (int)nw, A->rp.p, A->ci.p, b,
                                                        d_bad.p);
    }
    SG_CUDA(cudaGetLastError());
    d_old.release();
    d_front.release();
    // ---- sorted lists, owned-local map
    d_wpre.alloc((size_t)nw);
    d_scount.alloc((size_t)P);
    k_word_prefix<<<P, ST, 0, st>>>(d_bm.p, d_woff.p, d_wpre.p, d_scount.p);
    SG_CUDA(cudaGetLastError());
    std::vector<int> scount, bad;
    download(scount, d_scount.p, (size_t)P, st);
    download(bad, d_bad.p, 1, st);
    SG_CUDA(cudaStreamSynchronize(st));
    if (bad[0]) fail(SG_ERR_INTERNAL, "device set-up: a neighbour left its bitmap range");
    std::vector<int> sptr((size_t)P + 1, 0);
    for (int s = 0; s < P; ++s) {
        if ((long long)sptr[s] + scount[s] > INT_MAX / 2) return false;
        sptr[s + 1] = sptr[s] + scount[s];
    }
    const int nsub = sptr[P];
    if ((long long)nsub > (long long)SC_B * SC_B) return false;  // beyond one device scan
    d_sptr.upload(sptr, st);
    DBuf<int> d_sub, d_ownloc;
    d_sub.alloc((size_t)nsub);
    d_ownloc.alloc((size_t)n);
    k_fill_sub<<<grid_for(ctx, nw), ST, 0, st>>>(b, d_wpre.p, d_sptr.p, (int)nw, d_sub.p);
    k_fill_ownloc<<<grid_for(ctx, n), ST, 0, st>>>(d_owned.p, d_part.p, n, b, d_wpre.p, d_ownloc.p);
    SG_CUDA(cudaGetLastError());
    // ---- local CSR
    DBuf<int> d_rcnt, d_lrp, d_lci, d_lmap, d_ldiag, d_wl, d_wu, d_miss;
    DBuf<long long> d_G;
    d_rcnt.alloc((size_t)nsub);
    k_local_count<<<grid_for(ctx, nsub), ST, 0, st>>>(d_sub.p, d_sptr.p, P, nsub, A->rp.p,
                                                      A->ci.p, b, d_rcnt.p);
    SG_CUDA(cudaGetLastError());
    d_G.alloc((size_t)nsub + 1);
    const long long nnz_loc = device_scan(d_rcnt.p, nsub, d_G.p, scan_scratch, st);
    if (nnz_loc > INT_MAX) return false;
    SG_CUDA(cudaMemcpyAsync(d_G.p + nsub, &nnz_loc, sizeof(long long), cudaMemcpyHostToDevice, st));
    d_rcnt.release();
    d_lrp.alloc((size_t)nsub + P);
    d_lci.alloc((size_t)std::max(1ll, nnz_loc));
    d_lmap.alloc((size_t)std::max(1ll, nnz_loc));
    d_ldiag.alloc((size_t)nsub);
    d_wl.alloc((size_t)P);
    d_wu.alloc((size_t)P);
    d_wl.zero(st);
    d_wu.zero(st);
    d_miss.alloc((size_t)P);
    {
        std::vector<int> big((size_t)P, INT_MAX);
        d_miss.upload(big, st);
    }
    LocalOut o{d_lrp.p, d_lci.p, d_lmap.p, d_ldiag.p, d_wl.p, d_wu.p, d_miss.p};
    k_local_fill<<<grid_for(ctx, nsub), ST, 0, st>>>(d_sub.p, d_sptr.p, P, nsub, A->rp.p,
                                                     A->ci.p, b, d_wpre.p, d_G.p, o);
    SG_CUDA(cudaGetLastError());
    std::vector<int> miss, wl, wu;
    std::vector<long long> G;
    download(miss, d_miss.p, (size_t)P, st);
    download(wl, d_wl.p, (size_t)P, st);
    download(wu, d_wu.p, (size_t)P, st);
    download(G, d_G.p, (size_t)nsub + 1, st);
    SG_CUDA(cudaStreamSynchronize(st));
    std::vector<int> sub_h;
    download(sub_h, d_sub.p, (size_t)nsub, st);
    SG_CUDA(cudaStreamSynchronize(st));
    for (int s = 0; s < P; ++s)
        if (miss[s] != INT_MAX)
            fail(SG_ERR_SINGULAR, "ILU(0): row %d has no diagonal entry", sub_h[sptr[s] + miss[s]]);
    // ---- level schedules
    std::vector<long long> nz0((size_t)P);
    for (int s = 0; s < P; ++s) nz0[s] = G[sptr[s]];
    DBuf<long long> d_nz0;
    DBuf<int> d_lev_lo, d_lev_up, d_nlev;
    d_nz0.upload(nz0, st);
    d_lev_lo.alloc((size_t)nsub);
    d_lev_up.alloc((size_t)nsub);
    d_lev_lo.zero(st);  // as the host's level arrays: a repeated diagonal entry reads 0
    d_lev_up.zero(st);
    d_nlev.alloc((size_t)2 * P);
    d_bad.zero(st);
    LevArgs la{d_sptr.p, d_lrp.p, d_lci.p, d_ldiag.p, d_nz0.p, d_lev_lo.p, d_lev_up.p, d_nlev.p, P,
               d_bad.p};
    const int lv_smem_rows = 24 * 1024;  // 96 KB of shared levels per block at most
    int max_ns = 0;
    for (int s = 0; s < P; ++s) max_ns = std::max(max_ns, sptr[s + 1] - sptr[s]);
    const size_t lv_smem = sizeof(int) * (size_t)std::min(max_ns, lv_smem_rows);
    SG_CUDA(cudaFuncSetAttribute(k_levels, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lv_smem));
    k_levels<<<P, LV_T, lv_smem, st>>>(la, lv_smem_rows);
    SG_CUDA(cudaGetLastError());
    std::vector<int> nlev;
    download(nlev, d_nlev.p, (size_t)2 * P, st);
    download(bad, d_bad.p, 1, st);
    SG_CUDA(cudaStreamSynchronize(st));
    if (bad[0]) fail(SG_ERR_INTERNAL, "device set-up: a level schedule did not settle");
    std::vector<int> loff_f((size_t)P), loff_b((size_t)P);
    long long tf = 0, tb = 0;
    for (int s = 0; s < P; ++s) {
        loff_f[s] = (int)tf;
        loff_b[s] = (int)tb;
        tf += nlev[s] + 1;
        tb += nlev[P + s] + 1;
    }
    DBuf<int> d_loff_f, d_loff_b, d_ptr_f, d_ptr_b, d_perm_f, d_perm_b;
    d_loff_f.upload(loff_f, st);
    d_loff_b.upload(loff_b, st);
    d_ptr_f.alloc((size_t)tf);
    d_ptr_b.alloc((size_t)tb);
    d_ptr_f.zero(st);
    d_ptr_b.zero(st);
    d_perm_f.alloc((size_t)nsub);
    d_perm_b.alloc((size_t)nsub);
    int max_nl = 0;
    for (int t = 0; t < 2 * P; ++t) max_nl = std::max(max_nl, nlev[t]);
    const int lo_smem_levels = 16 * 1024;
    const size_t lo_smem = sizeof(int) * (size_t)std::min(max_nl, lo_smem_levels);
    SG_CUDA(cudaFuncSetAttribute(k_level_order, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)std::max<size_t>(lo_smem, 4)));
    k_level_order<<<2 * P, LV_T, std::max<size_t>(lo_smem, 4), st>>>(
        d_sptr.p, d_lev_lo.p, d_lev_up.p, d_loff_f.p, d_loff_b.p, d_nlev.p, P, d_ptr_f.p,
        d_ptr_b.p, d_perm_f.p, d_perm_b.p, lo_smem_levels);
    SG_CUDA(cudaGetLastError());
    // ---- slot layout
    DBuf<long long> d_cost;
    d_cost.alloc((size_t)3 * P);
    BankArgs ba{d_sptr.p, d_lrp.p, d_lci.p, d_ldiag.p, d_nz0.p, d_perm_f.p, d_perm_b.p,
                d_ptr_f.p, d_ptr_b.p, d_loff_f.p, d_loff_b.p, d_nlev.p, d_wl.p, d_wu.p,
                d_cost.p, P, pc->opts.sweep_dtype == SG_FP64 ? 2 : 1};
    k_bank_cost<<<(3 * P * 32 + 255) / 256, 256, 0, st>>>(ba);
    SG_CUDA(cudaGetLastError());
    // ---- everything back into the host structures of build_schwarz_host
    std::vector<long long> cost;
    std::vector<int> perm_f_all, perm_b_all;
    pc->nparts = P;
    pc->part.assign(part_in, part_in + n);
    pc->owned_ptr = optr;
    download(pc->owned, d_owned.p, (size_t)n, st);
    pc->sub_ptr = sptr;
    pc->sub.swap(sub_h);
    pc->ownloc_ptr = optr;
    download(pc->ownloc, d_ownloc.p, (size_t)n, st);
    download(pc->lrp, d_lrp.p, (size_t)nsub + P, st);
    download(pc->lci, d_lci.p, (size_t)nnz_loc, st);
    download(pc->lmap, d_lmap.p, (size_t)nnz_loc, st);
    download(pc->ldiag, d_ldiag.p, (size_t)nsub, st);
    download(pc->lev_lo, d_lev_lo.p, (size_t)nsub, st);
    download(pc->lev_up, d_lev_up.p, (size_t)nsub, st);
    download(pc->h_lev_ptr_f, d_ptr_f.p, (size_t)tf, st);
    download(pc->h_lev_ptr_b, d_ptr_b.p, (size_t)tb, st);
    download(perm_f_all, d_perm_f.p, (size_t)nsub, st);
    download(perm_b_all, d_perm_b.p, (size_t)nsub, st);
    download(cost, d_cost.p, (size_t)3 * P, st);
    SG_CUDA(cudaStreamSynchronize(st));
    pc->h_info.assign(P, SubInfo{});
    for (int s = 0; s < P; ++s) {
        SubInfo& inf = pc->h_info[s];
        const int ns = sptr[s + 1] - sptr[s];
        inf.n = ns;
        inf.row_off = sptr[s];
        inf.nlev_f = nlev[s];
        inf.nlev_b = nlev[P + s];
        inf.lev_off_f = loff_f[s];
        inf.lev_off_b = loff_b[s];
        inf.wl = wl[s];
        inf.wu = wu[s];
        inf.n_own = optr[s + 1] - optr[s];
        inf.own_off = optr[s];
        inf.csr_row_off = sptr[s] + s;
        inf.csr_nz_off = nz0[s];
        inf.cscale = 1.0 / std::sqrt((double)(optr[s + 1] - optr[s]));
        // slot layout: the cheapest of none / one pad word per 32 / per 16
        // rows, first in that order on ties (as the host set-up)
        inf.tshift = 0;
        long long best = -1;
        const int shifts[3] = {0, 5, 4};
        for (int c = 0; c < 3; ++c) {
            const int p = shifts[c];
            if (tslot(ns, p) > 65535) continue;
            if (best < 0 || cost[3 * s + c] < best) {
                best = cost[3 * s + c];
                inf.tshift = p;
            }
        }
    }
    schwarz_finish(pc, perm_f_all, perm_b_all);
    return true;
}

}  // namespace sg
