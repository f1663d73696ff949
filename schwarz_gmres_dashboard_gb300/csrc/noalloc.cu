// noalloc.cu -- a dot product that allocates nothing.
//
// Why it exists: some callers of this library cannot allocate device memory
// at the moment they need a reduction.
//  * Plug-ins hosted by an application that owns all device memory through
//    its own pool and forbids raw cudaMalloc/cudaFree once it has started.
//  * Real-time loops that cannot afford cudaMalloc's latency or the
//    implicit device-wide synchronisation of cudaFree.
// sg_dot needs scratch for its per-block partial sums and takes it from an
// sg_ctx, whose creation allocates.  sg_dot_noalloc runs the same kernel with
// that scratch in a fixed array compiled into this library instead.
//
// Limits and sharing
//  * The array holds 8192 partial sums (64 KiB); every GPU that loads the
//    library keeps it until the process exits.  One block sums 4096
//    elements, so n is limited to SG_DOT_NOALLOC_MAX_N = 8192 * 4096 =
//    33,554,432; a larger n is rejected with SG_ERR_INVALID_ARG before
//    anything is launched.
//  * Every call on a device uses the same array and arrival counter, and the
//    array keeps the last call's partial sums.  The counter is cleared before
//    each launch (a memset of 4 bytes, which allocates nothing).  Calls whose
//    kernels overlap on the GPU (different streams, or host threads calling
//    concurrently) race on the array and give wrong results: serialise them.
//  * The first call on a device, with that device current, looks up the
//    array's device address (cudaGetSymbolAddress) and caches it for the
//    life of the process; make that first call before any stream capture
//    begins.  cudaDeviceReset destroys the context the cached address
//    belongs to: do not call sg_dot_noalloc on that device afterwards.
#include <mutex>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

constexpr int NOALLOC_MAX_BLOCKS = 8192;
constexpr int NOALLOC_ROWS_PER_BLOCK = 4096;
static_assert((long long)NOALLOC_MAX_BLOCKS * NOALLOC_ROWS_PER_BLOCK == SG_DOT_NOALLOC_MAX_N,
              "header limit and scratch size disagree");
constexpr int NOALLOC_MAX_DEVICES = 64;

// the fixed scratch (per device that loads the library)
static __device__ __align__(256) double g_dot_partials[NOALLOC_MAX_BLOCKS];
static __device__ __align__(256) unsigned int g_dot_ticket[1];

struct NoallocScratch {
    double* partials = nullptr;
    unsigned int* ticket = nullptr;
    bool ready = false;
};
std::mutex g_noalloc_mu;
NoallocScratch g_noalloc[NOALLOC_MAX_DEVICES];

// Device addresses of the scratch on the current device (looked up once).
NoallocScratch noalloc_scratch() {
    int dev = 0;
    SG_CUDA(cudaGetDevice(&dev));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        fail(SG_ERR_UNSUPPORTED, "device %d is beyond the %d devices sg_dot_noalloc tracks", dev,
             NOALLOC_MAX_DEVICES);
    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    NoallocScratch& s = g_noalloc[dev];
    if (!s.ready) {
        void* p = nullptr;
        SG_CUDA(cudaGetSymbolAddress(&p, g_dot_partials));
        s.partials = static_cast<double*>(p);
        SG_CUDA(cudaGetSymbolAddress(&p, g_dot_ticket));
        s.ticket = static_cast<unsigned int*>(p);
        s.ready = true;
    }
    return s;
}

// status + thread-local message, as every other entry point reports errors
template <class F>
sg_status noalloc_guard(F&& f) {
    try {
        f();
        set_last_error("");
        return SG_OK;
    } catch (const Error& e) {
        set_last_error(e.msg.c_str());
        return e.status;
    } catch (...) {
        set_last_error("unknown internal error");
        return SG_ERR_INTERNAL;
    }
}

}  // namespace

}  // namespace sg

using namespace sg;

extern "C" sg_status sg_dot_noalloc(const double* x, const double* y, int n, double* result,
                                    void* stream) {
    return noalloc_guard([&] {
        SG_CHECK_ARG(result && (n == 0 || (x && y)), "NULL argument");
        SG_CHECK_ARG(n >= 0, "n must be >= 0");
        SG_CHECK_ARG((long long)n <= (long long)NOALLOC_MAX_BLOCKS * NOALLOC_ROWS_PER_BLOCK,
                     "n = %d exceeds the %lld elements sg_dot_noalloc's fixed scratch covers "
                     "(%d partial sums of %d elements)",
                     n, (long long)NOALLOC_MAX_BLOCKS * NOALLOC_ROWS_PER_BLOCK,
                     NOALLOC_MAX_BLOCKS, NOALLOC_ROWS_PER_BLOCK);
        const NoallocScratch sc = noalloc_scratch();
        cudaStream_t st = static_cast<cudaStream_t>(stream);
        const int blocks = n == 0 ? 1 : (n + NOALLOC_ROWS_PER_BLOCK - 1) / NOALLOC_ROWS_PER_BLOCK;
        SG_CUDA(cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned int), st));
        launch_dot_scratch(st, x, y, n, blocks, sc.partials, sc.ticket, result);
    });
}
