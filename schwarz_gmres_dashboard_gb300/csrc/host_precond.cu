// host_precond.cu -- a preconditioner that is a caller's host function: the
// flexible apply of FGMRES (FlexApply / fgmres_flex, src/core/fgmres.h:37,
// src/core/fgmres.cpp:164-172) and any Preconditioner plugin that is not one
// of the GPU kinds (src/precond/preconditioner.h:7-20).
//
// Inside a solve the apply is three stream-ordered steps: a device-to-host
// copy of the input (and of the launch's active flag and, for FGMRES, the
// basis vector's scale) into pinned buffers, cudaLaunchHostFunc running the
// caller's function on them, and a host-to-device copy of the output.  No
// host synchronisation is needed, and the steps are captured into the
// restart cycle's CUDA graph like any kernel.  An FP32 vector travels as
// FP32 and is widened / narrowed on the host around the call.
#include <cstring>

#include "dev_common.cuh"
#include "kernels.h"

namespace sg {

namespace {

template <class TI, class TO, bool SCALED, bool GATED>
void CUDART_CB host_apply_cb(void* data) {
    sg_precond* pc = static_cast<sg_precond*>(data);
    sg_precond::HostCtl* c = pc->h_ctl.p;
    if (GATED && !c->active) return;  // the cycle stopped: the output is never read
    c->calls++;
    const int n = pc->n;
    double* in = pc->h_in.p;
    double* out = pc->h_out.p;
    if (sizeof(TI) == sizeof(float)) {
        // widen in place, back to front (double i overwrites floats 2i, 2i+1,
        // which were already read)
        const float* f = reinterpret_cast<const float*>(in);
        for (int i = n - 1; i >= 0; --i) in[i] = (double)f[i];
    }
    const double s = SCALED ? c->scale : 1.0;
    if (SCALED)
        for (int i = 0; i < n; ++i) in[i] *= s;
    const int st = pc->host_fn(pc->host_user, in, out, n);
    if (st != 0 && c->status == 0) c->status = st;
    if (SCALED) {
        // the solver keeps directions in the units of the stored (unscaled)
        // basis vector: z_raw = M(s raw) / s
        const double inv = 1.0 / s;
        for (int i = 0; i < n; ++i) out[i] *= inv;
    }
    if (sizeof(TO) == sizeof(float)) {
        float* f = reinterpret_cast<float*>(out);
        for (int i = 0; i < n; ++i) f[i] = (float)out[i];
    }
}

template <class TI, class TO>
void enqueue_host_apply(sg_precond* pc, const TI* x, TO* y, const int* active,
                        const double* scale) {
    sg_ctx* ctx = pc->ctx;
    cudaStream_t s = ctx->stream;
    const int n = pc->n;
    sg_precond::HostCtl* c = pc->h_ctl.p;
    if (active)
        SG_CUDA(cudaMemcpyAsync(&c->active, active, sizeof(int), cudaMemcpyDeviceToHost, s));
    if (scale)
        SG_CUDA(cudaMemcpyAsync(&c->scale, scale, sizeof(double), cudaMemcpyDeviceToHost, s));
    SG_CUDA(cudaMemcpyAsync(pc->h_in.p, x, sizeof(TI) * (size_t)n, cudaMemcpyDeviceToHost, s));
    cudaHostFn_t fn;
    if (active) fn = scale ? host_apply_cb<TI, TO, true, true> : host_apply_cb<TI, TO, false, true>;
    else fn = scale ? host_apply_cb<TI, TO, true, false> : host_apply_cb<TI, TO, false, false>;
    SG_CUDA(cudaLaunchHostFunc(s, fn, pc));
    SG_CUDA(cudaMemcpyAsync(y, pc->h_out.p, sizeof(TO) * (size_t)n, cudaMemcpyHostToDevice, s));
}

}  // namespace

void host_precond_init(sg_precond* pc, sg_host_apply_fn fn, void* user, int n) {
    pc->kind = SG_PC_HOST;
    pc->host_fn = fn;
    pc->host_user = user;
    pc->n = n;
    pc->h_in.alloc((size_t)n);
    pc->h_out.alloc((size_t)n);
    pc->h_ctl.alloc(1);
    std::memset(pc->h_ctl.p, 0, sizeof(sg_precond::HostCtl));
    pc->h_ctl.p->active = 1;
    pc->h_ctl.p->scale = 1.0;
    pc->is_setup = true;
}

// the first error the function reported since the last call (then cleared)
int host_precond_status(sg_precond* pc) {
    if (pc->kind != SG_PC_HOST) return 0;
    const int st = pc->h_ctl.p->status;
    pc->h_ctl.p->status = 0;
    return st;
}

long long host_precond_calls(const sg_precond* pc) {
    return pc->kind == SG_PC_HOST ? pc->h_ctl.p->calls : 0;
}

template <class TI, class TO>
void host_precond_apply(sg_precond* pc, const TI* x, TO* y, const int* active,
                        const double* scale) {
    enqueue_host_apply<TI, TO>(pc, x, y, active, scale);
}

template void host_precond_apply<double, double>(sg_precond*, const double*, double*, const int*,
                                                 const double*);
template void host_precond_apply<double, float>(sg_precond*, const double*, float*, const int*,
                                                const double*);
template void host_precond_apply<float, float>(sg_precond*, const float*, float*, const int*,
                                               const double*);

}  // namespace sg
