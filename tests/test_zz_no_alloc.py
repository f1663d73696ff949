"""sg_dot_noalloc: the dot product for callers that cannot allocate device memory.

Who needs it: plug-ins inside an application that owns all device memory
through its own pool and forbids raw cudaMalloc, and real-time loops that
cannot pay cudaMalloc's latency or cudaFree's device-wide synchronisation.
sg_dot takes its reduction scratch from a context, which allocates;
sg_dot_noalloc keeps that scratch in a fixed array inside the library.

The test calls the entry point through the C ABI (ctypes) twice in a row,
on different sizes (the second call finds the first call's partial sums still
in the shared array), and checks each result against sg_dot -- the existing
entry point -- within the dot-product tolerance the other tests use
(1e-14 relative to sum |x_i y_i|: the two kernels add the same terms in
different block orders).  The device buffers come from torch; the entry point
itself allocates nothing, which the test checks through the device's free
memory around calls made after the first one (the first call on a device may
load the library's device code, which the driver allocates for).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_N = 33554432  # SG_DOT_NOALLOC_MAX_N


def test_dot_noalloc_matches_sg_dot_on_two_calls(sg):
    torch = pytest.importorskip("torch")
    from schwarz_gmres_dashboard_gb300 import _lib

    lib = _lib.load()
    for n, seed in ((1_000_003, 1), (262_147, 2)):
        x = sg.uniform(n, seed=seed)
        y = sg.uniform(n, seed=seed + 10)
        xd = torch.from_numpy(x).cuda()
        yd = torch.from_numpy(y).cuda()
        out = torch.full((1,), float("nan"), dtype=torch.float64, device="cuda")
        torch.cuda.synchronize()
        st = lib.sg_dot_noalloc(C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n,
                                C.c_void_p(out.data_ptr()), None)
        assert st == 0, lib.sg_last_error().decode()
        torch.cuda.synchronize()
        got = float(out.item())
        ref = sg.dot(xd, yd)  # the existing entry point (context scratch)
        assert abs(got - ref) <= 1e-14 * float(np.abs(x * y).sum()), (got, ref)


def test_dot_noalloc_allocates_nothing(sg):
    torch = pytest.importorskip("torch")
    from schwarz_gmres_dashboard_gb300 import _lib

    lib = _lib.load()
    n = 4_000_037
    xd = torch.from_numpy(sg.uniform(n, seed=7)).cuda()
    out = torch.zeros(3, dtype=torch.float64, device="cuda")
    args = (C.c_void_p(xd.data_ptr()), C.c_void_p(xd.data_ptr()), n)
    assert lib.sg_dot_noalloc(*args, C.c_void_p(out.data_ptr()), None) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    alloc0 = torch.cuda.memory_allocated()
    for i in (1, 2):
        st = lib.sg_dot_noalloc(*args, C.c_void_p(out.data_ptr() + 8 * i), None)
        assert st == 0, lib.sg_last_error().decode()
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_allocated() == alloc0
    v = out.cpu().numpy()
    assert v[0] == v[1] == v[2]  # same inputs, same order: same bits


def test_dot_noalloc_rejects_sizes_beyond_its_scratch(sg):
    torch = pytest.importorskip("torch")
    from schwarz_gmres_dashboard_gb300 import _lib

    lib = _lib.load()
    xd = torch.zeros(8, dtype=torch.float64, device="cuda")
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    st = lib.sg_dot_noalloc(C.c_void_p(xd.data_ptr()), C.c_void_p(xd.data_ptr()), MAX_N + 1,
                            C.c_void_p(out.data_ptr()), None)
    assert st == 1  # SG_ERR_INVALID_ARG, nothing launched
    assert b"exceeds" in lib.sg_last_error()


def test_dot_noalloc_inside_a_cuda_graph(sg):
    """The reason the entry point exists: a call captured into a CUDA graph
    (after a first call outside capture has looked up the scratch array) is
    replayed on new contents of x and gives the same sum as sg_dot."""
    torch = pytest.importorskip("torch")
    from schwarz_gmres_dashboard_gb300 import _lib

    lib = _lib.load()
    n = 1_000_003
    xd = torch.from_numpy(sg.uniform(n, seed=21)).cuda()
    yd = torch.from_numpy(sg.uniform(n, seed=22)).cuda()
    out = torch.zeros(1, dtype=torch.float64, device="cuda")
    args = (C.c_void_p(xd.data_ptr()), C.c_void_p(yd.data_ptr()), n, C.c_void_p(out.data_ptr()))
    assert lib.sg_dot_noalloc(*args, None) == 0  # first call, outside capture
    torch.cuda.synchronize()
    s = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g, stream=s):
        st = lib.sg_dot_noalloc(*args, C.c_void_p(s.cuda_stream))
    assert st == 0, lib.sg_last_error().decode()
    for scale in (2.0, -0.5):
        xd.mul_(scale)
        out.zero_()
        g.replay()
        torch.cuda.synchronize()
        ref = sg.dot(xd, yd)
        bound = 1e-14 * float((xd * yd).abs().sum().item())
        assert abs(float(out.item()) - ref) <= bound, (float(out.item()), ref)
