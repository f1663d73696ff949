"""The learned-stage oracle (oracle/learned_oracle.py) pinned on the CPU.

The stage has no reference counterpart, so the oracle's own mathematics is
checked here: its exact-FP64 forward pass and parameter gradient against
torch autograd (conv3d with zero padding, ReLU, mean squared error), its BF16
rounding against torch's bfloat16 conversion, and the grid transfers against
their definitions.  The GPU kernels are then compared with this oracle in
test_learned_gpu.py.
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle import learned_oracle as lo

torch = pytest.importorskip("torch")


def _random_params(seed, scale=0.3):
    rng = np.random.default_rng(seed)
    p = rng.uniform(-scale, scale, lo.NUM_PARAMS)
    p[: lo.NET_PARAMS] *= lo.param_mask()
    p[lo.NET_PARAMS] = 1.7
    return p


def _torch_net(params):
    layers, _c = lo.unpack(params)
    convs = []
    for l, (W, b) in enumerate(layers):
        cin = 2 if l == 0 else 16
        cout = 1 if l == lo.LAYERS - 1 else 16
        conv = torch.nn.Conv3d(cin, cout, 3, padding=1).double()
        # torch weight [co][ci][kz][ky][kx] = W[tap][ci][co], tap = kz*9 + ky*3 + kx
        w = np.transpose(W.reshape(3, 3, 3, 16, 16), (4, 3, 0, 1, 2))[:cout, :cin]
        conv.weight.data = torch.tensor(np.ascontiguousarray(w))
        conv.bias.data = torch.tensor(b[:cout].copy())
        convs.append(conv)
    return convs


def _torch_forward(convs, x2, D):
    B = x2.shape[0]
    x = torch.tensor(x2.reshape(B, D, D, D, 2).transpose(0, 4, 1, 2, 3).copy())
    for l, conv in enumerate(convs):
        x = conv(x)
        if l < len(convs) - 1:
            x = torch.relu(x)
    return x[:, 0].reshape(B, -1)


@pytest.mark.parametrize("D,B", [(8, 1), (8, 2)])
def test_forward_matches_torch(D, B):
    params = _random_params(1)
    rng = np.random.default_rng(2)
    x2 = rng.standard_normal((B, D ** 3, 2))
    y, _ = lo.forward(params, x2, D, emulate_bf16=False)
    yt = _torch_forward(_torch_net(params), x2, D).detach().numpy()
    assert np.max(np.abs(y - yt)) <= 1e-12 * max(1.0, np.max(np.abs(yt)))


@pytest.mark.parametrize("D,B", [(8, 1), (8, 3)])
def test_gradient_matches_torch_autograd(D, B):
    params = _random_params(3)
    rng = np.random.default_rng(4)
    x2 = rng.standard_normal((B, D ** 3, 2))
    t = rng.standard_normal((B, D ** 3))
    loss, g = lo.loss_and_grad(params, x2, t, D, emulate_bf16=False)
    convs = _torch_net(params)
    yt = _torch_forward(convs, x2, D)
    lt = ((yt - torch.tensor(t)) ** 2).mean()
    lt.backward()
    assert abs(loss - lt.item()) <= 1e-12 * abs(lt.item())
    layers_g = []
    for l, conv in enumerate(convs):
        cin = conv.weight.shape[1]
        cout = conv.weight.shape[0]
        gw = np.zeros((3, 3, 3, 16, 16))
        gw[..., :cin, :cout] = np.transpose(conv.weight.grad.numpy(), (2, 3, 4, 1, 0))
        gb = np.zeros(16)
        gb[:cout] = conv.bias.grad.numpy()
        layers_g.append(np.concatenate([gw.reshape(-1), gb]))
    ref = np.concatenate(layers_g)
    assert np.max(np.abs(g - ref)) <= 1e-11 * np.max(np.abs(ref))


def test_padded_parameters_get_no_gradient():
    params = _random_params(5)
    rng = np.random.default_rng(6)
    x2 = rng.standard_normal((1, 512, 2))
    _, g = lo.loss_and_grad(params, x2, rng.standard_normal((1, 512)), 8, emulate_bf16=True)
    assert np.all(g[lo.param_mask() == 0] == 0)


def test_bf16_rounding_matches_torch():
    rng = np.random.default_rng(7)
    x = np.concatenate([rng.standard_normal(20000) * 10.0 ** rng.integers(-8, 8, 20000),
                        [0.0, -0.0, 1.0, -1.0, 1.00390625, 1.01171875, 3.0e38]])
    ref = torch.tensor(x, dtype=torch.float32).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(lo.bf16(x), ref)


def test_grid_transfers():
    nx = 16
    # restriction of a constant, prolongation of a constant
    assert np.allclose(lo.restrict(np.full(nx ** 3, 2.5), nx), 2.5)
    assert np.allclose(lo.prolong(np.full((nx // 2) ** 3, -1.25), nx), -1.25)
    # prolongation reproduces linear functions away from the boundary
    c = np.arange(nx // 2, dtype=float)
    Y = np.broadcast_to(c[None, None, :], (nx // 2,) * 3).reshape(-1)
    f = lo.prolong(Y, nx).reshape(nx, nx, nx)
    xf = (np.arange(nx) + 0.5) / 2 - 0.5  # fine centres in coarse coordinates
    assert np.allclose(f[3, 5, 1:-1], xf[1:-1])
    # R P is a smoothing of the coarse field with row sums 1
    rp = lo.restrict(lo.prolong(np.eye((nx // 2) ** 3)[7], nx), nx)
    assert abs(rp.sum() - 1.0) < 1e-12


def test_stage_is_positively_homogeneous():
    # z(alpha v) = alpha z(v) for alpha > 0 with the s-normalisation
    nx = 16
    rng = np.random.default_rng(8)
    n = nx ** 3
    params = _random_params(9, 0.2)
    diag = np.exp(rng.standard_normal(n))

    def spmv(x):
        return diag * x

    def apply_m(x):
        return 0.5 * x / diag

    v = rng.standard_normal(n)
    z1, _ = lo.stage_apply(params, spmv, apply_m, diag, v, nx)
    z2, _ = lo.stage_apply(params, spmv, apply_m, diag, 3.0 * v, nx)
    assert np.allclose(z2, 3.0 * z1, rtol=1e-6, atol=1e-12)


def _spd_laplacian(nx, seed):
    """7-point -div(k grad u) with random positive face coefficients (scipy CSR)."""
    import scipy.sparse as sp
    rng = np.random.default_rng(seed)
    n = nx ** 3
    idx = np.arange(n).reshape(nx, nx, nx)
    rows, cols, vals = [], [], []
    diag = np.zeros(n)
    for axis in range(3):
        a = np.moveaxis(idx, axis, 0)
        i0, i1 = a[:-1].reshape(-1), a[1:].reshape(-1)
        k = np.exp(rng.standard_normal(i0.size))
        rows += [i0, i1]
        cols += [i1, i0]
        vals += [-k, -k]
        np.add.at(diag, i0, k)
        np.add.at(diag, i1, k)
    diag += 1.0  # Dirichlet boundary contributions
    rows.append(np.arange(n))
    cols.append(np.arange(n))
    vals.append(diag)
    return sp.csr_matrix((np.concatenate(vals), (np.concatenate(rows), np.concatenate(cols))),
                         shape=(n, n))


def test_prolong_adjoint_and_torch_interpolate():
    nx = 16
    rng = np.random.default_rng(10)
    c = rng.standard_normal((nx // 2) ** 3)
    w = rng.standard_normal(nx ** 3)
    assert abs(lo.prolong(c, nx) @ w - c @ lo.prolong_t(w, nx)) <= 1e-12 * np.abs(w).sum()
    t = torch.nn.functional.interpolate(torch.tensor(c).reshape(1, 1, 8, 8, 8), scale_factor=2,
                                        mode="trilinear", align_corners=False)
    assert np.allclose(t.numpy().reshape(-1), lo.prolong(c, nx), atol=1e-14)


def test_energy_gradient_matches_torch_autograd():
    nx, D, B = 16, 8, 2
    params = _random_params(11, 0.2)
    rng = np.random.default_rng(12)
    x2 = rng.standard_normal((B, D ** 3, 2))
    mats = [_spd_laplacian(nx, 20 + b) for b in range(B)]
    err = rng.standard_normal((B, nx ** 3))
    energy = np.array([err[b] @ (mats[b] @ err[b]) for b in range(B)])
    loss, g = lo.energy_loss_and_grad(params, x2, err, energy, [m.__matmul__ for m in mats], nx,
                                      emulate_bf16=False)
    convs = _torch_net(params)
    y = _torch_forward(convs, x2, D)
    c = params[lo.NET_PARAMS]
    lt = 0.0
    for b in range(B):
        up = torch.nn.functional.interpolate(y[b].reshape(1, 1, D, D, D), scale_factor=2,
                                             mode="trilinear", align_corners=False).reshape(-1)
        u = torch.tensor(err[b]) - c * up
        coo = mats[b].tocoo()
        At = torch.sparse_coo_tensor(np.vstack([coo.row, coo.col]), coo.data, coo.shape)
        lt = lt + (u @ torch.sparse.mm(At, u[:, None])[:, 0]) / (energy[b] * B)
    lt.backward()
    assert abs(loss - lt.item()) <= 1e-12 * abs(lt.item())
    ref = []
    for l, conv in enumerate(convs):
        cin, cout = conv.weight.shape[1], conv.weight.shape[0]
        gw = np.zeros((3, 3, 3, 16, 16))
        gw[..., :cin, :cout] = np.transpose(conv.weight.grad.numpy(), (2, 3, 4, 1, 0))
        gb = np.zeros(16)
        gb[:cout] = conv.bias.grad.numpy()
        ref.append(np.concatenate([gw.reshape(-1), gb]))
    ref = np.concatenate(ref)
    assert np.max(np.abs(g - ref)) <= 1e-10 * np.max(np.abs(ref))
