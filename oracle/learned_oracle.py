"""CPU restatement of the learned coarse-correction stage -- TEST INFRASTRUCTURE ONLY.

The stage has no counterpart in the reference (it plugs into the reference's
flexible GMRES, src/core/fgmres.cpp:164-172, as a preconditioner), so this
oracle restates the stage's own definition in numpy:

    z1 = M v;  r1 = v - A z1;  rc = R r1;  s = rms(rc)
    z  = z1 + s * c * P(net([rc / s, f]))

and its two training losses: the energy norm ||e1/s - c P y||_A^2 /
||e1/s||_A^2 with e1 = e - M r the error left after M, and the coarse mean
squared error against R e1 / (s c).

R: mean of the 2x2x2 children; P: cell-centred trilinear prolongation with
the neighbour index clamped at the boundary; f: standardised restricted
log A_ii; net: four 3x3x3 convolutions (16 channels, zero padding, ReLU after
the first three), parameters in the library's layout (per layer
W[27][c_in][c_out], tap = (dz+1)*9 + (dy+1)*3 + (dx+1), then 16 biases;
then the output scale c).

`emulate_bf16=True` rounds what the GPU kernels store in BF16 (inputs,
weights, activations, activation gradients) with round-to-nearest-even and
accumulates in FP64; `False` is the exact FP64 network (checked against torch
autograd in the tests).  Only the tests and ``__graft_entry__.smoke()`` use
this module; it is the checker, never the thing measured or shipped.
"""
from __future__ import annotations

import numpy as np

C = 16
TAPS = 27
LAYERS = 4
LAYER_W = TAPS * C * C
LAYER_P = LAYER_W + C
NET_PARAMS = LAYERS * LAYER_P
NUM_PARAMS = NET_PARAMS + 1


def bf16(x):
    """Round to the nearest BF16 value, ties to even (float64 result)."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).astype(np.float64)


def param_mask():
    """1 for the real parameters, 0 for the padded channels."""
    m = np.ones(NET_PARAMS)
    for l in range(LAYERS):
        base = l * LAYER_P
        W = m[base: base + LAYER_W].reshape(TAPS, C, C)
        if l == 0:
            W[:, 2:, :] = 0.0
        if l == LAYERS - 1:
            W[:, :, 1:] = 0.0
            m[base + LAYER_W + 1: base + LAYER_P] = 0.0
    return m


def unpack(params):
    """[(W[27][ci][co], b[16]) per layer], c"""
    p = np.asarray(params, dtype=np.float64)
    layers = []
    for l in range(LAYERS):
        base = l * LAYER_P
        layers.append((p[base: base + LAYER_W].reshape(TAPS, C, C),
                       p[base + LAYER_W: base + LAYER_P]))
    c = p[NET_PARAMS] if p.size > NET_PARAMS else 1.0
    return layers, c


def _offsets():
    for tap in range(TAPS):
        yield tap, tap // 9 - 1, (tap // 3) % 3 - 1, tap % 3 - 1


def conv3d(x, W, b=None):
    """x [B, D, D, D, C] (channel-last, zero padded): out[v][co] =
    sum_tap sum_ci x[v + off(tap)][ci] * W[tap][ci][co] + b[co]."""
    B, D = x.shape[0], x.shape[1]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros(x.shape[:4] + (W.shape[2],))
    for tap, dz, dy, dx in _offsets():
        sl = xp[:, 1 + dz: 1 + dz + D, 1 + dy: 1 + dy + D, 1 + dx: 1 + dx + D, :]
        out += sl @ W[tap]
    if b is not None:
        out += b
    return out


def conv3d_input_grad(g, W):
    """dx[v][ci] = sum_tap sum_co g[v - off(tap)][co] * W[tap][ci][co]."""
    D = g.shape[1]
    gp = np.pad(g, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    out = np.zeros(g.shape[:4] + (W.shape[1],))
    for tap, dz, dy, dx in _offsets():
        sl = gp[:, 1 - dz: 1 - dz + D, 1 - dy: 1 - dy + D, 1 - dx: 1 - dx + D, :]
        out += sl @ W[tap].T
    return out


def conv3d_weight_grad(x, g):
    """dW[tap][ci][co] = sum_v x[v + off(tap)][ci] * g[v][co]; db = sum_v g."""
    D = x.shape[1]
    xp = np.pad(x, ((0, 0), (1, 1), (1, 1), (1, 1), (0, 0)))
    dW = np.zeros((TAPS, x.shape[4], g.shape[4]))
    g2 = g.reshape(-1, g.shape[4])
    for tap, dz, dy, dx in _offsets():
        sl = xp[:, 1 + dz: 1 + dz + D, 1 + dy: 1 + dy + D, 1 + dx: 1 + dx + D, :]
        dW[tap] = sl.reshape(-1, x.shape[4]).T @ g2
    return dW, g2.sum(axis=0)


def pack_input(x2, D):
    """[B, nc, 2] -> [B, D, D, D, 16] with channels 2..15 zero."""
    x2 = np.asarray(x2, dtype=np.float64)
    B = x2.shape[0]
    X = np.zeros((B, D, D, D, C))
    X[..., :2] = x2.reshape(B, D, D, D, 2)
    return X


def forward(params, x2, D, emulate_bf16=True):
    """Network output y [B, nc] and the activations [X0, A1, A2, A3]."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    layers, _c = unpack(params)
    A = rnd(pack_input(x2, D))
    acts = [A]
    for l in range(LAYERS - 1):
        W, b = layers[l]
        A = rnd(np.maximum(conv3d(A, rnd(W), b), 0.0))
        acts.append(A)
    W, b = layers[LAYERS - 1]
    y = conv3d(A, rnd(W))[..., 0] + b[0]
    return y.reshape(y.shape[0], -1), acts


def loss_and_grad(params, x2, t, D, emulate_bf16=True):
    """mean (y - t)^2 and its gradient (NET_PARAMS, library layout, padded 0)."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    y, acts = forward(params, x2, D, emulate_bf16)
    t = np.asarray(t, dtype=np.float64).reshape(y.shape)
    count = y.size
    loss = float(((y - t) ** 2).sum() / count)
    B = y.shape[0]
    G = np.zeros((B, D, D, D, C))
    G[..., 0] = rnd((2.0 * (y - t) / count)).reshape(B, D, D, D)
    return loss, backward(params, acts, G, emulate_bf16)


def energy_loss_and_grad(params, x2, err, energy, spmvs, nx, emulate_bf16=True):
    """Energy-norm loss mean_b ||err_b - c P y_b||_A^2 / energy_b and its
    gradient; spmvs[b](u) = A_b u, energy_b = err_b^T A_b err_b."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    D = nx // 2
    y, acts = forward(params, x2, D, emulate_bf16)
    _layers, c = unpack(params)
    B = y.shape[0]
    loss = 0.0
    G = np.zeros((B, D, D, D, C))
    for b in range(B):
        u = np.asarray(err[b], dtype=np.float64) - c * prolong(y[b], nx)
        w = spmvs[b](u)
        loss += float(u @ w) / (energy[b] * B)
        G[b, ..., 0] = rnd(-2.0 * c * prolong_t(w, nx) / (energy[b] * B)).reshape(D, D, D)
    return loss, backward(params, acts, G, emulate_bf16)


def backward(params, acts, G, emulate_bf16=True):
    """Parameter gradient from the output gradient G [B, D, D, D, 16] (channel 0)."""
    rnd = bf16 if emulate_bf16 else (lambda a: np.asarray(a, dtype=np.float64))
    layers, _c = unpack(params)
    grads = [None] * LAYERS
    for l in range(LAYERS - 1, -1, -1):
        dW, db = conv3d_weight_grad(acts[l], G)
        grads[l] = (dW, db)
        if l > 0:
            W, _b = layers[l]
            G = rnd(conv3d_input_grad(G, rnd(W)) * (acts[l] > 0))
    flat = np.zeros(NET_PARAMS)
    for l, (dW, db) in enumerate(grads):
        flat[l * LAYER_P: l * LAYER_P + LAYER_W] = dW.reshape(-1)
        flat[l * LAYER_P + LAYER_W: (l + 1) * LAYER_P] = db
    return flat * param_mask()


# ------------------------------------------------------------------ grid transfer
def restrict(v, nx, ny=None, nz=None):
    """Mean of the 2x2x2 children (index f = (z*ny + y)*nx + x)."""
    ny, nz = ny or nx, nz or nx
    a = np.asarray(v, dtype=np.float64).reshape(nz // 2, 2, ny // 2, 2, nx // 2, 2)
    return a.mean(axis=(1, 3, 5)).reshape(-1)


def _interp_1d(n):
    nc = n // 2
    P = np.zeros((n, nc))
    for f in range(n):
        c = f // 2
        o = c + 1 if f % 2 else c - 1
        o = min(max(o, 0), nc - 1)
        P[f, c] += 0.75
        P[f, o] += 0.25
    return P


def prolong(c, nx, ny=None, nz=None):
    """Cell-centred trilinear prolongation (weights 3/4, 1/4 per axis)."""
    ny, nz = ny or nx, nz or nx
    Y = np.asarray(c, dtype=np.float64).reshape(nz // 2, ny // 2, nx // 2)
    out = np.einsum("ai,bj,ck,ijk->abc", _interp_1d(nz), _interp_1d(ny), _interp_1d(nx), Y)
    return out.reshape(-1)


def prolong_t(w, nx, ny=None, nz=None):
    """Adjoint (transpose) of `prolong`."""
    ny, nz = ny or nx, nz or nx
    W = np.asarray(w, dtype=np.float64).reshape(nz, ny, nx)
    out = np.einsum("ai,bj,ck,abc->ijk", _interp_1d(nz), _interp_1d(ny), _interp_1d(nx), W)
    return out.reshape(-1)


def feature(diag, nx):
    """Standardised restricted log A_ii."""
    c = restrict(np.log(np.asarray(diag, dtype=np.float64)), nx)
    sd = c.std()
    return (c - c.mean()) / sd if sd > 1e-12 else np.zeros_like(c)


def stage_apply(params, spmv, apply_m, diag, v, nx):
    """z = M v + s c P(net([R r1 / s, f])) with r1 = v - A M v; returns (z, z1)."""
    D = nx // 2
    z1 = apply_m(v)
    r1 = v - spmv(z1)
    rc = restrict(r1, nx)
    s = float(np.sqrt(np.mean(rc ** 2)))
    inv = 1.0 / s if s > 0 else 0.0
    x2 = np.stack([rc * inv, feature(diag, nx)], axis=-1)[None]
    y, _acts = forward(params, x2.astype(np.float32), D, emulate_bf16=True)
    _layers, c = unpack(params)
    return z1 + s * c * prolong(y[0], nx), z1


def training_pair(spmv, apply_m, diag, r, e, nx):
    """(input R r1 / s, feature f, coarse target R(e1) / s, fine target e1 / s,
    energy (e1/s)^T A (e1/s)) of a pair (r, e), e1 = e - M r."""
    z1 = apply_m(r)
    rc = restrict(r - spmv(z1), nx)
    e1 = e - z1
    ec = restrict(e1, nx)
    s = float(np.sqrt(np.mean(rc ** 2)))
    inv = 1.0 / s if s > 0 else 0.0
    fine = e1 * inv
    return rc * inv, feature(diag, nx), ec * inv, fine, float(fine @ spmv(fine))
