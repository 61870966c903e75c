"""numpy restatement of the learned unary (pa_unary_net).

TEST INFRASTRUCTURE ONLY.  The product never imports this module; it is used
by ``tests/`` as the checker of the GPU network and by ``bench.py`` for the
CPU baseline of the learned-unary workload.

The network has no counterpart in the reference: it maps a descriptor field
to part log scores and is trained on the log of the AdaBoost score grids
(``computeScoreGrid`` normalised, ``clip_scores_fill`` + ``computeLogGrid``:
libPartDetect/partdetect_test.cpp:344-405, libPictStruct/objectdetect_aux.hpp:42-60).

Layers (zero padding, bias): 1x1 dim -> 64, ReLU; three 3x3 64 -> 64, ReLU;
3x3 64 -> P.  Parameters flat, in order W0 [64][dim], b0, W1..W3
[64][9][64], b1..b3, W4 [P][9][64], b4; taps (dy, dx) row-major.

``mode="gpu"`` rounds where the GPU rounds: the field, the weights, every
hidden activation and every back-propagated gradient to bf16
(round-to-nearest-even); sums run in float64 and round to float32 where
the GPU's tensor-core accumulators end.  ``mode="exact"`` runs everything in
float64 with no rounding; its gradient is the analytic gradient of the
loss, checked against central differences in the tests.
"""
from __future__ import annotations

import numpy as np

HIDDEN = 64
LOG_CLIP = np.log(np.float32(1e-4), dtype=np.float32)


def bf16(x) -> np.ndarray:
    """float32 -> nearest bf16 (ties to even), returned as float32."""
    a = np.ascontiguousarray(x, dtype=np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    u = (u + 0x7FFF + ((u >> 16) & 1)) & 0xFFFF0000
    return u.astype(np.uint32).view(np.float32).reshape(a.shape)


def layout(dim: int, P: int):
    """[(w_offset, w_shape, b_offset, cout)] for the five layers, and n_params."""
    out, o = [], 0
    for l in range(5):
        cout = P if l == 4 else HIDDEN
        shape = (cout, dim) if l == 0 else (cout, 9, HIDDEN)
        n = int(np.prod(shape))
        out.append((o, shape, o + n, cout))
        o += n + cout
    return out, o


def unpack(params, dim: int, P: int):
    lay, n = layout(dim, P)
    p = np.asarray(params)
    assert p.size == n
    return [(p[wo:wo + int(np.prod(sh))].reshape(sh), p[bo:bo + co]) for wo, sh, bo, co in lay]


def _shift(x, dy, dx):
    """out[f, y, x] = x[f, y + dy, x + dx], zero outside."""
    n, H, W, C = x.shape
    out = np.zeros_like(x)
    ys, ye = max(0, -dy), min(H, H - dy)
    xs, xe = max(0, -dx), min(W, W - dx)
    if ys < ye and xs < xe:
        out[:, ys:ye, xs:xe] = x[:, ys + dy:ye + dy, xs + dx:xe + dx]
    return out


TAPS = [(dy, dx) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]


def _conv(x, w):
    """x [n][H][W][cin] (float64), w [cout][taps][cin] or [cout][cin]."""
    if w.ndim == 2:
        return x @ w.T
    acc = 0.0
    for t, (dy, dx) in enumerate(TAPS):
        acc = acc + _shift(x, dy, dx) @ w[:, t, :].T
    return acc


def _conv_input_grad(dz, w):
    """d/dx of sum(dz * conv(x, w)): sum over taps of shift(dz, -t) @ w[:, t]."""
    acc = 0.0
    for t, (dy, dx) in enumerate(TAPS):
        acc = acc + _shift(dz, -dy, -dx) @ w[:, t, :]
    return acc


def _conv_weight_grad(x, dz, taps):
    """dW[co][t][ci] = sum over positions of dz[pos][co] * x[pos + t][ci]."""
    n, H, W, cin = x.shape
    d2 = dz.reshape(-1, dz.shape[-1])
    if taps == 1:
        return d2.T @ x.reshape(-1, cin)
    return np.stack([d2.T @ _shift(x, dy, dx).reshape(-1, cin) for dy, dx in TAPS], axis=1)


def forward(params, fields, P: int, mode: str = "gpu"):
    """Returns (y [P][n][ny][nx] float32 or float64, inputs of layers 0..4)."""
    x = np.asarray(fields)
    dim = x.shape[-1]
    layers = unpack(params, dim, P)
    g = mode == "gpu"
    rnd = bf16 if g else (lambda a: a)
    h = rnd(x.astype(np.float32) if g else x.astype(np.float64)).astype(np.float64)
    ins = [h]
    for l, (w, b) in enumerate(layers):
        wq = rnd(w.astype(np.float32) if g else w).astype(np.float64)
        z = _conv(h, wq)
        if g:
            z = z.astype(np.float32) + b.astype(np.float32)
        else:
            z = z + b.astype(np.float64)
        if l == 4:
            y = np.moveaxis(z, -1, 0)
            return (y.astype(np.float32) if g else y), ins
        h = rnd(np.maximum(z, 0)).astype(np.float64)
        ins.append(h)
    raise AssertionError


def targets(scores):
    """Log-score targets and the mask of the cells in the loss."""
    s = np.asarray(scores, dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        t = np.where(s < 0, LOG_CLIP, np.log(np.where(s > 0, s, 1), dtype=np.float32))
    return t.astype(np.float32), s != 0


def backward(params, fields, scores, P: int, mode: str = "gpu"):
    """(loss, gradient flat like params).  loss = sum of squared errors over
    the cells in the mask / (n * P * ny * nx)."""
    x = np.asarray(fields)
    dim = x.shape[-1]
    layers = unpack(params, dim, P)
    g = mode == "gpu"
    rnd = bf16 if g else (lambda a: a)
    y, ins = forward(params, fields, P, mode)
    t, m = targets(scores)
    count = y.size
    if g:
        d = (y - t).astype(np.float32)
        loss = float(np.sum(np.where(m, d.astype(np.float64) ** 2, 0.0))) / count
        gy = np.where(m, np.float32(2) * d * np.float32(1.0 / count), np.float32(0))
    else:
        d = y - t.astype(np.float64)
        loss = float(np.sum(np.where(m, d * d, 0.0))) / count
        gy = np.where(m, 2.0 * d / count, 0.0)
    dz = np.zeros(ins[4].shape[:-1] + (HIDDEN,), dtype=np.float64)
    dz[..., :P] = rnd(np.moveaxis(gy, 0, -1).astype(np.float32) if g else np.moveaxis(gy, 0, -1))
    grads = []
    for l in range(4, -1, -1):
        w, b = layers[l]
        cout = w.shape[0]
        dzl = dz[..., :cout]
        dw = _conv_weight_grad(ins[l], dzl, 1 if l == 0 else 9)
        db = dzl.reshape(-1, cout).sum(axis=0)
        grads.append((dw, db))
        if l == 0:
            break
        wq = rnd(w.astype(np.float32) if g else w).astype(np.float64)
        din = _conv_input_grad(dzl, wq)
        if g:
            din = din.astype(np.float32)
        dz = rnd(np.where(ins[l] > 0, din, 0)).astype(np.float64)
    grads.reverse()
    flat = np.concatenate([np.concatenate([dw.reshape(-1), db]) for dw, db in grads])
    return loss, (flat.astype(np.float32) if g else flat)


def adam(params, grads, m, v, step: int, lr, b1=0.9, b2=0.999, eps=1e-8):
    """One Adam step in float32 as the GPU runs it; returns (params, m, v)."""
    f = np.float32
    g = np.asarray(grads, dtype=f)
    m = f(b1) * m + (f(1) - f(b1)) * g
    v = f(b2) * v + (f(1) - f(b2)) * g * g
    bc1, bc2 = f(1.0 - b1 ** step), f(1.0 - b2 ** step)
    p = params - f(lr) * (m / bc1) / (np.sqrt(v / bc2) + f(eps))
    return p.astype(f), m.astype(f), v.astype(f)
