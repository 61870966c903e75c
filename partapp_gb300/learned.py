"""Training, evaluation and per-part fall-back of the learned unary.

The network (``partapp_gb300.UnaryNet``, pa_unary_net in the C-ABI) is fit by
mean squared error to the log score maps that the AdaBoost part detectors
produce on the same descriptor fields (pa_score_grids, then the reference's
clip_scores_fill + log: s < 0 -> log 1e-4, s == 0 left out).  Every step runs
on the GPU: the AdaBoost targets by the stump kernel, the forward and
backward passes by the tensor-core convolution kernels, the update by the
Adam kernel.  Synthetic descriptor fields are drawn on the device from a
seed: elements Gamma(0.5, 1) (= z^2 / 2, z standard normal), L2-normalised
per location, the distribution of the synthetic part-detection workloads.

Fall-back rule: a part stays on the net only if its maximum absolute
log-score error against AdaBoost over a calibration slice is at most
``bound`` (1e-2); otherwise its unary is the AdaBoost map.
"""
from __future__ import annotations

import time

import numpy as np

LOG_CLIP = float(np.log(np.float32(1e-4)))


def bind_torch_stream(ctx):
    """Makes the context issue its kernels on torch's current stream, so the
    fields and targets torch produces are complete before the net reads
    them (the context's own stream is not ordered with torch's)."""
    import torch

    ctx.set_stream(torch.cuda.current_stream().cuda_stream)


def synth_fields(n: int, ny: int, nx: int, dim: int, seed: int, device="cuda"):
    """[n][ny][nx][dim] float32 CUDA tensor of seeded synthetic descriptors."""
    import torch

    g = torch.Generator(device=device)
    g.manual_seed(int(seed) & (2**63 - 1))
    z = torch.randn((n, ny, nx, dim), generator=g, device=device, dtype=torch.float32)
    x = 0.5 * z * z
    x /= torch.linalg.vector_norm(x, dim=-1, keepdim=True)
    return x


def log_targets(scores):
    """The reference's clip + log of normalised AdaBoost scores, and the mask
    of the cells that enter the loss (torch, element-wise)."""
    import torch

    t = torch.where(scores < 0, torch.full_like(scores, LOG_CLIP),
                    torch.log(torch.where(scores > 0, scores, torch.ones_like(scores))))
    return t, scores != 0


def init_output_bias(ctx, net, cls_list, fields):
    """Sets the output biases to each part's mean log-score target on
    `fields` (data-dependent initialisation; resets the Adam state)."""
    import torch

    t, m = log_targets(ctx.score_grids(cls_list[:net.P], fields))
    mean = (torch.where(m, t, torch.zeros_like(t)).flatten(1).sum(1) /
            m.flatten(1).sum(1).clamp(min=1)).cpu().numpy()
    p = net.get_params()
    p[p.size - net.P:] = mean.astype(np.float32)
    net.set_params(p)


def train(ctx, net, cls_list, n_fields: int = 20000, batch: int = 32, ny: int = 60, nx: int = 80,
          lr: float = 1e-3, lr_final: float = 1e-4, epochs: int = 1, seed: int = 1,
          log_every: int = 0):
    """Trains `net` on n_fields seeded fields (field i of the training set is
    drawn from seed (seed, i // batch)); cosine decay from lr to lr_final.
    Returns the per-step losses."""
    import math

    bind_torch_stream(ctx)
    steps_per_epoch = max(1, n_fields // batch)
    total = steps_per_epoch * epochs
    init_output_bias(ctx, net, cls_list, synth_fields(batch, ny, nx, net.dim, seed * 1_000_003))
    losses = []
    t0 = time.time()
    for ep in range(epochs):
        for b in range(steps_per_epoch):
            it = ep * steps_per_epoch + b
            fields = synth_fields(batch, ny, nx, net.dim, seed * 1_000_003 + b)
            scores = ctx.score_grids(cls_list[:net.P], fields)
            cur = lr_final + 0.5 * (lr - lr_final) * (1 + math.cos(math.pi * it / max(1, total)))
            losses.append(net.train_step(fields, scores, lr=cur))
            if log_every and (it % log_every == 0 or it == total - 1):
                print(f"step {it}/{total} loss {losses[-1]:.4f} ({time.time() - t0:.1f} s)",
                      flush=True)
    return np.array(losses)


def evaluate(ctx, net, cls_list, n_fields: int = 2000, batch: int = 32, ny: int = 60,
             nx: int = 80, seed: int = 2):
    """Errors of the net against AdaBoost on fresh seeded fields, per part:
    max |log-score error|, mean squared error, and the mean squared error of
    the best constant (each part's mean target) for comparison."""
    import torch

    bind_torch_stream(ctx)
    P = net.P
    n_b = max(1, n_fields // batch)
    mx = torch.zeros(P, dtype=torch.float64, device="cuda")
    se = torch.zeros(P, dtype=torch.float64, device="cuda")
    s1 = torch.zeros(P, dtype=torch.float64, device="cuda")
    s2 = torch.zeros(P, dtype=torch.float64, device="cuda")
    cnt = torch.zeros(P, dtype=torch.float64, device="cuda")
    for b in range(n_b):
        fields = synth_fields(batch, ny, nx, net.dim, seed * 1_000_003 + b)
        scores = ctx.score_grids(cls_list[:P], fields)
        t, m = log_targets(scores)
        y = net.forward(fields)
        d = torch.where(m, (y - t).abs(), torch.zeros_like(y)).double()
        mx = torch.maximum(mx, d.flatten(1).amax(1))
        se += (d * d).flatten(1).sum(1)
        tm = torch.where(m, t, torch.zeros_like(t)).double()
        s1 += tm.flatten(1).sum(1)
        s2 += (tm * tm).flatten(1).sum(1)
        cnt += m.flatten(1).sum(1).double()
    mse = (se / cnt).cpu().numpy()
    var = (s2 / cnt - (s1 / cnt) ** 2).cpu().numpy()
    return dict(max_abs_err=mx.cpu().numpy(), mse=mse, const_mse=var,
                gain=1.0 - mse / np.maximum(var, 1e-30), n_fields=n_b * batch)


def calibrate(max_abs_err, bound: float = 1e-2) -> np.ndarray:
    """Per-part flags: 1 = the net's unary, 0 = the AdaBoost fall-back."""
    return (np.asarray(max_abs_err) <= bound).astype(np.int32)
