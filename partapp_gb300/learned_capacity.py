"""Capacity study of the learned unary: how close can a network get to the
AdaBoost log-score maps it stands in for, measured against the 1e-2
maximum-error rule that keeps a part on the net.

The AdaBoost score of a location depends on that location's descriptor
alone: s = sum_i (v[f_i] < t_i ? a_i : -a_i) / sum(alpha), a sum of single-
coordinate steps, then the reference's clip (s < 0 -> 1e-4) and log.  One
step moves s by 2 alpha_i / sum(alpha) (~0.004 here), i.e. ~0.08 in log units
at typical scores, so a stand-in meets |error| <= 1e-2 on a cell only if it
decides every one of the cell's 500 tests exactly.

Two measurements, both against the stump kernel's exact scores:

  construction: one ReLU ramp per stump, h_i = clamp((v[f_i] - t_i) / delta
      + 1/2, 0, 1), vote a_i (2 h_i - 1) -- the network a 960 -> 2*500 -> 1
      ReLU layer per part can represent exactly as delta -> 0 -- evaluated
      with the ramp's affine map in FP32 or BF16 (the learned net's operand
      type), for several delta;
  trained: per-location networks 960 -> H -> H -> P (ReLU), FP32, Adam on
      the squared log-score error, for several widths H.

Each reports per part the maximum |log error| over the evaluation cells,
its 99.9th percentile, the fraction of cells above 1e-2 and the mean.

  python -m partapp_gb300.learned_capacity   (one GPU, about a minute)
"""
from __future__ import annotations

import json
import time

import numpy as np

from . import learned, synth


def _errors(y, t, m):
    """Per-part error statistics of predictions y against targets t (mask m)."""
    import torch

    d = torch.where(m, (y - t).abs(), torch.zeros_like(y))
    out = []
    for p in range(y.shape[0]):
        dp = d[p][m[p]].float()
        q = torch.quantile(dp[torch.randperm(dp.numel(), device=dp.device)[:1 << 20]], 0.999)
        out.append(dict(max=float(dp.max()), p999=float(q), frac_over=float((dp > 1e-2).float().mean()),
                        mean=float(dp.mean())))
    return out


def _summary(errs):
    return dict(max=[round(e["max"], 4) for e in errs], p999=[round(e["p999"], 4) for e in errs],
                frac_over_1e2=[round(e["frac_over"], 4) for e in errs],
                mean=[round(e["mean"], 4) for e in errs])


def construction(models, fields, scores, deltas=(1e-3, 1e-5, 1e-7)):
    """The ramp network evaluated in FP32 and BF16 affine arithmetic."""
    import torch

    P = len(models["f"])
    x = fields.reshape(-1, fields.shape[-1])
    t_all, m = learned.log_targets(scores.reshape(P, -1))
    res = {}
    for dt in (torch.float32, torch.bfloat16):
        for delta in deltas:
            ys = []
            for p in range(P):
                f = torch.as_tensor(models["f"][p], device=x.device, dtype=torch.long)
                th = torch.as_tensor(models["theta"][p], device=x.device)
                pol = torch.as_tensor(models["p"][p], device=x.device)
                al = torch.as_tensor(models["alpha"][p], device=x.device)
                w = (pol / delta).to(dt)           # ramp slope, sign = polarity
                b = (-pol * th / delta + 0.5).to(dt)
                v = x[:, f].to(dt)
                h = (v * w + b).float().clamp(0.0, 1.0)  # 1: the test v*p < theta*p fails
                vote = al * (1.0 - 2.0 * h)
                s = vote.sum(1) / al.sum()
                y, _ = learned.log_targets(s[None])
                ys.append(y[0])
            y = torch.stack(ys)
            res[f"{str(dt).split('.')[-1]}, delta {delta:g}"] = _summary(_errors(y, t_all, m))
    return res


def trained(ctx, cls, models, train_fields, eval_fields, eval_scores, widths=(64, 512, 4096),
            steps=1500, batch=8192, lr=1e-3):
    import torch

    P = len(models["f"])
    x_all = train_fields.reshape(-1, train_fields.shape[-1])
    sc = ctx.score_grids(cls, train_fields).reshape(P, -1)
    t_all, m_all = learned.log_targets(sc)
    xe = eval_fields.reshape(-1, eval_fields.shape[-1])
    te, me = learned.log_targets(eval_scores.reshape(P, -1))
    g = torch.Generator(device=x_all.device)
    g.manual_seed(3)
    res = {}
    for H in widths:
        net = torch.nn.Sequential(torch.nn.Linear(x_all.shape[1], H), torch.nn.ReLU(),
                                  torch.nn.Linear(H, H), torch.nn.ReLU(),
                                  torch.nn.Linear(H, P)).to(x_all.device)
        with torch.no_grad():
            net[-1].bias.copy_((torch.where(m_all, t_all, 0).sum(1) / m_all.sum(1)).float())
        opt = torch.optim.Adam(net.parameters(), lr=lr)
        sched = torch.optim.lr_scheduler.CosineAnnealingLR(opt, steps, eta_min=lr / 10)
        t0 = time.time()
        for it in range(steps):
            idx = torch.randint(0, x_all.shape[0], (batch,), generator=g, device=x_all.device)
            y = net(x_all[idx]).T
            d = torch.where(m_all[:, idx], y - t_all[:, idx], 0)
            loss = (d * d).mean()
            opt.zero_grad(set_to_none=True)
            loss.backward()
            opt.step()
            sched.step()
        with torch.no_grad():
            ye = torch.cat([net(xe[i:i + 65536]).T for i in range(0, xe.shape[0], 65536)], 1)
        r = _summary(_errors(ye, te, me))
        r["train_s"] = round(time.time() - t0, 1)
        r["final_loss"] = float(loss.detach())
        res[f"H {H}"] = r
    return res


def main():
    import torch

    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    ctx = pa.Context(0)
    learned.bind_torch_stream(ctx)
    rng = np.random.default_rng(11)
    models = synth.make_models(rng, n_parts=10, n_stumps=500, D=960)
    cls = ctx.classifiers(models)
    train_fields = learned.synth_fields(256, 60, 80, 960, seed=101)   # 1.23 M locations
    eval_fields = learned.synth_fields(64, 60, 80, 960, seed=202)     # 0.31 M locations
    eval_scores = ctx.score_grids(cls, eval_fields)
    out = {"workload": "10 classifiers x 500 stumps, 960-d Gamma(0.5, 1) descriptors "
                       "L2-normalised; evaluation on 307 200 fresh locations",
           "construction": construction(models, eval_fields, eval_scores),
           "trained": trained(ctx, cls, models, train_fields, eval_fields, eval_scores)}
    print(json.dumps(out))
    ctx.close()
    del torch


if __name__ == "__main__":
    main()
