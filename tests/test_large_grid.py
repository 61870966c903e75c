"""The 1024x1024, 48-rotation workload (sigma_x, sigma_y ~ U(4, 24) px,
log-normal unaries): wide kernels and rows wider than one shared-memory row.

Parity is checked against the oracle at a reduced grid with the same kernel
widths, one full-size message against the FP32 oracle, and the full-size
PS through properties that do not depend on an oracle run: finite maps, the
argmax at the marginal's maximum, the root posterior as log-sum-exp over
rotations, local maxima that are local maxima, and bit-identical reruns."""
import math

import numpy as np
import pytest

from partapp_gb300 import synth

pytestmark = pytest.mark.gpu

LOG_ZERO = np.float32(-1e6)
R = 48


@pytest.fixture(scope="module")
def ctx():
    import torch

    from partapp_gb300 import build
    import partapp_gb300 as pa

    build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pa.Context(0)
    yield c
    c.close()


@pytest.fixture(scope="module")
def orc():
    import oracle

    oracle.build()
    return oracle


def _exp(**kw):
    import partapp_gb300 as pa

    return pa.exp_param(R=R, **kw)


def lognormal_unary(rng, P, H, W):
    """log of LogNormal(0, 1) scores: N(0, 1) log-unaries."""
    return rng.standard_normal((P, R, H, W), dtype=np.float32)


def large_tree(rng):
    return synth.make_tree(rng, R=R, offset_range=(10.0, 40.0), sigma_range=(4.0, 24.0))


def maxnorm_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(np.exp(a - a.max()) - np.exp(b - b.max())).max())


def test_reduced_grid_ps_matches_oracle(ctx, orc):
    rng = np.random.default_rng(1024)
    H, W = 96, 128
    tree = large_tree(rng)
    u = lognormal_unary(rng, 10, H, W)
    e = orc.make_exp(R=R)
    want = orc.ps_infer(e, tree, u)
    want64 = orc.ps_infer(e, tree, u.astype(np.float64), f64=True, want_hyps=False)
    got = ctx.compute_root_posterior_rot(_exp(), tree, u)
    for p in range(10):
        assert maxnorm_err(got["log_marg"][p], want["log_marg"][p]) <= 1e-4, p
        assert maxnorm_err(got["log_marg"][p], want64["log_marg"][p]) <= 1e-3, p


def test_full_size_message_matches_oracle(ctx, orc):
    """One 1024 x 1024 x 48 message with the widest x kernel (sigma 24 px):
    the row pass runs in column chunks."""
    rng = np.random.default_rng(4)
    H = W = 1024
    child = lognormal_unary(rng, 1, H, W)[0]
    step = synth.rot_step_rad(R)
    args = (np.array([23.5, -31.0]), np.array([-12.25, 17.0]), np.diag([24.0 ** 2, 5.0 ** 2]),
            2 * step, 2.0 * step)
    e = orc.make_exp(R=R)
    want = orc.rot_joint_marginal(e, child, *args)
    got = ctx.rot_joint_marginal(_exp(), child, *args)
    oob = want == LOG_ZERO
    assert np.array_equal(got[oob], want[oob])
    assert maxnorm_err(got, want) <= 1e-5


def test_full_size_ps_properties(ctx):
    import torch

    rng = np.random.default_rng(48)
    H = W = 1024
    tree = large_tree(rng)
    u = torch.from_numpy(lognormal_unary(rng, 10, H, W)).cuda()
    e = _exp(local_max=200)
    a = ctx.compute_root_posterior_rot(e, tree, u)
    b = ctx.compute_root_posterior_rot(e, tree, u)
    assert torch.equal(a["log_marg"], b["log_marg"])  # no order-dependent accumulation
    marg = a["log_marg"]
    assert bool(torch.isfinite(marg).all())
    for p in range(10):
        m = marg[p]
        best = a["best_conf"][p]
        r, x, y = int(best[2]), int(best[4]), int(best[5])
        assert float(m[r, y, x]) == float(m.max()) == float(best[6])
        # local maxima: no 8-neighbour strictly greater, adjacent rotations strictly smaller
        hyps = a["part_hyps"][p][: a["n_part_hyps"][p]]
        assert len(hyps) == 200
        mc = m.cpu().numpy()
        for h in hyps[:50]:
            r, x, y, v = int(h[2]), int(h[4]), int(h[5]), h[6]
            assert mc[r, y, x] == v
            win = mc[r, max(0, y - 1):y + 2, max(0, x - 1):x + 2]
            assert win.max() == v
            if r > 0:
                assert mc[r - 1, y, x] < v
            if r < R - 1:
                assert mc[r + 1, y, x] < v
        assert math.isfinite(a["log_z"][p])
    # root posterior = log sum over the kept (all) rotations of the root marginal
    root = 9
    mr = marg[root].double().cpu().numpy()
    rp = a["root_post"].cpu().numpy()
    for (y, x) in ((0, 0), (511, 600), (1023, 1023), (300, 17)):
        col = mr[:, y, x]
        want = col.max() + math.log(np.exp(col - col.max()).sum())
        assert abs(rp[y, x] - want) <= 1e-4 * max(1.0, abs(want))


def test_bf16_tensor_path_error_vs_fp64(ctx, orc):
    """The BF16 banded-Toeplitz spatial filter (tcgen05, FP32 accumulation):
    per-part error of the marginals against the FP64 oracle, next to the
    FP32 shared-memory path's.  Message arithmetic in BF16 carries about
    2^-9 relative rounding per operand, so its bound is looser than the FP32
    path's 1e-3; the argmax must still land on the FP64 maximum or on a cell
    within the same error of it."""
    import partapp_gb300 as pa

    rng = np.random.default_rng(4096)
    H, W = 128, 160
    tree = large_tree(rng)
    u = lognormal_unary(rng, 10, H, W)
    e = orc.make_exp(R=R)
    want64 = orc.ps_infer(e, tree, u.astype(np.float64), f64=True, want_hyps=False)
    fp32 = ctx.compute_root_posterior_rot(_exp(), tree, u)
    ctx.set_message_math(pa.PA_MSG_BF16_TENSOR)
    try:
        bf16 = ctx.compute_root_posterior_rot(_exp(), tree, u)
    finally:
        ctx.set_message_math(pa.PA_MSG_FP32)
    errs = []
    for p in range(10):
        e32 = maxnorm_err(fp32["log_marg"][p], want64["log_marg"][p])
        e16 = maxnorm_err(bf16["log_marg"][p], want64["log_marg"][p])
        errs.append((p, e32, e16))
        assert e32 <= 1e-3
        assert e16 <= 5e-3, (p, e16)
        m = want64["log_marg"][p].reshape(-1)
        b = bf16["best_conf"][p]
        flat = (int(b[2]) * H + int(b[5])) * W + int(b[4])
        assert m.max() - m[flat] <= 5e-3, p
    print("per-part max-normalised error vs FP64 (part, fp32, bf16):", errs)
