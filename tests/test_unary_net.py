"""The learned unary (pa_unary_net): the numpy oracle, then the GPU network
through the C-ABI against it.

Tolerances (the GPU accumulates BF16 products in FP32 on the tensor cores in
its own order; the oracle sums in float64 and rounds where the GPU rounds):
  * forward log scores: |gpu - oracle| <= 2e-3 * (1 + max |oracle|) per cell
    (a rounding difference can move one BF16 activation by 2^-8 relative);
  * loss: relative 1e-4; gradients per layer: relative L2 error <= 5e-3;
  * Adam: the oracle's FP32 update of the GPU's own gradient, relative 1e-5;
  * the oracle itself: float64 analytic gradient = central differences to
    relative 1e-6.
"""
import numpy as np
import pytest

from oracle import unary_net as orn
from partapp_gb300 import synth


def _rand_params(rng, dim, P, scale=1.0):
    lay, n = orn.layout(dim, P)
    p = np.zeros(n, dtype=np.float64)
    for wo, sh, bo, co in lay:
        fan = sh[-1] * (9 if len(sh) == 3 else 1)
        p[wo:wo + int(np.prod(sh))] = rng.standard_normal(int(np.prod(sh))) * scale * np.sqrt(2.0 / fan)
        p[bo:bo + co] = rng.uniform(-0.1, 0.1, co)
    return p


def _rand_scores(rng, shape):
    s = rng.uniform(-1, 1, shape).astype(np.float32)
    s[rng.random(shape) < 0.05] = 0.0  # LOG_ZERO cells, left out of the loss
    return s


# ----------------------------------------------------------------- oracle
def test_oracle_gradient_matches_central_differences():
    rng = np.random.default_rng(3)
    dim, P, n, H, W = 64, 3, 2, 4, 5
    params = _rand_params(rng, dim, P)
    x = synth.make_descriptors(rng, n, H, W, dim).astype(np.float64)
    s = _rand_scores(rng, (P, n, H, W))
    loss, g = orn.backward(params, x, s, P, mode="exact")
    idx = rng.choice(params.size, 60, replace=False)
    lay, _ = orn.layout(dim, P)
    idx = np.concatenate([idx, [lay[4][2], lay[0][2] + 5, lay[2][0] + 100]])  # biases, a hidden weight
    for i in idx:
        h = 1e-6 * max(1.0, abs(params[i]))
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd = (orn.backward(pp, x, s, P, mode="exact")[0] - orn.backward(pm, x, s, P, mode="exact")[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(g[i])) + 1e-9, (i, fd, g[i])


def test_oracle_rounded_mode_tracks_exact():
    rng = np.random.default_rng(4)
    dim, P, n, H, W = 128, 4, 2, 5, 6
    params = _rand_params(rng, dim, P)
    x = synth.make_descriptors(rng, n, H, W, dim)
    s = _rand_scores(rng, (P, n, H, W))
    l64, g64 = orn.backward(params, x, s, P, mode="exact")
    l16, g16 = orn.backward(params, x, s, P, mode="gpu")
    assert abs(l16 - l64) <= 2e-2 * l64
    assert np.linalg.norm(g16 - g64) <= 5e-2 * np.linalg.norm(g64)


def test_bf16_rounding_is_nearest_even():
    v = np.array([1.0, 1.0 + 2 ** -8, 1.0 + 3 * 2 ** -9, 1.0 + 2 ** -9, -2.5, 0.0], np.float32)
    got = orn.bf16(v)
    assert got.tolist() == [1.0, 1.0, 1.0 + 2 ** -7, 1.0, -2.5, 0.0]


# ------------------------------------------------------------------- GPU
@pytest.fixture(scope="module")
def pa():
    from partapp_gb300 import build

    build.build()
    import partapp_gb300

    return partapp_gb300


@pytest.fixture(scope="module")
def ctx(pa):
    import torch

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pa.Context(0)
    # the inputs below are made by torch kernels: run on torch's stream
    c.set_stream(torch.cuda.current_stream().cuda_stream)
    yield c
    c.close()


def _layer_errs(g, want, dim, P):
    lay, _ = orn.layout(dim, P)
    out = []
    for wo, sh, bo, co in lay:
        for a, b in ((wo, wo + int(np.prod(sh))), (bo, bo + co)):
            out.append(np.linalg.norm(g[a:b] - want[a:b]) / max(np.linalg.norm(want[a:b]), 1e-30))
    return out


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,H,W", [(192, 3, 7, 150), (960, 2, 6, 80), (64, 1, 1, 1),
                                       (1344, 1, 3, 20)])
def test_forward_matches_oracle(ctx, pa, dim, n, H, W):
    """Shapes: two row tiles (W = 150), 960-d fields, a 1 x 1 field, 21 channel blocks."""
    import torch

    rng = np.random.default_rng(dim + W)
    P = 10
    net = pa.UnaryNet(ctx, dim=dim, n_parts=P, seed=5)
    params = _rand_params(rng, dim, P).astype(np.float32)
    net.set_params(params)
    assert np.array_equal(net.get_params(), params)
    x = synth.make_descriptors(rng, n, H, W, dim)
    want, _ = orn.forward(params, x, P, mode="gpu")
    xd = torch.from_numpy(x).cuda()
    got = net.forward(xd).cpu().numpy()
    tol = 2e-3 * (1.0 + np.abs(want).max())
    assert np.abs(got - want).max() <= tol
    # BF16 fields give the same bits as FP32 fields (the cast is RNE either way)
    got_b = net.forward(xd.to(torch.bfloat16)).cpu().numpy()
    assert np.array_equal(got_b, got)
    got_e = net.forward(xd, exp_out=True).cpu().numpy()
    assert np.allclose(got_e, np.exp(got.astype(np.float64)), rtol=2e-6, atol=0)
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("dim,n,H,W", [(128, 2, 6, 70), (960, 2, 5, 140)])
def test_backward_and_adam_match_oracle(ctx, pa, dim, n, H, W):
    import torch

    rng = np.random.default_rng(11 + dim)
    P = 10
    net = pa.UnaryNet(ctx, dim=dim, n_parts=P, seed=6)
    params = _rand_params(rng, dim, P).astype(np.float32)
    net.set_params(params)
    x = synth.make_descriptors(rng, n, H, W, dim)
    s = _rand_scores(rng, (P, n, H, W))
    loss, g = net.backward(torch.from_numpy(x).cuda(), torch.from_numpy(s).cuda(), want_grads=True)
    wl, wg = orn.backward(params, x, s, P, mode="gpu")
    assert abs(loss - wl) <= 1e-4 * wl
    errs = _layer_errs(g, wg, dim, P)
    assert max(errs) <= 5e-3, errs
    # one Adam step on the GPU's own gradient
    net.adam(lr=1e-3)
    m = np.zeros_like(params)
    want_p, _, _ = orn.adam(params, g, m, m.copy(), 1, 1e-3)
    got_p = net.get_params()
    assert np.allclose(got_p, want_p, rtol=1e-5, atol=1e-7)
    net.close()


@pytest.mark.gpu
def test_training_gains_over_the_constant_unary(ctx, pa):
    """Trained on AdaBoost log scores of seeded synthetic fields, the net
    explains part of their variance on fresh fields (gain = 1 - MSE / the
    MSE of each part's mean; about 0.15 on average after these 128 steps).  The targets are sums of 500 single-coordinate
    steps clipped at log 1e-4; the fall-back rule keeps every part whose
    maximum error exceeds 1e-2 on AdaBoost."""
    from partapp_gb300 import learned

    rng = np.random.default_rng(21)
    models = synth.make_models(rng, n_parts=10, n_stumps=500, D=960)
    cls = ctx.classifiers(models)
    net = pa.UnaryNet(ctx, dim=960, n_parts=10, seed=7)
    before = learned.evaluate(ctx, net, cls, n_fields=64, batch=16, ny=30, nx=40, seed=9)
    losses = learned.train(ctx, net, cls, n_fields=1024, batch=16, ny=30, nx=40, lr=2e-3,
                           lr_final=2e-4, epochs=2, seed=8)
    after = learned.evaluate(ctx, net, cls, n_fields=64, batch=16, ny=30, nx=40, seed=9)
    assert np.isfinite(losses).all()
    # the output biases start at the mean targets: the loss starts at the
    # constant predictor's level and must fall below it
    assert losses[-8:].mean() < 0.9 * losses[:8].mean()
    assert (after["mse"] < before["mse"]).all()  # before: the untrained net
    # parts whose targets are nearly all clipped (log 1e-4) have little
    # variance to explain: no part may end worse than its constant, and the
    # parts together must gain
    assert (after["mse"] <= 1.02 * after["const_mse"]).all(), after["gain"]
    assert after["gain"].mean() > 0.05, after["gain"]
    flags = learned.calibrate(after["max_abs_err"])
    assert flags.tolist() == (after["max_abs_err"] <= 1e-2).astype(int).tolist()
    net.close()


@pytest.mark.gpu
@pytest.mark.parametrize("on_net", ["all", "mixed", "none"])
def test_find_obj_learned_equals_its_parts(ctx, pa, on_net):
    """pa_find_obj_batch_learned = the net's scores (or AdaBoost's for the
    parts off the net) -> pa_unary_maps -> pa_ps_infer (bIsSparse)."""
    import torch

    R, H, W = 12, 48, 64
    imgs = [synth.make_image(500 + i, R=R, H=H, W=W, n_stumps=60, D=128, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i in range(2)]
    cls = ctx.classifiers(imgs[0]["models"])
    net = pa.UnaryNet(ctx, dim=128, n_parts=10, seed=3)
    P = 10
    flags = {"all": np.ones(P, np.int32), "none": np.zeros(P, np.int32),
             "mixed": (np.arange(P) % 2).astype(np.int32)}[on_net]
    desc = torch.from_numpy(np.stack([im["desc"] for im in imgs])).cuda()
    fields = desc.to(torch.bfloat16)
    e = pa.exp_param(R=R, interpolate=True)
    got = pa.find_obj_batch_learned(ctx, e, [im["tree"] for im in imgs], net, fields,
                                    imgs[0]["Tig"], H, W, part_on_net=flags, cls_list=cls,
                                    desc=desc, want_marg=True)
    for i, im in enumerate(imgs):
        sc_net = net.forward(fields[i], exp_out=True)
        sc_ada = ctx.score_grids(cls, desc[i])
        sc = torch.where(torch.from_numpy(flags.astype(bool)).cuda()[:, None, None, None],
                         sc_net, sc_ada).contiguous()
        lu = ctx.unary_maps(sc, im["Tig"], H, W, interpolate=True)
        want = ctx.compute_root_posterior_rot(e, im["tree"], lu, is_sparse=True)
        g = got[i]["log_marg"].cpu().numpy()
        w = want["log_marg"].cpu().numpy() if hasattr(want["log_marg"], "cpu") else want["log_marg"]
        assert np.abs(g - w).max() <= 1e-5 * max(1.0, np.abs(w).max())
        assert np.array_equal(got[i]["best_conf"][:, 2:6], want["best_conf"][:, 2:6])
    if on_net == "none":
        plain = ctx.find_obj_batch(e, [im["tree"] for im in imgs], cls, desc, imgs[0]["Tig"], H,
                                   W, want_marg=True)
        no_fields = pa.find_obj_batch_learned(ctx, e, [im["tree"] for im in imgs], net, None,
                                              imgs[0]["Tig"], H, W, part_on_net=flags,
                                              cls_list=cls, desc=desc, want_marg=True)
        for a, b, c in zip(got, plain, no_fields):
            assert np.array_equal(a["best_conf"], b["best_conf"])
            assert np.array_equal(a["log_marg"].cpu().numpy(), b["log_marg"].cpu().numpy())
            assert np.array_equal(c["log_marg"].cpu().numpy(), b["log_marg"].cpu().numpy())
    net.close()


@pytest.mark.gpu
def test_net_errors_are_statuses(ctx, pa):
    import torch

    with pytest.raises(pa.PaError):
        pa.UnaryNet(ctx, dim=100, n_parts=10)
    with pytest.raises(pa.PaError):
        pa.UnaryNet(ctx, dim=64, n_parts=65)
    net = pa.UnaryNet(ctx, dim=64, n_parts=4)
    with pytest.raises(ValueError):
        net.set_params(np.zeros(3, np.float32))
    with pytest.raises(pa.PaError):
        net.adam(lr=-1.0)
    x = torch.zeros((1, 4, 4, 64), device="cuda")
    y = net.forward(x)  # zero fields: biases only
    assert torch.isfinite(y).all()
    net.close()
