"""Parity at the workload the throughput numbers are quoted on.

find_obj at 640x480, 24 rotations, 22 AdaBoost classifiers of 500 stumps over
960-d descriptors at stride 4 (one 160x120 field per rotation, Gamma(0.5, 1)
values L2-normalised per location), the 10-part tree with per-image pairwise
terms (offsets U(10, 60) px, sigma U(2, 12) px, i.e. spatial kernels of up to
73 taps, rotation sigma U(1, 3) bins), through pa_find_obj_batch as bench.py
calls it, against the FP32 oracle and its FP64 twin:

  * all 22 score grids bit-exact (computeScoreGrid, partdetect_test.cpp:344-405);
  * all 10 log marginals and the root posterior within TOL_F32 per cell after
    max-normalisation of the FP32 oracle and TOL_F64 of the FP64 one;
  * best_conf identical, apart from the documented near-tie rule;
  * log Z of every part against the FP64 log-sum-exp of the FP64 marginal.

The uneven-batch case runs images of the batching workload's shapes (sides
200..640 px rounded to 4, rotation counts 12 / 24 / 48) through
pa_find_obj_multi against the oracle and against one-image calls.

The oracle runs on host threads (its C calls release the GIL).
"""
import concurrent.futures as cf
import math
import os

import numpy as np
import pytest

import oracle as orc_mod
from partapp_gb300 import synth
from test_gpu_parity import TOL_F32, TOL_F64, compare_ps, maxnorm_err

pytestmark = pytest.mark.gpu

STRIDE, D = 4, 960


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
    yield c
    c.close()


@pytest.fixture(scope="module")
def orc():
    orc_mod.build()
    return orc_mod


def _pool():
    return cf.ThreadPoolExecutor(max_workers=max(2, min(16, os.cpu_count() or 2)))


def _device_descriptors(seed, R, ny, nx):
    """[R][ny][nx][960] on cuda:0: Gamma(0.5, 1) = z^2 / 2, L2-normalised."""
    import torch

    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    z = torch.randn((R, ny, nx, D), generator=g, device="cuda", dtype=torch.float32)
    z.mul_(z).mul_(0.5)
    z.div_(torch.linalg.vector_norm(z, dim=-1, keepdim=True))
    return z


def _log_unary(orc, scores, Tig, H, W):
    """[P][R][ny][nx] score grids -> [P][R][H][W] log unaries (bilinear map,
    clip_scores_fill, computeLogGrid), as the oracle's find_obj forms them."""
    P, R = scores.shape[:2]
    out = np.empty((P, R, H, W), np.float32)
    for p in range(P):
        for r in range(R):
            out[p, r] = orc.clip_log(orc.transform_grid(scores[p, r], (H, W), Tig, 0.0, 1))
    return out


def _oracle_ps(orc, pool, e, tree, lu):
    """FP32 and FP64 oracle PS of one image, queued on the pool."""
    return (pool.submit(orc.ps_infer, e, tree, lu, False, True, False),
            pool.submit(orc.ps_infer, e, tree, lu.astype(np.float64), True, True, False))


def _check_image(lu, got, futs):
    want, want64 = futs[0].result(), futs[1].result()
    compare_ps(got, want, want64)
    assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32
    assert maxnorm_err(got["root_post"], want64["root_post"]) <= TOL_F64
    for p in range(lu.shape[0]):
        m = want64["log_marg"][p]
        lz = m.max() + math.log(np.exp(m - m.max()).sum())
        assert abs(got["log_z"][p] - lz) <= 1e-3 * max(1.0, abs(lz)), (p, got["log_z"][p], lz)


def test_bench_workload_two_images(ctx, orc):
    import torch

    R, H, W = 24, 480, 640
    ny, nx = H // STRIDE, W // STRIDE
    rng = np.random.default_rng(4242)
    models = synth.make_models(rng, n_parts=22, n_stumps=500, D=D)
    trees = [synth.make_tree(rng, R=R, offset_range=(10.0, 60.0), sigma_range=(2.0, 12.0))
             for _ in range(2)]
    # the widest spatial kernel the workload allows: sigma 12 px, 73 taps
    trees[0]["C"][2] = [144.0, 0.0, 0.0, 144.0]
    descs = torch.stack([_device_descriptors(77 + i, R, ny, nx) for i in range(2)])
    cls = ctx.classifiers(models)
    Tig = synth.grid_to_image(STRIDE)
    from partapp_gb300 import exp_param

    sc = torch.zeros((22, 2 * R, ny, nx), dtype=torch.float32, device="cuda")
    got = ctx.find_obj_batch(exp_param(R=R), trees, cls, descs, Tig, H, W, want_marg=True,
                             want_root=True, scores_out=sc)
    sc = sc.cpu().numpy().reshape(22, 2, R, ny, nx)
    host = descs.cpu().numpy()
    e = orc.make_exp(R=R, sparse=True)
    with _pool() as pool:
        futs = {(c, i): pool.submit(orc.adaboost_eval, models["f"][c], models["p"][c],
                                    models["theta"][c], models["alpha"][c], host[i])
                for c in range(22) for i in range(2)}
        for (c, i), f in futs.items():
            assert np.array_equal(sc[c, i], f.result()), f"classifier {c}, image {i}"
        lus = [_log_unary(orc, sc[:10, i], Tig, H, W) for i in range(2)]
        ps = [_oracle_ps(orc, pool, e, trees[i], lus[i]) for i in range(2)]
        for i in range(2):
            g = dict(got[i], log_marg=got[i]["log_marg"].cpu().numpy(),
                     root_post=got[i]["root_post"].cpu().numpy())
            _check_image(lus[i], g, ps[i])


def test_uneven_batch_shapes(ctx, orc):
    """Sides 200..640 px (multiples of 4) and R in {12, 24, 48}, 960-d
    descriptors, 10 x 500 stumps, per-image trees as in the workload."""
    from partapp_gb300 import exp_param

    shapes = [(48, 200, 640), (24, 264, 200), (12, 640, 324), (48, 200, 640)]
    rng = np.random.default_rng(515)
    models = synth.make_models(rng, n_parts=10, n_stumps=500, D=D)
    cls = ctx.classifiers(models)
    Tig = synth.grid_to_image(STRIDE)
    imgs = []
    for i, (R, H, W) in enumerate(shapes):
        tree = synth.make_tree(rng, R=R, offset_range=(10.0, 60.0), sigma_range=(2.0, 12.0))
        imgs.append(dict(exp=exp_param(R=R), tree=tree,
                         desc=_device_descriptors(900 + i, R, H // STRIDE, W // STRIDE),
                         Tig=Tig, H=H, W=W))
    got = ctx.find_obj_multi(imgs, cls, want_marg=True)
    with _pool() as pool:
        futs = []
        for i, im in enumerate(imgs):
            one = ctx.find_obj(im["exp"], im["tree"], cls, im["desc"], Tig, im["H"], im["W"])
            assert np.array_equal(got[i]["best_conf"], one["best_conf"]), i
            gm = got[i]["log_marg"].cpu().numpy()
            assert np.array_equal(gm, one["log_marg"].cpu().numpy()), i
            e = orc.make_exp(R=im["exp"].num_rotation_steps, sparse=True)
            futs.append((i, gm, e, pool.submit(orc.find_obj, e, im["tree"], models,
                                               im["desc"].cpu().numpy(), Tig, im["H"], im["W"])))
        f64 = [pool.submit(orc.ps_infer, e, imgs[i]["tree"],
                           f.result()["log_unary"].astype(np.float64), True, True, False)
               for i, gm, e, f in futs]
        for (i, gm, e, f), w64 in zip(futs, f64):
            compare_ps(dict(got[i], log_marg=gm), f.result(), w64.result())
