"""pa_find_obj_queue: the message passing of a wave of images of uneven sizes
and rotation counts in one persistent launch draining a device work queue.

  * every image equals its pa_find_obj_multi result bit for bit (marginals,
    best_conf, log Z), with waves of several sizes (1, 2 and all images);
  * a subset matches the FP32 / FP64 oracle (compare_ps);
  * the workload's own shapes (960-d descriptors, sides up to 640 px,
    R = 48) equal one-image calls bit for bit;
  * a start gate the host never opens makes every dependency wait run out:
    the call returns PA_ERR_TIMEOUT and the context stays usable.
"""
import numpy as np
import pytest

from partapp_gb300 import synth
from test_gpu_parity import compare_ps

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def ctx():
    import torch

    from partapp_gb300 import build

    build.build()
    import partapp_gb300 as pa

    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pa.Context(0)
    yield c
    c.close()


def _small_images(device=True):
    import torch

    import partapp_gb300 as pa

    shapes = [(12, 48, 64), (12, 48, 64), (12, 40, 56), (16, 48, 64), (8, 32, 48), (24, 48, 64),
              (12, 48, 64)]
    imgs = [synth.make_image(800 + i, R=R, H=H, W=W, n_stumps=60, D=96, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i, (R, H, W) in enumerate(shapes)]
    batch = [dict(exp=pa.exp_param(R=im["R"]), tree=im["tree"],
                  desc=torch.from_numpy(im["desc"]).cuda(), Tig=im["Tig"], H=im["H"], W=im["W"])
             for im in imgs]
    return imgs, batch


def _same(a, b):
    assert np.array_equal(a["best_conf"], b["best_conf"])
    assert np.array_equal(np.asarray(a["log_z"]), np.asarray(b["log_z"]))
    assert np.array_equal(a["log_marg"].cpu().numpy(), b["log_marg"].cpu().numpy())


@pytest.mark.parametrize("per_wave", [1, 2, 32])
def test_queue_equals_multi(ctx, orc, per_wave):
    imgs, batch = _small_images()
    cls = ctx.classifiers(imgs[0]["models"])
    want = ctx.find_obj_multi(batch, cls, want_marg=True)
    got = ctx.find_obj_queue(batch, cls, want_marg=True, images_per_wave=per_wave)
    for i in range(len(batch)):
        _same(got[i], want[i])
    if per_wave == 32:
        for i in (2, 4, 5):
            im = imgs[i]
            e = orc.make_exp(R=im["R"], sparse=True)
            w = orc.find_obj(e, im["tree"], imgs[0]["models"], im["desc"], im["Tig"], im["H"],
                             im["W"])
            w64 = orc.ps_infer(e, im["tree"], w["log_unary"].astype(np.float64), f64=True,
                               want_hyps=False)
            compare_ps(dict(got[i], log_marg=got[i]["log_marg"].cpu().numpy()), w, w64)


def test_queue_workload_shapes_equal_one_image_calls(ctx):
    """960-d descriptors, 10 x 500 stumps, sides up to 640 px, R in {12, 24, 48},
    per-image trees with offsets U(10, 60) px and sigma U(2, 12) px."""
    import torch

    import partapp_gb300 as pa

    shapes = [(48, 200, 640), (24, 264, 200), (12, 640, 324), (48, 200, 640), (24, 480, 640)]
    rng = np.random.default_rng(616)
    models = synth.make_models(rng, n_parts=10, n_stumps=500, D=960)
    cls = ctx.classifiers(models)
    Tig = synth.grid_to_image(4)
    g = torch.Generator(device="cuda")
    g.manual_seed(5)
    batch = []
    for R, H, W in shapes:
        z = torch.randn((R, H // 4, W // 4, 960), generator=g, device="cuda")
        z.mul_(z).mul_(0.5)
        z.div_(torch.linalg.vector_norm(z, dim=-1, keepdim=True))
        tree = synth.make_tree(rng, R=R, offset_range=(10.0, 60.0), sigma_range=(2.0, 12.0))
        batch.append(dict(exp=pa.exp_param(R=R), tree=tree, desc=z, Tig=Tig, H=H, W=W))
    got = ctx.find_obj_queue(batch, cls, want_marg=True)
    for i, im in enumerate(batch):
        one = ctx.find_obj(im["exp"], im["tree"], cls, im["desc"], Tig, im["H"], im["W"])
        _same(got[i], one)


def test_queue_wait_runs_out_and_context_survives(ctx):
    """The host holds the start gate: no tile may start, every dependency wait
    runs out after the bound, the call reports PA_ERR_TIMEOUT."""
    import partapp_gb300 as pa

    imgs, batch = _small_images()
    cls = ctx.classifiers(imgs[0]["models"])
    with pytest.raises(pa.PaError) as ei:
        ctx.find_obj_queue(batch[:3], cls, hold_start=True, wait_timeout_ms=100.0)
    assert ei.value.status == pa.PA_ERR_TIMEOUT
    got = ctx.find_obj_queue(batch[:3], cls, want_marg=True)
    want = ctx.find_obj_multi(batch[:3], cls, want_marg=True)
    for a, b in zip(got, want):
        _same(a, b)
