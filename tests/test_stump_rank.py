"""Rank form of the stump test (k_rank_buckets + k_rank_votes) against the
oracle's evaluateFeaturePoint (libAdaBoost/AdaBoost.h:131-160), bit-exact:

  * features carrying 40 and 100 distinct thresholds (7-step searches);
  * a feature with 130 distinct thresholds: the set does not qualify and the
    float kernels run (also bit-exact);
  * 33 classifiers (more than one warp each per CTA allows): float kernels;
  * descriptor fields that start off a 16-byte boundary (scalar loads);
  * NaN descriptor values: the rank form gives what the float kernels give
    (the sign-folded test is false for NaN, as v < t is).
"""
import numpy as np
import pytest

from partapp_gb300 import synth

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


def _check(ctx, orc, m, desc, parts=None):
    cls = ctx.classifiers(m)
    got = ctx.score_grids(cls, desc)
    got = got.cpu().numpy() if hasattr(got, "cpu") else got
    host = desc.cpu().numpy() if hasattr(desc, "cpu") else desc
    for p in parts if parts is not None else range(len(m["f"])):
        want = orc.adaboost_eval(m["f"][p], m["p"][p], m["theta"][p], m["alpha"][p], host)
        assert np.array_equal(got[p], want), f"classifier {p}"
    return got


def _crowd(m, rng, feature, n_distinct, desc):
    """Put n_distinct distinct thresholds on one feature, spread over the
    classifiers, some of them equal to descriptor values (ties)."""
    n_cls, n_st = m["f"].shape
    vals = np.sort(rng.uniform(0.0, 0.1, n_distinct).astype(np.float32))
    flat = desc.reshape(-1, desc.shape[-1])[:, feature]
    vals[: min(8, n_distinct)] = flat[: min(8, n_distinct)]
    for k, v in enumerate(vals):
        c, i = k % n_cls, (k * 7) % n_st
        m["f"][c, i] = feature
        m["theta"][c, i] = v


@pytest.mark.parametrize("distinct", [40, 100])
def test_rank_deep_search(ctx, orc, distinct):
    rng = np.random.default_rng(31 + distinct)
    R, ny, nx, D = 2, 9, 31, 960
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    m = synth.make_models(rng, n_parts=22, n_stumps=160, D=D)
    _crowd(m, rng, 5, distinct, desc)
    _crowd(m, rng, 900, 17, desc)
    _check(ctx, orc, m, desc)


def test_rank_fallback_many_thresholds(ctx, orc):
    rng = np.random.default_rng(77)
    R, ny, nx, D = 2, 9, 31, 960
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    m = synth.make_models(rng, n_parts=22, n_stumps=160, D=D)
    _crowd(m, rng, 11, 130, desc)
    _check(ctx, orc, m, desc)


def test_float_path_33_classifiers(ctx, orc):
    rng = np.random.default_rng(78)
    R, ny, nx, D = 2, 9, 31, 960
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    m = synth.make_models(rng, n_parts=33, n_stumps=100, D=D)
    _check(ctx, orc, m, desc)


def test_rank_unaligned_fields(ctx, orc):
    import torch

    rng = np.random.default_rng(79)
    R, ny, nx, D = 3, 9, 31, 960
    host = synth.make_descriptors(rng, R, ny, nx, D)
    buf = torch.empty(host.size + 1, dtype=torch.float32, device="cuda")
    desc = buf[1:].view(R, ny, nx, D)
    desc.copy_(torch.from_numpy(host))
    assert desc.data_ptr() % 16 != 0
    m = synth.make_models(rng, n_parts=12, n_stumps=200, D=D)
    _check(ctx, orc, m, desc)


def test_rank_nan_matches_float_path(ctx):
    rng = np.random.default_rng(80)
    R, ny, nx, D = 2, 9, 31, 960
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    flat = desc.reshape(-1)
    flat[3::53] = np.nan
    flat[7::97] = -np.nan
    flat[11::61] = np.inf
    m = synth.make_models(rng, n_parts=33, n_stumps=120, D=D)
    # the same 22 classifiers in a rank-eligible set and inside a 33-set
    sub = {k: (v[:22] if isinstance(v, np.ndarray) else v) for k, v in m.items()}
    rank = ctx.score_grids(ctx.classifiers(sub), desc)
    flt = ctx.score_grids(ctx.classifiers(m), desc)
    assert np.array_equal(rank, flt[:22])
