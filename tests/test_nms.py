"""Hypothesis suppression, nms_recursive (libPictStruct/objectdetect_aux.cpp:
407-451), as saveRecoResults runs it on an image's merged root hypotheses.

The oracle (oracle/oracle.cpp, orc_nms_recursive) restates the double loop
with the reference's typing; it is pinned by hand-made cases (a hypothesis on
top of a better one is suppressed, one just outside the ellipse is not, the
ellipse's axes scale with the earlier hypothesis' scale, a suppressed
hypothesis still suppresses later ones).  The GPU flags must equal the
oracle's exactly, for ragged counts and coordinates placed on the ellipse's
edge.
"""
import numpy as np
import pytest

import oracle as orc_mod


@pytest.fixture(scope="module")
def orc():
    orc_mod.build()
    return orc_mod


def test_pins(orc):
    # train box 20 x 50: the ellipse of a scale-1 hypothesis has half axes 10, 25
    x = [100.0, 105.0, 109.9, 100.0, 300.0, 300.0, 318.0]
    y = [100.0, 100.0, 100.0, 124.9, 100.0, 100.0, 100.0]
    s = [1.0, 1.0, 1.0, 1.0, 2.0, 1.0, 1.0]
    sc = [9.0, 8.0, 7.0, 6.0, 5.0, 4.0, 3.0]
    got = orc.nms_recursive(x, y, s, sc, 20.0, 50.0)
    # 1: inside 0's ellipse; 2: x 9.9 < 10; 3: y 24.9 < 25; 5: on 4; 6: 18 < 20 (4 has scale 2)
    assert got.tolist() == [False, True, True, True, False, True, True]
    got = orc.nms_recursive([0.0, 10.0, 20.0], [0.0] * 3, [1.0] * 3, [3.0, 2.0, 1.0], 20.0, 50.0)
    assert got.tolist() == [False, False, False]  # exactly on the edge: 1.0 is not < 1
    got = orc.nms_recursive([0.0, 6.0, 12.0], [0.0] * 3, [1.0] * 3, [3.0, 2.0, 1.0], 20.0, 50.0)
    assert got.tolist() == [False, True, True]  # 2 is suppressed by 1, itself suppressed
    with pytest.raises(ValueError):
        orc.nms_recursive([0.0, 1.0], [0.0, 0.0], [1.0, 1.0], [1.0, 2.0], 20.0, 50.0)
    assert orc.nms_recursive([], [], [], [], 20.0, 50.0).shape == (0,)


def _case(rng, n):
    x = rng.uniform(0, 640, n).astype(np.float32)
    y = rng.uniform(0, 480, n).astype(np.float32)
    s = rng.uniform(0.5, 2.0, n).astype(np.float32)
    sc = np.sort(rng.normal(0, 5, n).astype(np.float32))[::-1].copy()
    sc[n // 3: n // 3 + 5] = sc[n // 3]  # ties are sorted too
    # some pairs on the edge of the earlier one's ellipse
    for k in range(1, n, 7):
        x[k] = np.float32(x[k - 1] + np.float32(0.5 * s[k - 1] * 25.0))
        y[k] = y[k - 1]
    return x, y, s, sc


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 255, 256, 257, 3001])
def test_gpu_matches_oracle(orc, n):
    import torch

    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    x, y, s, sc = _case(np.random.default_rng(n), n)
    want = orc.nms_recursive(x, y, s, sc, 25.0, 62.5)
    ctx = pa.Context(0)
    try:
        got = ctx.nms_recursive(x, y, s, sc, 25.0, 62.5)
        dev = ctx.nms_recursive(*[torch.from_numpy(v).cuda() for v in (x, y, s, sc)], 25.0, 62.5)
        assert np.array_equal(got, want)
        assert np.array_equal(dev.cpu().numpy().astype(bool), want)
        if n > 1:
            bad = sc.copy()
            bad[n - 1] = bad[0] + 1.0
            with pytest.raises(pa.PaError):
                ctx.nms_recursive(x, y, s, bad, 25.0, 62.5)
        assert ctx.nms_recursive(x[:0], y[:0], s[:0], sc[:0], 25.0, 62.5).shape == (0,)
    finally:
        ctx.close()


@pytest.mark.gpu
def test_invalid_arguments_are_errors():
    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    v = np.zeros(4, np.float32)
    ctx = pa.Context(0)
    try:
        for w, h in ((0.0, 50.0), (20.0, -1.0), (float("nan"), 50.0)):
            with pytest.raises(pa.PaError):
                ctx.nms_recursive(v, v, v + 1, v, w, h)
        with pytest.raises(ValueError):
            ctx.nms_recursive(v, v[:3], v, v, 20.0, 50.0)
        big = np.zeros(65537, np.float32)  # past the O(n^2) cap, refused before any work
        with pytest.raises(pa.PaError):
            ctx.nms_recursive(big, big, big + 1, big, 20.0, 50.0)
        assert ctx.nms_recursive(v, v, v + 1, v, 20.0, 50.0).tolist() == [False, True, True, True]
    finally:
        ctx.close()


# ------------------------------------------------------------------ libNms
# nms_recursive of libNms (libNms/nms.cpp:132-225) on rectangles, built from
# hypotheses by rect_from_hyp (:23-56): the test is the Mahalanobis distance
# of a later rectangle's centre in the earlier rectangle's frame, with the
# squared edge lengths as variances and ellipse_size^2 as the bound.


def test_rect_from_hyp_pins(orc):
    # scale 1.3 (float 1.29999995...) x 200 -> 259 px high, x 80 -> 103 px wide
    r = orc.rect_from_hyp(100.5, 50.25, 1.3, 200.0, 80.0)
    assert r.tolist() == [[49.0, -79.25], [152.0, -79.25], [152.0, 179.75], [49.0, 179.75]]


def test_rect_from_hyp_host_entry_matches_oracle(orc):
    """pa_rect_from_hyp runs on the host (no GPU needed)."""
    import partapp_gb300 as pa

    rng = np.random.default_rng(7)
    for _ in range(500):
        x, y = rng.uniform(-50, 700, 2).astype(np.float32)
        s = np.float32(rng.uniform(0.2, 3.0))
        h, w = rng.uniform(10, 300, 2)
        assert np.array_equal(pa.rect_from_hyp(x, y, s, h, w), orc.rect_from_hyp(x, y, s, h, w))


def test_nms_rects_pins(orc):
    box = lambda x, y, s: orc.rect_from_hyp(x, y, s, 100.0, 40.0)  # 40 wide, 100 high at scale 1
    run = lambda *bs: orc.nms_rects(np.stack(bs), np.arange(len(bs), 0, -1), 0.5).tolist()
    # ellipse 0.5: half axes 20 (x) and 50 (y) around an earlier scale-1 centre
    assert run(box(0, 0, 1), box(19.9, 0, 1)) == [False, True]
    assert run(box(0, 0, 1), box(20, 0, 1), box(40, 0, 1)) == [False] * 3  # on the edge: not < 1
    assert run(box(0, 0, 1), box(0, 49.9, 1)) == [False, True]
    assert run(box(0, 0, 1), box(0, 50, 1)) == [False, False]
    assert run(box(500, 0, 2), box(539, 0, 1)) == [False, True]  # scale 2: half axes 40, 100
    # a suppressed rectangle still suppresses later ones
    assert run(box(0, 0, 1), box(15, 0, 1), box(30, 0, 1)) == [False, True, True]
    with pytest.raises(ValueError):
        orc.nms_rects(np.stack([box(0, 0, 1), box(1, 0, 1)]), [1.0, 2.0])


def _rects_case(rng, n):
    """Hypothesis rectangles and rotated rectangles (general corners), scores
    descending with ties, centres crowded so that many pairs are close."""
    out = []
    for k in range(n):
        if k % 3 == 2:  # a rotated rectangle given by its corners
            cx, cy = rng.uniform(0, 200, 2)
            a = rng.uniform(0, np.pi)
            w, h = rng.uniform(5, 60, 2)
            u, v = np.array([np.cos(a), np.sin(a)]), np.array([-np.sin(a), np.cos(a)])
            c = np.array([cx, cy])
            out.append(np.stack([c - u * w / 2 - v * h / 2, c + u * w / 2 - v * h / 2,
                                 c + u * w / 2 + v * h / 2, c - u * w / 2 + v * h / 2]))
        else:
            x, y = rng.uniform(0, 200, 2).astype(np.float32)
            out.append(orc_mod.rect_from_hyp(x, y, np.float32(rng.uniform(0.3, 2.0)), 60.0, 25.0))
    sc = np.sort(rng.integers(0, max(2, n // 3), n).astype(np.float64))[::-1].copy()
    return np.stack(out) if out else np.zeros((0, 4, 2)), sc


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 2, 255, 256, 257, 2049])
def test_nms_rects_gpu_matches_oracle(orc, n):
    import torch

    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    rects, sc = _rects_case(np.random.default_rng(100 + n), n)
    ctx = pa.Context(0)
    try:
        for ell in (0.5, 0.3):
            want = orc.nms_rects(rects, sc, ell)
            assert np.array_equal(ctx.nms_rects(rects, sc, ell), want)
            dev = ctx.nms_rects(torch.from_numpy(rects).cuda(), torch.from_numpy(sc).cuda(), ell)
            assert np.array_equal(dev.cpu().numpy().astype(bool), want)
        if n > 1:
            bad = sc.copy()
            bad[n - 1] = bad[0] + 1.0
            with pytest.raises(pa.PaError):
                ctx.nms_rects(rects, bad)
        # a zero-width rectangle suppresses nothing (its test is NaN), as in the reference
        flat = rects.copy()
        flat[0, :, 0] = flat[0, 0, 0]
        assert np.array_equal(ctx.nms_rects(flat, sc), orc.nms_rects(flat, sc))
    finally:
        ctx.close()
