"""SHAPEv5 shape-context descriptor grids (computeDescriptorGrid,
libPartDetect/partdetect_aux.cpp:77-190; libKMA2/ShapeDescriptor.cpp:168-261).

The CPU tests pin the oracle's restatement with known answers; the GPU tests
compare pa_descriptor_grid with the oracle on seeded synthetic grey images
(smoothed noise with a few straight step edges: the LSP images the reference
ran on are not available) and feed the descriptors through the window
classifier."""
import math

import numpy as np
import pytest

INT_MIN = np.float32(-2147483648.0)
ATAN2_FRAC = 2e-4  # descriptor entries that atan2f's last bit may move (measured ~1e-5)


def axes(deg, flip=False):
    """partdetect_test.cpp:171-185: x axis (cos, sin), negated when flipped;
    y axis (-sin, cos)."""
    r = math.radians(deg)
    ax = np.array([math.cos(r), math.sin(r)])
    ay = np.array([-math.sin(r), math.cos(r)])
    return (-ax if flip else ax), ay


def grey_image(seed, h=96, w=128):
    from scipy.ndimage import gaussian_filter

    rng = np.random.default_rng(seed)
    img = gaussian_filter(rng.uniform(0, 255, (h, w)), 1.5)
    yy, xx = np.mgrid[0:h, 0:w]
    for _ in range(4):  # a few straight step edges
        a = rng.uniform(0, np.pi)
        c = rng.uniform(0.3, 0.7) * (h * abs(math.sin(a)) + w * abs(math.cos(a)))
        img = img + 60.0 * ((xx * math.cos(a) + yy * math.sin(a)) > c)
    img = (img - img.min()) / (img.max() - img.min()) * 255.0
    return img.astype(np.float32)


# ------------------------------------------------------------ oracle pins
def test_patch_tables_known_values(orc):
    """initPatchMask(21): exp(-d^2 / 90) inside radius^2 = 100, 0 outside;
    precompute_patch_idx: lrpos = 3 log(1 + r / 10), lcpos in [0, 4)."""
    m, lc, lr = orc.patch_tables()
    assert m[10, 10] == 1.0
    assert m[10, 0] == 0.0 and m[0, 0] == 0.0  # d^2 = 100 is outside (strict <)
    assert m[10, 1] == np.float32(math.exp(-81.0 / 90.0)) or abs(m[10, 1] - math.exp(-0.9)) < 1e-7
    d2 = (np.arange(21)[:, None] - 10) ** 2 + (np.arange(21)[None, :] - 10) ** 2
    assert ((m > 0) == (d2 < 100)).all()
    assert lr[10, 10] == 0.0
    assert abs(lr[10, 20] - 3 * math.log(2.0)) < 1e-6
    assert lc.min() >= 0.0 and lc.max() < 4.0 + 1e-6
    assert np.allclose(m, m.T)


def test_uniform_patch_gives_int_min(orc):
    """No gradient -> no edge -> 0/0 normalisation -> NaN -> (int) on x86-64."""
    v = orc.shape_descriptor(np.full((21, 21), 128.0, np.float32))
    assert (v == INT_MIN).all()


def test_vertical_ramp_edge_bins_one_orientation(orc):
    """A vertical ramp has dy = 0 and dx > 0 along one column: every Canny
    edge pixel has orientation 0, so only orientation bin 0 of each
    (radius, angle) cell can be non-zero; values are integers in [0, 255]."""
    row = np.array([0.0] * 9 + [50.0, 128.0, 206.0] + [255.0] * 9, np.float32)
    v = orc.shape_descriptor(np.tile(row, (21, 1)))
    nz = np.nonzero(v)[0]
    assert len(nz) > 0 and (nz % 8 == 0).all()
    assert (v == np.round(v)).all() and v.min() >= 0 and v.max() <= 255


def test_feature_grid_axis_aligned(orc):
    """Rotation 0: the box is [0, w] x [0, h], nx = floor((w + 1) / step) + 1."""
    ax, ay = axes(0.0)
    rect, nx, ny = orc.feature_grid(128, 96, ax, ay, 4.0)
    assert np.allclose(rect, [0, 128, 0, 96])
    assert (nx, ny) == (math.floor(129 / 4) + 1, math.floor(97 / 4) + 1)


def test_descriptor_grid_valid_positions(orc):
    """A cell is computed iff its image position lies desc_size + 1 inside."""
    img = grey_image(3, 64, 80)
    ds, step = 10, 4.0
    for deg in (0.0, 30.0):
        ax, ay = axes(deg)
        rect, nx, ny = orc.feature_grid(80, 64, ax, ay, step)
        cells, valid = orc.descriptor_grid(img, ax, ay, step, ds)
        iy, ix = np.mgrid[0:ny, 0:nx]
        x2, y2 = rect[0] + ix * step, rect[2] + iy * step
        px, py = x2 * ax[0] + y2 * ay[0], x2 * ax[1] + y2 * ay[1]
        want = (px >= ds + 1) & (px <= 80 - (ds + 1)) & (py >= ds + 1) & (py <= 64 - (ds + 1))
        assert np.array_equal(valid.astype(bool), want)
        assert (cells[~want] == 0).all()
        v = cells[want]
        assert ((v == INT_MIN) | ((v >= 0) & (v <= 255) & (v == np.round(v)))).all()


def test_recursive_gaussian_impulse_response(orc):
    """smooth() (gauss_iir.cpp:1391-1400) is Deriche's recursive Gaussian:
    away from the borders an impulse comes out as a separable bump close to
    exp(-d^2 / (2 sigma^2)), with unit-order gain."""
    sigma = 1.6
    img = np.zeros((64, 64), np.float32)
    img[32, 32] = 1.0
    out = orc.smooth(img, sigma).astype(np.float64)
    c = out[32, 32]
    d = np.arange(-4, 5)
    row = out[32, 32 + d] / c
    assert np.abs(row - np.exp(-d**2 / (2 * sigma**2))).max() < 0.03
    assert np.allclose(row, out[32 + d, 32] / c, atol=1e-5)  # same filter along y and x
    sep = np.outer(out[:, 32], out[32, :]) / c
    assert np.abs(out - sep).max() < 1e-6 * abs(c) + 1e-9
    assert 0.9 < out.sum() < 1.1


def test_large_windows_sample_the_smoothed_image(orc):
    """desc_size > 10: patch_scale = (2 d + 1) / 21 > 1, the patches come from
    the image smoothed with sigma = patch_scale (partdetect_aux.cpp:88-98)."""
    img = grey_image(1, 48, 56)
    ax, ay = axes(0.0)
    cells, valid = orc.descriptor_grid(img, ax, ay, 4.0, 12)
    assert valid.sum() > 0
    v = cells[valid.astype(bool)]
    assert ((v == INT_MIN) | ((v >= 0) & (v <= 255))).all()


# --------------------------------------------------------------- GPU parity
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


def _compare(got, want, vg, vw):
    assert np.array_equal(vg, vw)
    g, w = got[vw.astype(bool)], want[vw.astype(bool)]
    diff = g != w
    return float(diff.mean()) if g.size else 0.0, float(np.abs(g - w)[diff].max()) if diff.any() else 0.0


@pytest.mark.gpu
@pytest.mark.parametrize("deg,flip", [(0.0, False), (15.0, False), (97.5, True), (-142.5, False)])
def test_descriptor_grid_matches_oracle(ctx, orc, deg, flip):
    img = grey_image(10 + abs(int(deg)), 96, 128)
    ax, ay = axes(deg, flip)
    want, vw = orc.descriptor_grid(img, ax, ay, 4.0, 10)
    got, vg = ctx.descriptor_grid(img, ax, ay, 4.0, 10)
    frac, worst = _compare(got, want, vg, vw)
    print(f"rot {deg} flip {flip}: {vw.sum()} cells, mismatching entries {frac:.2e}, max |d| {worst}")
    # every float and double operation follows the reference's types and
    # order; the one library call whose last bit differs between CUDA and the
    # host's libm is atan2f (glibc's is not correctly rounded either), which
    # moves a quantised value by one in ~1e-5 of the entries
    assert frac <= ATAN2_FRAC and worst <= 2
    assert vw.sum() > 100


@pytest.mark.gpu
def test_descriptor_grid_device_memory_and_smaller_window(ctx, orc):
    import torch

    img = grey_image(5, 80, 100)
    ax, ay = axes(45.0)
    want, vw = orc.descriptor_grid(img, ax, ay, 3.0, 7)
    got, vg = ctx.descriptor_grid(torch.from_numpy(img).cuda(), ax, ay, 3.0, 7)
    frac, worst = _compare(got.cpu().numpy(), want, vg.cpu().numpy(), vw)
    assert frac <= ATAN2_FRAC and worst <= 2


@pytest.mark.gpu
@pytest.mark.parametrize("desc_size,deg", [(12, 20.0), (16, -60.0)])
def test_descriptor_grid_smoothed_source(ctx, orc, desc_size, deg):
    """Windows wider than the 21-pixel patch: the recursive Gaussian runs on
    the GPU first; still bit-exact."""
    img = grey_image(30 + desc_size, 96, 112)
    ax, ay = axes(deg)
    want, vw = orc.descriptor_grid(img, ax, ay, 4.0, desc_size)
    got, vg = ctx.descriptor_grid(img, ax, ay, 4.0, desc_size)
    frac, worst = _compare(got, want, vg, vw)
    print(f"desc_size {desc_size}: {vw.sum()} cells, mismatching entries {frac:.2e}, max |d| {worst}")
    assert frac <= ATAN2_FRAC and worst <= 2 and vw.sum() > 20


@pytest.mark.gpu
def test_descriptor_grid_errors(ctx, pa):
    with pytest.raises(pa.PaError) as ei:
        ctx.descriptor_grid(grey_image(1, 40, 40), [0.0, 0.0], [0.0, 1.0], 4.0, 5)
    assert ei.value.status == pa.PA_ERR_INVALID
    with pytest.raises(pa.PaError) as ei:
        ctx.descriptor_grid(grey_image(1, 40, 40), *axes(0.0), -1.0, 5)
    assert ei.value.status == pa.PA_ERR_INVALID


@pytest.mark.gpu
def test_descriptor_grid_feeds_window_classifier(ctx, orc):
    """Descriptors -> computeScoreGrid over 2 x 5 windows of cells (960-d),
    on the GPU end to end, against the oracle on the oracle's descriptors."""
    from partapp_gb300 import synth

    img = grey_image(21, 96, 128)
    ax, ay = axes(30.0)
    cw, vw = orc.descriptor_grid(img, ax, ay, 4.0, 10)
    cg, vg = ctx.descriptor_grid(img, ax, ay, 4.0, 10)
    rng = np.random.default_rng(4)
    m = synth.make_models(rng, n_parts=3, n_stumps=200, D=960)
    m["theta"] = rng.uniform(0, 60, m["theta"].shape).astype(np.float32)  # integer-valued features
    cls = ctx.classifiers(m)
    got = ctx.score_grids_window(cls, cg[None], vg[None], 2, 5, 1.0)
    for p in range(3):
        want = orc.score_grid_window(m["f"][p], m["p"][p], m["theta"][p], m["alpha"][p], cw, vw, 2,
                                     5, 1.0)
        # exact stump sums; a window that holds one of atan2f's rare moved
        # descriptor values may score differently
        assert (got[p, 0] == want).mean() >= 0.998, p


# ------------------------------------------------------ partdetect_dense
def _pd_models(seed, windows, n_stumps=120, desc_step=4):
    """Classifiers over each window's gx * gy * 96 features, thresholds in the
    descriptors' integer range."""
    rng = np.random.default_rng(seed)
    dims = [((wx // desc_step) + 1) * ((wy // desc_step) + 1) * 96 for wx, wy, _, _ in windows]
    f = np.stack([rng.integers(0, d, n_stumps) for d in dims]).astype(np.int32)
    theta = rng.uniform(0, 60, (len(windows), n_stumps)).astype(np.float32)
    p = np.where(rng.random((len(windows), n_stumps)) < 0.5, -1.0, 1.0).astype(np.float32)
    alpha = rng.uniform(0, 1, (len(windows), n_stumps)).astype(np.float32)
    return dict(f=f, p=p, theta=theta, alpha=alpha), dims


WINDOWS = [(4, 16, 2.0, 8.0), (8, 8, 4.0, 4.0), (0, 4, 0.0, 2.0)]  # 2x5 (960-d), 3x3, 1x2 cells


def test_mirror_border_is_symmetric_padding(orc):
    """add_image_border2 mirrors including the edge pixel: numpy 'symmetric'."""
    img = np.arange(30, dtype=np.float32).reshape(5, 6)
    out, used = orc.add_border(img, 2)
    assert used == 2 and np.array_equal(out, np.pad(img, 2, mode="symmetric"))
    out, used = orc.add_border(img, 9)  # wider than the image: reduced to min(w, h) - 1
    assert used == 4 and out.shape == (13, 14)


def test_partdetect_constant_classifier(orc):
    """A classifier whose every stump votes +alpha scores 1 on every complete
    window: its log unary is 0 where a window lands and LOG_ZERO elsewhere."""
    img = grey_image(2, 48, 64)
    n = 40
    m = dict(f=np.zeros((1, n), np.int32), p=np.ones((1, n), np.float32),
             theta=np.full((1, n), 1e9, np.float32), alpha=np.full((1, n), 0.5, np.float32))
    e = orc.make_exp(R=4)
    lu = orc.partdetect(e, m, [(0, 0, 0.0, 0.0)], 4, 10, 1.0, img)
    assert lu.shape == (1, 4, 48, 64)
    v = np.unique(lu)
    assert set(v.tolist()) <= {0.0, float(np.float32(-1e6))}
    assert (lu == 0).sum() > 50


@pytest.mark.gpu
@pytest.mark.parametrize("R,flip,ratio", [(6, False, 1.0), (4, True, 0.5)])
def test_partdetect_matches_oracle(ctx, orc, pa, R, flip, ratio):
    """pa_partdetect (border, per-rotation descriptor grids, window scores of
    three window shapes, squeeze, TM_DIRECT into the image, clip/log) against
    the oracle's partdetect_dense: bit-exact log unaries."""
    img = grey_image(40 + R, 72, 96)
    m, dims = _pd_models(R, WINDOWS)
    cls = [pa.Classifier.from_stumps(ctx, m["f"][i], m["p"][i], m["theta"][i], m["alpha"][i],
                                     dims[i]) for i in range(len(dims))]
    want = orc.partdetect(orc.make_exp(R=R), m, WINDOWS, 4, 10, ratio, img, flip)
    got = ctx.partdetect(pa.exp_param(R=R), img, cls, WINDOWS, 4, 10, ratio, flip)
    assert got.shape == want.shape
    z = want == np.float32(-1e6)
    diff = got != want
    print(f"R {R} flip {flip} ratio {ratio}: {int((~z).sum())} mapped cells, "
          f"{int(diff.sum())} differ in the last bits")
    # the same cells carry scores (the grids, windows and the rotated grid ->
    # image map are exact); the log of a score may differ in its last bit
    # between CUDA's logf and the host's (the unary-map bound), and a window
    # that holds one of atan2f's rare moved descriptor values scores differently
    assert np.array_equal(got == np.float32(-1e6), z)
    off = np.abs(got[~z] - want[~z]) > 4e-7 * np.maximum(1.0, np.abs(want[~z]))
    print(f"  cells beyond the logf bound: {int(off.sum())}")
    assert off.mean() <= 1e-3
    assert (~z).sum() > 100


@pytest.mark.gpu
@pytest.mark.parametrize("ratio,flip", [(0.25, False), (0.3, True)])
def test_partdetect_small_window_step(ctx, orc, pa, ratio, flip):
    """Window steps of 1 and 1.2 px (<= sqrt 2): rotated grid cells share
    pixels of the TM_DIRECT map and the reference's last writer wins."""
    img = grey_image(11, 40, 48)
    wins = WINDOWS[:2]
    m, dims = _pd_models(1, wins)
    cls = [pa.Classifier.from_stumps(ctx, m["f"][i], m["p"][i], m["theta"][i], m["alpha"][i],
                                     dims[i]) for i in range(len(wins))]
    want = orc.partdetect(orc.make_exp(R=3), m, wins, 4, 10, ratio, img, flip)
    got = ctx.partdetect(pa.exp_param(R=3), img, cls, wins, 4, 10, ratio, flip)
    z = want == np.float32(-1e6)
    assert np.array_equal(got == np.float32(-1e6), z)
    off = np.abs(got[~z] - want[~z]) > 4e-7 * np.maximum(1.0, np.abs(want[~z]))
    assert off.mean() <= 1e-3 and (~z).sum() > 1000


def _maxnorm(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.abs(np.exp(a - a.max()) - np.exp(b - b.max())).max())


@pytest.mark.gpu
def test_find_obj_from_image_two_scales(ctx, orc, pa):
    """--find_obj from a grey image at two scales: pa_partdetect (scale 0.875:
    3.5 px descriptor step, 9 px descriptors; scale 1.125: 4.5 px, 11 px ->
    pre-smoothed patches) then pa_ps_infer with bIsSparse, against the
    oracle's partdetect_dense + computeRootPosteriorRot."""
    from partapp_gb300 import synth

    img = grey_image(77, 64, 80)
    wins = [(4, 16, 2.0, 8.0)] * 10
    m, dims = _pd_models(9, wins)
    cls = [pa.Classifier.from_stumps(ctx, m["f"][i], m["p"][i], m["theta"][i], m["alpha"][i],
                                     dims[i]) for i in range(10)]
    kw = dict(n_scales=2, scale_range=(0.75, 1.25))
    want_lu = orc.partdetect(orc.make_exp(R=4, **kw), m, wins, 4, 10, 1.0, img)
    got_lu = ctx.partdetect(pa.exp_param(R=4, **kw), img, cls, wins, 4, 10, 1.0)
    assert got_lu.shape == want_lu.shape == (10, 2, 4, 64, 80)
    z = want_lu == np.float32(-1e6)
    assert np.array_equal(got_lu == np.float32(-1e6), z)
    off = np.abs(got_lu[~z] - want_lu[~z]) > 4e-7 * np.maximum(1.0, np.abs(want_lu[~z]))
    assert off.mean() <= 1e-3
    rng = np.random.default_rng(3)
    tree = synth.make_tree(rng, R=4, offset_range=(3.0, 10.0), sigma_range=(1.0, 3.0))
    want = orc.ps_infer(orc.make_exp(R=4, sparse=True, max_local_max=50, **kw), tree, want_lu)
    got = ctx.compute_root_posterior_rot(pa.exp_param(R=4, local_max=50, **kw), tree, got_lu,
                                         is_sparse=True)
    for p in range(10):
        for s in range(2):
            assert _maxnorm(got["log_marg"][p, s], want["log_marg"][p, s]) <= 1e-4, (p, s)
    assert np.array_equal(got["best_conf"][:, [0, 2, 4, 5]], want["best_conf"][:, [0, 2, 4, 5]])


# ------------------------------------------- detection masks and the ROI
def _positions(orc, w, h, deg, step, flip=False):
    ax, ay = axes(deg, flip)
    rect, nx, ny = orc.feature_grid(w, h, ax, ay, step)
    iy, ix = np.mgrid[0:ny, 0:nx]
    x2, y2 = rect[0] + ix * step, rect[2] + iy * step
    return ax, ay, (0.0 + x2 * ax[0]) + y2 * ay[0], (0.0 + x2 * ax[1]) + y2 * ay[1]


def blob_mask(seed, h, w, frac=0.5):
    """A detection mask of a few rectangles of ones (values 1 or 0.25) on zeros."""
    rng = np.random.default_rng(seed)
    m = np.zeros((h, w), np.float32)
    while (m != 0).mean() < frac:
        y0, x0 = rng.integers(0, h - 4), rng.integers(0, w - 4)
        m[y0:y0 + rng.integers(4, h // 2), x0:x0 + rng.integers(4, w // 2)] = rng.choice([1.0, 0.25])
    return m


def test_descriptor_grid_mask_and_roi_pins(orc):
    """partdetect_aux.cpp:128-145: after the inside test a position is skipped
    when detection_mask[(long) y][(long) x] == 0, then when it lies outside the
    ROI; the descriptors that remain are those of the unmasked grid."""
    img = grey_image(5, 64, 80)
    ds, step = 10, 4.0
    mask = blob_mask(6, 64, 80)
    for deg in (0.0, 37.0):
        ax, ay, px, py = _positions(orc, 80, 64, deg, step)
        full, vf = orc.descriptor_grid(img, ax, ay, step, ds)
        cells, valid = orc.descriptor_grid(img, ax, ay, step, ds, mask=mask)
        inside = vf.astype(bool)
        on = np.zeros_like(inside)
        on[inside] = mask[py[inside].astype(np.int64), px[inside].astype(np.int64)] != 0
        assert np.array_equal(valid.astype(bool), on)
        assert np.array_equal(cells[on], full[on]) and (cells[~on] == 0).all()
        assert 0 < on.sum() < inside.sum()
        roi = (20, 14, 41, 30)  # QRect(20, 14, 41, 30): x in [20, 60], y in [14, 43]
        cells, valid = orc.descriptor_grid(img, ax, ay, step, ds, roi=roi)
        want = inside & (px >= 20) & (px <= 60) & (py >= 14) & (py <= 43)
        assert np.array_equal(valid.astype(bool), want)
        assert np.array_equal(cells[want], full[want])
        # the whole image as the ROI tests nothing
        _, valid = orc.descriptor_grid(img, ax, ay, step, ds, roi=(0, 0, 80, 64))
        assert np.array_equal(valid, vf)
        # only a mask value equal to 0 removes a position: -0 does, NaN does not
        odd = np.where(mask == 0, np.float32(np.nan), np.float32(-0.0))
        _, valid = orc.descriptor_grid(img, ax, ay, step, ds, mask=odd)
        want = np.zeros_like(inside)
        want[inside] = np.isnan(odd[py[inside].astype(np.int64), px[inside].astype(np.int64)])
        assert np.array_equal(valid.astype(bool), want) and want.any()


def test_default_roi_drops_last_column_when_desc_size_is_zero(orc):
    """The default QRect(0, 0, x() - 1, y() - 1) has right() = x() - 2: with
    desc_size 0 the inside test alone would admit x up to x() - 1."""
    img = grey_image(7, 40, 48)
    ax, ay, px, py = _positions(orc, 48, 40, 0.0, 1.0)
    _, valid = orc.descriptor_grid(img, ax, ay, 1.0, 0)
    want = (px >= 1) & (px <= 46) & (py >= 1) & (py <= 38)
    assert np.array_equal(valid.astype(bool), want)
    _, valid = orc.descriptor_grid(img, ax, ay, 1.0, 0, roi=(0, 0, 48, 40))
    assert valid.astype(bool)[(px == 47) & (py == 20)].all()


def test_partdetect_mask_restricts_scored_cells(orc):
    """partdetect_test.cpp:135-146: each scale's mask sits in a zero array the
    size of the bordered image, so an all-ones mask only drops windows that
    reach into the mirrored border; a zero mask leaves every grid empty
    (not squeezed, :436-449) and every unary LOG_ZERO."""
    img = grey_image(8, 48, 64)
    wins = WINDOWS[:2]
    m, _ = _pd_models(4, wins)
    e = orc.make_exp(R=3)
    full = orc.partdetect(e, m, wins, 4, 10, 1.0, img)
    ones = orc.partdetect(e, m, wins, 4, 10, 1.0, img, mask=np.ones((1, 48, 64), np.float32))
    z = np.float32(-1e6)
    assert ((ones == full) | (ones == z)).all()
    assert (ones == z).sum() > (full == z).sum() and (ones != z).sum() > 100
    none = orc.partdetect(e, m, wins, 4, 10, 1.0, img, mask=np.zeros((1, 48, 64), np.float32))
    assert (none == z).all()


@pytest.mark.gpu
@pytest.mark.parametrize("deg,flip", [(0.0, False), (-67.5, True)])
def test_descriptor_grid_masked_matches_oracle(ctx, orc, deg, flip):
    import torch

    img = grey_image(60, 80, 112)
    mask = blob_mask(61, 80, 112)
    ax, ay = axes(deg, flip)
    for kw in (dict(mask=mask), dict(roi=(9, 17, 70, 45)), dict(mask=mask, roi=(30, 0, 82, 80))):
        want, vw = orc.descriptor_grid(img, ax, ay, 4.0, 10, **kw)
        got, vg = ctx.descriptor_grid(img, ax, ay, 4.0, 10, **kw)
        frac, worst = _compare(got, want, vg, vw)
        assert frac <= ATAN2_FRAC and worst <= 2 and vw.sum() > 20, kw
        assert (got[~vw.astype(bool)] == 0).all()
    dimg, dmask = torch.from_numpy(img).cuda(), torch.from_numpy(mask).cuda()
    got, vg = ctx.descriptor_grid(dimg, ax, ay, 4.0, 10, mask=dmask, roi=(9, 17, 70, 45))
    want, vw = orc.descriptor_grid(img, ax, ay, 4.0, 10, mask=mask, roi=(9, 17, 70, 45))
    frac, worst = _compare(got.cpu().numpy(), want, vg.cpu().numpy(), vw)
    assert frac <= ATAN2_FRAC and worst <= 2


@pytest.mark.gpu
def test_descriptor_grid_desc_size_zero(ctx, orc):
    """desc_size 0: the default ROI (right() = x() - 2) decides the last column."""
    img = grey_image(62, 40, 48)
    for deg in (0.0, 30.0):
        ax, ay = axes(deg)
        want, vw = orc.descriptor_grid(img, ax, ay, 1.0, 0)
        got, vg = ctx.descriptor_grid(img, ax, ay, 1.0, 0)
        frac, worst = _compare(got, want, vg, vw)
        assert frac <= ATAN2_FRAC and worst <= 2


@pytest.mark.gpu
@pytest.mark.parametrize("n_scales", [1, 2])
def test_partdetect_masked_matches_oracle(ctx, orc, pa, n_scales):
    """pa_partdetect_masked: per-scale masks read at the border offset; an
    all-zero mask (scale 1 of the two-scale case) empties every grid."""
    import torch

    img = grey_image(63, 64, 88)
    m, dims = _pd_models(5, WINDOWS)
    cls = [pa.Classifier.from_stumps(ctx, m["f"][i], m["p"][i], m["theta"][i], m["alpha"][i],
                                     dims[i]) for i in range(len(dims))]
    kw = dict(n_scales=2, scale_range=(0.875, 1.125)) if n_scales == 2 else {}
    masks = np.stack([blob_mask(64 + s, 64, 88, 0.6) for s in range(n_scales)])
    if n_scales == 2:
        masks[1] = 0
    want = orc.partdetect(orc.make_exp(R=4, **kw), m, WINDOWS, 4, 10, 1.0, img, mask=masks)
    for dev in (False, True):
        args = (torch.from_numpy(img).cuda(), torch.from_numpy(masks).cuda()) if dev else (img, masks)
        got = ctx.partdetect(pa.exp_param(R=4, **kw), args[0], cls, WINDOWS, 4, 10, 1.0,
                             mask=args[1])
        got = got.cpu().numpy() if dev else got
        assert got.shape == want.shape
        z = want == np.float32(-1e6)
        assert np.array_equal(got == np.float32(-1e6), z)
        off = np.abs(got[~z] - want[~z]) > 4e-7 * np.maximum(1.0, np.abs(want[~z]))
        assert off.mean() <= 1e-3 and (~z).sum() > 100
    if n_scales == 2:
        assert z[:, 1].all()
