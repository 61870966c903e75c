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
    # bit-exact: every float and double operation follows the reference's
    # types and order (atan2f, the one libm call whose last bit could differ
    # between CUDA and the host, has not moved a quantised value here)
    assert frac == 0.0
    assert vw.sum() > 100


@pytest.mark.gpu
def test_descriptor_grid_device_memory_and_smaller_window(ctx, orc):
    import torch

    img = grey_image(5, 80, 100)
    ax, ay = axes(45.0)
    want, vw = orc.descriptor_grid(img, ax, ay, 3.0, 7)
    got, vg = ctx.descriptor_grid(torch.from_numpy(img).cuda(), ax, ay, 3.0, 7)
    frac, _ = _compare(got.cpu().numpy(), want, vg.cpu().numpy(), vw)
    assert frac == 0.0


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
    assert frac == 0.0 and vw.sum() > 20


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
        assert np.array_equal(got[p, 0], want), p  # exact descriptors, exact stump sums
