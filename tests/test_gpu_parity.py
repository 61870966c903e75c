"""Parity of the CUDA path (through the C-ABI) with the CPU oracle.

Tolerances:
  * AdaBoost scores, feature indexing, NO_CLASS_VALUE masks: bit-exact;
  * log unary maps: the same grid cells and float bilinear weights as the
    reference; the log differs from log(double) by at most a few ulp:
    |d| <= 4e-7 * max(1, |v|);
  * messages / marginals: per cell after max-normalisation,
    |exp(a - max a) - exp(b - max b)| <= 1e-4 against the FP32 oracle
    (TOL_F32) and <= 1e-3 against the FP64 oracle (TOL_F64);
  * argmax (rotation, x, y) per part: identical to the FP32 oracle, except
    where the two cells are a near-tie of the FP64 marginal (values within
    1e-4, the marginal tolerance); at most one such part per case.
"""
import math

import numpy as np
import pytest

import oracle as orc_mod
from partapp_gb300 import synth

pytestmark = pytest.mark.gpu

TOL_F32 = 1e-4
TOL_F64 = 1e-3
LOG_ZERO = np.float32(-1e6)


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


def maxnorm_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    pa_ = np.exp(a - a.max())
    pb_ = np.exp(b - b.max())
    return float(np.abs(pa_ - pb_).max())


def small_tree(rng, R):
    return synth.make_tree(rng, R=R, offset_range=(3.0, 10.0), sigma_range=(1.0, 3.0))


# --------------------------------------------------------------- AdaBoost
def test_score_grids_bit_exact(ctx, orc):
    rng = np.random.default_rng(1)
    R, ny, nx, D = 3, 7, 33, 200
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    m = synth.make_models(rng, n_parts=4, n_stumps=150, D=D)
    # plant exact ties v == theta on both polarities
    for p in range(4):
        for i in range(0, 150, 7):
            m["theta"][p, i] = desc[i % R, i % ny, i % nx, m["f"][p, i]]
    cls = ctx.classifiers(m)
    got = ctx.score_grids(cls, desc)
    for p in range(4):
        want = orc.adaboost_eval(m["f"][p], m["p"][p], m["theta"][p], m["alpha"][p], desc)
        assert np.array_equal(got[p], want), f"part {p}"
        assert cls[p].info()[2] == orc.sum_alpha(m["alpha"][p])


@pytest.mark.parametrize("polarity,n_parts", [("unit", 22), ("unit", 13), ("unit", 10),
                                              ("general", 22), ("special", 22)])
def test_score_grids_960_pipelined_bit_exact(ctx, orc, polarity, n_parts):
    """The 960-dim path (staged tiles, sign-folded stump test) on a ragged
    tile count, 22 classifiers and planted v == theta ties; a classifier with
    a non-unit polarity exercises the literal v*p < theta*p form; "special"
    plants +-inf and -0 descriptor values and +-0 and negative thresholds.
    (NaN descriptor values are outside the folded test's domain: it is exact
    for every non-NaN v.)"""
    rng = np.random.default_rng(9)
    R, ny, nx, D = 2, 7, 33, 960
    desc = synth.make_descriptors(rng, R, ny, nx, D)
    m = synth.make_models(rng, n_parts=n_parts, n_stumps=120, D=D)
    for p in range(n_parts):
        for i in range(0, 120, 5):
            m["theta"][p, i] = desc[i % R, (i // 3) % ny, i % nx, m["f"][p, i]]
    if polarity == "special":
        flat = desc.reshape(-1)
        for k, v in enumerate((np.inf, -np.inf, -0.0, 0.0)):
            flat[k::37] = v
        m["theta"][:, ::11] = 0.0
        m["theta"][:, 3::11] = -0.0
        m["theta"][:, 5::11] = -m["theta"][:, 5::11]
    if polarity == "general":
        m["p"][3, ::7] = 0.5
        m["p"][4, ::9] = -2.0
    cls = ctx.classifiers(m)
    got = ctx.score_grids(cls, desc)
    for p in range(n_parts):
        want = orc.adaboost_eval(m["f"][p], m["p"][p], m["theta"][p], m["alpha"][p], desc)
        assert np.array_equal(got[p], want), f"part {p}"


def test_classifier_text_format(ctx, orc):
    text = "4\n3\t\n0\t1\t0.5\t0.1\t0.25\t\n2\t-1\t0.75\t0.2\t0.6\t\n3\t1\t0.125\t0.3\t0.9\t\n"
    from partapp_gb300 import Classifier

    cl = Classifier.parse(ctx, text)
    assert cl.info() == (4, 3, np.float32(0.5 + 0.75 + 0.125))
    v = np.array([[[[0.2, 0.0, 0.7, 0.95]]]], dtype=np.float32)
    got = ctx.score_grids([cl], v, normalize=False)
    want = orc.adaboost_eval([0, 2, 3], [1, -1, 1], [0.25, 0.6, 0.9], [0.5, 0.75, 0.125], v,
                             normalize=False)
    assert got[0, 0, 0, 0] == want[0, 0, 0]


def test_malformed_classifier_text_is_an_error(ctx, pa):
    """Bad model files give PA_ERR_INVALID: out-of-range or non-numeric
    counts, a stump count the text cannot hold, truncated stumps, feature
    indices outside [0, D)."""
    for text in ("", "abc", "1e30 5\n", "nan 3\n", "960 nan\n", "960 1000000000\n",
                 "960 2\n1 1 0.5 0 0.1\n", "960 1\n1e12 1 1 0 0.1\n",
                 "960 1\n-1 1 1 0 0.1\n", "960 1\n960 1 1 0 0.1\n", "0 1\n0 1 1 0 0\n"):
        with pytest.raises(pa.PaError):
            pa.Classifier.parse(ctx, text)


@pytest.mark.parametrize("grid_step", [1.0, 2.0])
def test_score_grids_window_bit_exact(ctx, orc, grid_step):
    rng = np.random.default_rng(2)
    F, ny, nx, dc, gx, gy = 2, 11, 13, 16, 3, 2
    cells = synth.make_descriptors(rng, F, ny, nx, dc)
    valid = (rng.random((F, ny, nx)) > 0.05).astype(np.uint8)
    m = synth.make_models(rng, n_parts=3, n_stumps=80, D=gx * gy * dc)
    cls = ctx.classifiers(m)
    got = ctx.score_grids_window(cls, cells, valid, gx, gy, grid_step)
    for p in range(3):
        for k in range(F):
            want = orc.score_grid_window(m["f"][p], m["p"][p], m["theta"][p], m["alpha"][p],
                                         cells[k], valid[k], gx, gy, grid_step)
            assert np.array_equal(got[p, k], want), (p, k)


# -------------------------------------------------------------- unary maps
@pytest.mark.parametrize("interpolate", [True, False])
@pytest.mark.parametrize("Tig", [synth.grid_to_image(4.0), synth.grid_to_image(4.0, 1.5, 2.25)])
def test_unary_maps(ctx, orc, interpolate, Tig):
    rng = np.random.default_rng(3)
    P, R, ny, nx, H, W = 2, 3, 15, 20, 60, 80
    s = rng.uniform(-1, 1, (P, R, ny, nx)).astype(np.float32)
    s[:, :, 3, 4] = 0.0
    got = ctx.unary_maps(s, Tig, H, W, interpolate=interpolate)
    for p in range(P):
        for r in range(R):
            img = orc.transform_grid(s[p, r], (H, W), Tig, 0.0, 1 if interpolate else 2)
            want = orc.clip_log(img)
            z = want == LOG_ZERO
            assert np.array_equal(got[p, r] == LOG_ZERO, z)
            d = np.abs(got[p, r][~z] - want[~z])
            assert np.all(d <= 4e-7 * np.maximum(1.0, np.abs(want[~z])))


def test_unary_maps_rotated_grid(ctx, orc):
    rng = np.random.default_rng(4)
    a = math.radians(22.5)
    Tig = np.array([[4 * math.cos(a), -4 * math.sin(a), 30.0],
                    [4 * math.sin(a), 4 * math.cos(a), 5.0], [0, 0, 1]])
    s = rng.uniform(-1, 1, (1, 2, 14, 18)).astype(np.float32)
    got = ctx.unary_maps(s, Tig, 64, 72, interpolate=True)
    for r in range(2):
        want = orc.clip_log(orc.transform_grid(s[0, r], (64, 72), Tig, 0.0, 1))
        z = want == LOG_ZERO
        assert np.array_equal(got[0, r] == LOG_ZERO, z)
        assert np.max(np.abs(got[0, r][~z] - want[~z])) <= 4e-6


@pytest.mark.parametrize("Tig", [
    synth.grid_to_image(0.75, 3.0, 2.0),                       # separable, grid step < 1 px
    np.array([[0.9 * math.cos(0.4), -0.9 * math.sin(0.4), 20.0],
              [0.9 * math.sin(0.4), 0.9 * math.cos(0.4), 4.0], [0, 0, 1]]),  # rotated, < sqrt 2
    np.array([[-1.3 * math.cos(1.1), -1.3 * math.sin(1.1), 60.0],
              [-1.3 * math.sin(1.1), 1.3 * math.cos(1.1), 30.0], [0, 0, 1]]),  # flipped
])
def test_unary_maps_direct_colliding(ctx, orc, Tig):
    """TM_DIRECT maps that send several cells to one pixel keep the
    reference's last writer (x1 outer, y1 inner loop): bit-exact cells and
    zero pattern against the oracle's transform_grid_fixed_size."""
    rng = np.random.default_rng(9)
    P, R, ny, nx, H, W = 2, 2, 41, 57, 48, 64
    s = rng.uniform(-1, 1, (P, R, ny, nx)).astype(np.float32)
    s[:, :, ::7, ::5] = 0.0  # NO_CLASS_VALUE cells never write
    got = ctx.unary_maps(s, Tig, H, W, interpolate=False)
    for p in range(P):
        for r in range(R):
            want = orc.clip_log(orc.transform_grid(s[p, r], (H, W), Tig, 0.0, 2))
            z = want == LOG_ZERO
            assert np.array_equal(got[p, r] == LOG_ZERO, z)
            d = np.abs(got[p, r][~z] - want[~z])
            assert np.all(d <= 4e-7 * np.maximum(1.0, np.abs(want[~z])))
            assert (~z).sum() > 200


# ---------------------------------------------------------------- messages
@pytest.mark.parametrize("R", [24, 12, 8, 48])
def test_rot_joint_marginal(ctx, orc, R):
    rng = np.random.default_rng(10 + R)
    H, W = 50, 70
    child = synth.random_log_unary(rng, 1, R, H, W, zero_frac=0.02)[0]
    step = synth.rot_step_rad(R)
    for k, rs, oc, op, sig in [(0, 1.3, (4.2, -3.1), (-2.6, 5.7), (1.5, 2.5)),
                               (2, 2.9, (-9.5, 7.25), (6.0, -4.5), (3.0, 1.2)),
                               (-1, 0.0, (0.5, 0.5), (-0.5, 0.5), (0.7, 0.9))]:
        e = orc.make_exp(R=R)
        args = (np.array(oc), np.array(op), np.diag([sig[0] ** 2, sig[1] ** 2]), k * step, rs * step)
        want = orc.rot_joint_marginal(e, child, *args)
        got = ctx.rot_joint_marginal(_pa_exp(R), child, *args)
        oob = want == LOG_ZERO
        assert np.array_equal(got[oob], want[oob])
        assert maxnorm_err(got, want) <= 1e-5
        want64 = orc.rot_joint_marginal(e, child.astype(np.float64), *args, f64=True)
        assert maxnorm_err(got, want64) <= 1e-4


@pytest.mark.parametrize("R,W", [(48, 1100), (16, 1500)])
def test_rot_joint_marginal_wide_rows(ctx, orc, R, W):
    """Rows too wide for one shared-memory row (wide x kernels, sigma up to
    24 px as in the 1024x1024 workload): the row pass runs in column chunks
    with a halo and must equal the oracle as the single-chunk path does."""
    rng = np.random.default_rng(77 + R)
    H = 20
    child = synth.random_log_unary(rng, 1, R, H, W, zero_frac=0.01)[0]
    step = synth.rot_step_rad(R)
    for k, rs, oc, op, sig in [(1, 1.7, (31.0, -12.5), (-20.25, 7.5), (24.0, 3.0)),
                               (0, 2.2, (-55.5, 4.0), (40.0, -2.0), (9.0, 1.5))]:
        e = orc.make_exp(R=R)
        args = (np.array(oc), np.array(op), np.diag([sig[0] ** 2, sig[1] ** 2]), k * step,
                rs * step)
        want = orc.rot_joint_marginal(e, child, *args)
        got = ctx.rot_joint_marginal(_pa_exp(R), child, *args)
        oob = want == LOG_ZERO
        assert np.array_equal(got[oob], want[oob])
        assert maxnorm_err(got, want) <= 1e-5


def _pa_exp(R, **kw):
    import partapp_gb300

    return partapp_gb300.exp_param(R=R, **kw)


def flat_of(best, R, H, W):
    r, x, y = int(best[2]), int(best[4]), int(best[5])
    return (r * H + y) * W + x


def compare_ps(got, want, want64=None, check_argmax=True):
    P = want["log_marg"].shape[0]
    for p in range(P):
        err = maxnorm_err(got["log_marg"][p], want["log_marg"][p])
        assert err <= TOL_F32, (p, err)
        if want64 is not None:
            assert maxnorm_err(got["log_marg"][p], want64["log_marg"][p]) <= TOL_F64
    if check_argmax:
        _, R, H, W = want["log_marg"].shape
        flips = 0
        for p in range(P):
            g, w = got["best_conf"][p], want["best_conf"][p]
            if (g[2], g[4], g[5]) == (w[2], w[4], w[5]):
                assert abs(g[6] - w[6]) <= 1e-5 * max(1.0, abs(w[6])), (p, g[6], w[6])
                continue
            assert want64 is not None, f"part {p}: argmax {g[[2, 4, 5]]} != {w[[2, 4, 5]]}"
            m = want64["log_marg"][p].reshape(-1)
            gap = abs(m[flat_of(g, R, H, W)] - m[flat_of(w, R, H, W)])
            assert gap <= 1e-4, f"part {p}: argmax moved off a non-tied maximum (gap {gap})"
            flips += 1
        assert flips <= 1, f"{flips} near-tie argmax flips"


def oracle64(orc, e, tree, log_unary):
    return orc.ps_infer(e, tree, np.asarray(log_unary, dtype=np.float64), f64=True,
                        want_hyps=False)


@pytest.mark.parametrize("R", [24, 16])
def test_ps_infer_matches_oracle(ctx, orc, R):
    rng = np.random.default_rng(20 + R)
    H, W = 60, 80
    tree = small_tree(rng, R)
    u = synth.random_log_unary(rng, 10, R, H, W)
    e = orc.make_exp(R=R)
    want = orc.ps_infer(e, tree, u)
    want64 = orc.ps_infer(e, tree, u.astype(np.float64), f64=True)
    got = ctx.compute_root_posterior_rot(_pa_exp(R), tree, u)
    compare_ps(got, want, want64)
    assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32
    # FP64 log-partition of every marginal
    for p in range(10):
        m = want64["log_marg"][p]
        lz = m.max() + math.log(np.exp(m - m.max()).sum())
        assert abs(got["log_z"][p] - lz) <= 1e-3 * max(1.0, abs(lz))


@pytest.mark.parametrize("R,H,W,case", [(24, 60, 80, "spread"), (12, 96, 128, "zeros"),
                                        (16, 64, 96, "flat")])
def test_log_z_is_fp64_logsumexp_of_the_device_map(ctx, R, H, W, case):
    """The log-partition reduction on its own: log Z of every part against an
    FP64 log-sum-exp (numpy, pairwise summation) of the same device marginal,
    |d| <= 1e-12 * max(1, |log Z|).  "flat" keeps nearly every cell within a
    few nats of the maximum, "zeros" plants LOG_ZERO cells."""
    rng = np.random.default_rng(600 + R)
    tree = small_tree(rng, R)
    if case == "flat":
        u = np.log(rng.uniform(0.95, 1.0, (10, R, H, W))).astype(np.float32)
    else:
        u = synth.random_log_unary(rng, 10, R, H, W, 0.2 if case == "zeros" else 0.0)
    got = ctx.compute_root_posterior_rot(_pa_exp(R), tree, u)
    for p in range(10):
        m = np.asarray(got["log_marg"][p], dtype=np.float64)
        M = m.max()
        lz = M + math.log(np.exp(m - M).sum())
        assert abs(got["log_z"][p] - lz) <= 1e-12 * max(1.0, abs(lz)), (p, got["log_z"][p], lz)


@pytest.mark.parametrize("variant", ["flip", "upright", "strip", "no_pairwise", "interp_direct"])
def test_ps_variants(ctx, orc, variant):
    rng = np.random.default_rng(sum(map(ord, variant)))
    R, H, W = 24, 48, 64
    tree = small_tree(rng, R)
    u = synth.random_log_unary(rng, 10, R, H, W)
    kw, flip = {}, False
    if variant == "flip":
        flip = True
    if variant == "upright":
        tree["is_upright"][[8, 9]] = 1
    if variant == "strip":
        kw["strip"] = 0.1
    if variant == "no_pairwise":
        kw["use_pairwise"] = False
    e = orc.make_exp(R=R, **kw)
    t_or = dict(tree)
    if flip:  # loadJoints mirroring, objectdetect_aux.cpp:98-116
        t_or = dict(tree, offset_c=tree["offset_c"] * [-1, 1], offset_p=tree["offset_p"] * [-1, 1],
                    rot_mean=-tree["rot_mean"])
    want = orc.ps_infer(e, t_or, u)
    got = ctx.compute_root_posterior_rot(_pa_exp(R, **kw), tree, u, flip=flip)
    compare_ps(got, want, oracle64(orc, e, t_or, u))
    if kw.get("use_pairwise", True):
        assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32


# ------------------------------------------------------- full covariance
@pytest.mark.parametrize("R,sparse", [(24, False), (12, False), (24, True), (12, True)])
def test_rot_joint_marginal_full_covariance(ctx, orc, R, sparse):
    """Non-diagonal C: gaussFilter2dOffset (rotation into the eigenbasis,
    eigen-axis filter, rotation back) against the oracle; sparse = bIsSparse,
    the TM_DIRECT forward rotation (multi_array_filter.hpp:351-355)."""
    rng = np.random.default_rng(40 + R + 7 * int(sparse))
    H, W = 50, 70
    child = synth.random_log_unary(rng, 1, R, H, W, zero_frac=0.02)[0]
    step = synth.rot_step_rad(R)
    for k, rs, oc, op, Cm in [(1, 1.5, (4.2, -3.1), (-2.6, 5.7), [[4.0, 1.5], [1.5, 2.0]]),
                              (0, 0.0, (-6.0, 2.5), (3.0, -1.0), [[1.0, -0.6], [-0.6, 6.25]]),
                              (-2, 2.5, (0.5, 9.0), (1.5, -8.0), [[30.0, 12.0], [12.0, 9.0]])]:
        e = orc.make_exp(R=R, sparse=sparse)
        args = (np.array(oc), np.array(op), np.array(Cm), k * step, rs * step)
        want = orc.rot_joint_marginal(e, child, *args)
        got = ctx.rot_joint_marginal(_pa_exp(R), child, *args, is_sparse=sparse)
        oob = want == LOG_ZERO
        assert np.array_equal(got[oob], want[oob])
        assert maxnorm_err(got, want) <= 1e-5
        want64 = orc.rot_joint_marginal(e, child.astype(np.float64), *args, f64=True)
        assert maxnorm_err(got, want64) <= 1e-4
        if sparse:  # the two forward rotations give different messages
            dense = orc.rot_joint_marginal(orc.make_exp(R=R), child, *args)
            assert maxnorm_err(dense, want) > 1e-3


@pytest.mark.parametrize("flip,sparse", [(False, False), (True, False), (False, True),
                                         (True, True)])
def test_ps_full_covariance(ctx, orc, flip, sparse):
    """A tree whose joints mix diagonal and full covariances (learned joints
    carry correlations, objectdetect_learnparam.cpp:465)."""
    rng = np.random.default_rng(31 + int(flip) + 2 * int(sparse))
    R, H, W = 16, 44, 60
    tree = small_tree(rng, R)
    for j, rho in ((1, 0.5), (4, -0.35), (6, 0.2), (8, -0.6)):
        c = tree["C"][j]
        off = rho * math.sqrt(c[0] * c[3])
        tree["C"][j] = [c[0], off, off, c[3]]
    u = synth.random_log_unary(rng, 10, R, H, W)
    e = orc.make_exp(R=R, sparse=sparse)
    t_or = dict(tree)
    if flip:  # loadJoints mirroring: x of the offsets, the off-diagonal of C
        t_or = dict(tree, offset_c=tree["offset_c"] * [-1, 1], offset_p=tree["offset_p"] * [-1, 1],
                    C=tree["C"] * [1, -1, -1, 1], rot_mean=-tree["rot_mean"])
    want = orc.ps_infer(e, t_or, u)
    got = ctx.compute_root_posterior_rot(_pa_exp(R), tree, u, flip=flip, is_sparse=sparse)
    compare_ps(got, want, oracle64(orc, e, t_or, u))
    assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32


# ---------------------------------------------------------- --find_obj path
@pytest.mark.parametrize("interpolate", [True, False])
def test_find_obj_pipeline(ctx, orc, interpolate):
    img = synth.make_image(7, R=12, H=64, W=96, n_stumps=120, D=96, offset_range=(3, 10),
                           sigma_range=(1, 3))
    e = orc.make_exp(R=12)
    want = orc.find_obj(e, img["tree"], img["models"], img["desc"], img["Tig"], 64, 96,
                        interpolate=interpolate)
    cls = ctx.classifiers(img["models"])
    got = ctx.find_obj(_pa_exp(12, interpolate=interpolate), img["tree"], cls, img["desc"],
                       img["Tig"], 64, 96)
    compare_ps(got, want, oracle64(orc, e, img["tree"], want["log_unary"]))
    assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32


def test_find_obj_full_covariance(ctx, orc):
    """--find_obj with correlated joints: findObjectImageRotJoints passes
    bIsSparse = true (objectdetect_findrot.cpp:740), so the upward messages of
    the full-covariance joints take the TM_DIRECT forward rotation."""
    img = synth.make_image(17, R=12, H=64, W=96, n_stumps=120, D=96, offset_range=(3, 10),
                           sigma_range=(1.5, 3))
    tree = img["tree"]
    for j, rho in ((0, 0.45), (3, -0.5), (5, 0.3)):
        c = tree["C"][j]
        off = rho * math.sqrt(c[0] * c[3])
        tree["C"][j] = [c[0], off, off, c[3]]
    e = orc.make_exp(R=12)
    want = orc.find_obj(e, tree, img["models"], img["desc"], img["Tig"], 64, 96)
    cls = ctx.classifiers(img["models"])
    got = ctx.find_obj(_pa_exp(12), tree, cls, img["desc"], img["Tig"], 64, 96)
    compare_ps(got, want, oracle64(orc, orc.make_exp(R=12, sparse=True), tree, want["log_unary"]))
    assert maxnorm_err(got["root_post"], want["root_post"]) <= TOL_F32
    # the same unaries through pa_ps_infer with bIsSparse = true agree
    ps = ctx.compute_root_posterior_rot(_pa_exp(12), tree, want["log_unary"], is_sparse=True)
    assert maxnorm_err(ps["log_marg"], got["log_marg"]) <= 1e-6


def test_find_obj_batch_device_resident(ctx, orc):
    import torch

    imgs = [synth.make_image(100 + i, R=12, H=48, W=64, n_stumps=60, D=96, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i in range(3)]
    models = imgs[0]["models"]
    e = orc.make_exp(R=12)
    desc = torch.from_numpy(np.stack([im["desc"] for im in imgs])).cuda()
    cls = ctx.classifiers(models)
    got = ctx.find_obj_batch(_pa_exp(12), [im["tree"] for im in imgs], cls, desc, imgs[0]["Tig"],
                             48, 64, want_marg=True, want_root=True)
    for i, im in enumerate(imgs):
        want = orc.find_obj(e, im["tree"], models, im["desc"], im["Tig"], 48, 64)
        g = dict(got[i], log_marg=got[i]["log_marg"].cpu().numpy())
        compare_ps(g, want, oracle64(orc, e, im["tree"], want["log_unary"]))
        assert maxnorm_err(got[i]["root_post"].cpu().numpy(), want["root_post"]) <= TOL_F32


def test_find_obj_scales(ctx, orc):
    """pa_find_obj_scales: with one scale it is pa_find_obj bit for bit; with
    two (grids of stride 4 and 5, their own Tig) it matches the oracle's
    per-scale unaries followed by computeRootPosteriorRot over both scales."""
    import torch

    R, H, W = 8, 48, 64
    img = synth.make_image(201, R=R, H=H, W=W, n_stumps=60, D=96, offset_range=(3, 8),
                           sigma_range=(1, 2.5))
    tree, models = img["tree"], img["models"]
    rng = np.random.default_rng(202)
    descs = [img["desc"], synth.make_descriptors(rng, R, 9, 12, 96)]
    tigs = [img["Tig"], synth.grid_to_image(5.0, 1.0, 2.0)]
    cls = ctx.classifiers(models)
    one = ctx.find_obj_scales(_pa_exp(R), tree, cls, descs[:1], tigs[:1], H, W)
    ref = ctx.find_obj(_pa_exp(R), tree, cls, descs[0], tigs[0], H, W)
    assert np.array_equal(one["log_marg"], ref["log_marg"])
    assert np.array_equal(one["best_conf"], ref["best_conf"])
    assert np.array_equal(one["root_post"], ref["root_post"])
    kw = dict(n_scales=2, scale_range=(0.8, 1.25))
    lu = np.stack([orc.find_obj(orc.make_exp(R=R), tree, models, d, T, H, W)["log_unary"]
                   for d, T in zip(descs, tigs)], axis=1)
    want = orc.ps_infer(orc.make_exp(R=R, sparse=True, **kw), tree, lu)
    for dev in (False, True):
        ds = [torch.from_numpy(d).cuda() for d in descs] if dev else descs
        got = ctx.find_obj_scales(_pa_exp(R, **kw), tree, cls, ds, tigs, H, W)
        marg = got["log_marg"].cpu().numpy() if dev else got["log_marg"]
        assert marg.shape == (10, 2, R, H, W)
        for p in range(10):
            for sc in range(2):
                assert maxnorm_err(marg[p, sc], want["log_marg"][p, sc]) <= TOL_F32, (p, sc)
        assert np.array_equal(got["best_conf"][:, [0, 2, 4, 5]], want["best_conf"][:, [0, 2, 4, 5]])
        # the same unaries through pa_ps_infer give the same marginals
        ps = ctx.compute_root_posterior_rot(_pa_exp(R, **kw), tree, lu, is_sparse=True)
        assert maxnorm_err(ps["log_marg"], marg) <= 1e-6


def test_find_obj_batch_host_ring_matches_device(ctx):
    """Host descriptors go through the copy/compute ring one image at a time;
    results (and the strided score-grid output) must equal the batched
    device-resident call bit for bit."""
    import torch

    imgs = [synth.make_image(300 + i, R=12, H=48, W=64, n_stumps=60, D=96, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i in range(4)]
    models = imgs[0]["models"]
    cls = ctx.classifiers(models)
    desc = np.stack([im["desc"] for im in imgs])
    trees = [im["tree"] for im in imgs]
    sc_host = np.zeros((10, 4 * 12, 12, 16), dtype=np.float32)
    host = ctx.find_obj_batch(_pa_exp(12), trees, cls, desc, imgs[0]["Tig"], 48, 64,
                              want_marg=True, want_root=True, scores_out=sc_host)
    sc_dev = torch.zeros((10, 4 * 12, 12, 16), dtype=torch.float32, device="cuda")
    dev = ctx.find_obj_batch(_pa_exp(12), trees, cls, torch.from_numpy(desc).cuda(),
                             imgs[0]["Tig"], 48, 64, want_marg=True, want_root=True,
                             scores_out=sc_dev)
    assert np.array_equal(sc_host, sc_dev.cpu().numpy())
    for h, d in zip(host, dev):
        assert np.array_equal(h["best_conf"], d["best_conf"])
        assert np.array_equal(h["log_marg"], d["log_marg"].cpu().numpy())
        assert np.array_equal(h["root_post"], d["root_post"].cpu().numpy())
        assert np.array_equal(h["log_z"], d["log_z"])


def test_full_size_320x240_one_image(ctx, orc):
    """The plain single-image workload: 320x240, 24 rotations, 10 parts x 500
    stumps over 960-dim descriptors at stride 4, bilinear upsampling."""
    img = synth.make_image(2024)
    e = orc.make_exp(R=24)
    want = orc.find_obj(e, img["tree"], img["models"], img["desc"], img["Tig"], 240, 320)
    cls = ctx.classifiers(img["models"])
    got = ctx.find_obj(_pa_exp(24), img["tree"], cls, img["desc"], img["Tig"], 240, 320)
    compare_ps(got, want, oracle64(orc, e, img["tree"], want["log_unary"]))


# ------------------------------------------------------------ multi-scale
@pytest.mark.parametrize("mem", ["host", "device"])
def test_ps_multi_scale(ctx, orc, mem):
    """num_scale_steps = 3: one pass per scale at scale_from_index(s)
    (objectdetect_findrot.cpp:503-678); maps [P][S][R][H][W], root posterior
    [S][H][W], argmax and part maxima of the last scale, root maxima over the
    scale stack."""
    import torch

    rng = np.random.default_rng(91)
    R, H, W, S = 12, 40, 56, 3
    tree = small_tree(rng, R)
    u = synth.random_log_unary(rng, 10 * S, R, H, W).reshape(10, S, R, H, W)
    kw = dict(n_scales=S, scale_range=(0.5, 2.0))
    e = orc.make_exp(R=R, max_local_max=200, **kw)
    want = orc.ps_infer(e, tree, u)
    pe = _pa_exp(R, local_max=200, **kw)
    uin = torch.from_numpy(u).cuda() if mem == "device" else u
    got = ctx.compute_root_posterior_rot(pe, tree, uin)
    if mem == "device":
        got["log_marg"] = got["log_marg"].cpu().numpy()
        got["root_post"] = got["root_post"].cpu().numpy()
    assert got["log_marg"].shape == (10, S, R, H, W) and got["root_post"].shape == (S, H, W)
    want64 = orc.ps_infer(e, tree, u.astype(np.float64), f64=True, want_hyps=False)
    for s in range(S):
        last = dict(log_marg=want["log_marg"][:, s], best_conf=want["best_conf"])
        g = dict(log_marg=got["log_marg"][:, s], best_conf=got["best_conf"])
        compare_ps(g, last, dict(log_marg=want64["log_marg"][:, s]), check_argmax=(s == S - 1))
        assert maxnorm_err(got["root_post"][s], want["root_post"][s]) <= TOL_F32
    assert (got["best_conf"][:, 0] == S - 1).all()
    assert np.array_equal(got["best_conf"][:, 1], want["best_conf"][:, 1])
    assert got["log_z"].shape == (S, 10)
    for p in range(10):
        g = {tuple(r) for r in got["part_hyps"][p, :20, 2:6:1][:, [0, 2, 3]].tolist()}
        w = {tuple(r) for r in want["part_hyps"][p, :20, 2:6:1][:, [0, 2, 3]].tolist()}
        assert len(g & w) >= 18, p
    assert (got["part_hyps"][:, :, 0] == 0).all()
    assert abs(int(got["n_root_hyps"][0]) - want["n_root_hyps"]) <= 2
    g = {tuple(r) for r in got["root_hyps"][:20, 0:3].tolist()}
    w = {tuple(r) for r in want["root_hyps"][:20, 0:3].tolist()}
    assert len(g & w) >= 18
    # maxima on every scale, in the oracle's proportions
    ng, nw = int(got["n_root_hyps"][0]), want["n_root_hyps"]
    hg = np.unique(got["root_hyps"][:ng, 0], return_counts=True)
    hw = np.unique(want["root_hyps"][:nw, 0], return_counts=True)
    assert len(hw[0]) == S and np.array_equal(hg[0], hw[0])
    assert np.abs(hg[1] - hw[1]).max() <= 2


def test_ps_multi_scale_without_pairwise(ctx, orc):
    """use_pairwise off: getMaxStates reads scale 0 only (:73-110)."""
    rng = np.random.default_rng(92)
    R, H, W, S = 6, 30, 40, 2
    tree = small_tree(rng, R)
    u = np.floor(rng.uniform(0, 6, (10, S, R, H, W))).astype(np.float32) - 3.0
    kw = dict(n_scales=S, scale_range=(0.5, 1.5))
    want = orc.ps_infer(orc.make_exp(R=R, use_pairwise=False, max_local_max=60, **kw), tree, u)
    got = ctx.compute_root_posterior_rot(_pa_exp(R, use_pairwise=False, local_max=60, **kw),
                                         tree, u)
    assert np.array_equal(got["log_marg"], want["log_marg"])
    assert np.array_equal(got["best_conf"], want["best_conf"])
    assert np.array_equal(got["n_part_hyps"], want["n_part_hyps"])
    for p in range(10):
        n = int(want["n_part_hyps"][p])
        assert np.array_equal(got["part_hyps"][p, :n], want["part_hyps"][p, :n]), p


# ----------------------------------------------------------- local maxima
@pytest.mark.parametrize("K,levels", [(50, 9), (1000, 2)])
def test_local_max_exact_on_unaries(ctx, orc, K, levels):
    """findLocalMax (objectdetect_aux.cpp:193-264) on maps with many ties and
    plateaus: with use_pairwise off the marginals are the masked unaries, so
    the GPU lists must equal the oracle's exactly -- the K largest values in
    stable order when there are more than K maxima (K=50), and enumeration
    order (rotation, then x, then y) otherwise (few maxima, K=1000)."""
    rng = np.random.default_rng(K)
    R, H, W = 6, 40, 52
    if levels > 2:  # noisy, heavily tied: thousands of maxima
        u = np.floor(rng.uniform(0, levels, (10, R, H, W))).astype(np.float32) - 5.0
    else:  # a few quantised bumps: few maxima, including tied plateaus
        r, y, x = np.meshgrid(np.arange(R), np.arange(H), np.arange(W), indexing="ij")
        u = np.zeros((10, R, H, W), dtype=np.float32)
        for p in range(10):
            for _ in range(3):
                cr, cy, cx = rng.integers(0, R), rng.uniform(0, H), rng.uniform(0, W)
                u[p] += np.exp(-((y - cy) ** 2 + (x - cx) ** 2) / 60.0 - (r - cr) ** 2 / 4.0)
        u = np.floor(u * 4.0).astype(np.float32)
    tree = small_tree(rng, R)
    e = orc.make_exp(R=R, use_pairwise=False, max_local_max=K)
    want = orc.ps_infer(e, tree, u)
    got = ctx.compute_root_posterior_rot(_pa_exp(R, use_pairwise=False, local_max=K), tree, u)
    assert np.array_equal(got["n_part_hyps"], want["n_part_hyps"])
    for p in range(10):
        n = int(want["n_part_hyps"][p])
        assert np.array_equal(got["part_hyps"][p, :n], want["part_hyps"][p, :n]), p
    if levels == 2:
        assert (want["n_part_hyps"] < K).any()  # the enumeration-order branch ran
    else:
        assert (want["n_part_hyps"] == K).all()


def test_local_max_with_pairwise_overlaps_oracle(ctx, orc):
    rng = np.random.default_rng(44)
    R, H, W = 12, 48, 64
    tree = small_tree(rng, R)
    u = synth.random_log_unary(rng, 10, R, H, W)
    e = orc.make_exp(R=R, max_local_max=200)
    want = orc.ps_infer(e, tree, u)
    got = ctx.compute_root_posterior_rot(_pa_exp(R, local_max=200), tree, u)
    for p in range(10):
        g = {tuple(r) for r in got["part_hyps"][p, :20, 2:6:1][:, [0, 2, 3]].tolist()}
        w = {tuple(r) for r in want["part_hyps"][p, :20, 2:6:1][:, [0, 2, 3]].tolist()}
        assert len(g & w) >= 18, p
    assert abs(int(got["n_root_hyps"][0]) - want["n_root_hyps"]) <= 2
    g = {tuple(r) for r in got["root_hyps"][:20, 1:3].tolist()}
    w = {tuple(r) for r in want["root_hyps"][:20, 1:3].tolist()}
    assert len(g & w) >= 18


# ------------------------------------------------------------------ errors
def test_errors_are_statuses(ctx, pa):
    rng = np.random.default_rng(5)
    R = 12
    u = synth.random_log_unary(rng, 10, R, 20, 24)
    tree = small_tree(rng, R)
    for c01, c10 in ((0.5, 0.25), (40.0, 40.0)):  # not symmetric; not positive definite
        bad = dict(tree, C=tree["C"].copy())
        bad["C"][0, 1], bad["C"][0, 2] = c01, c10
        with pytest.raises(pa.PaError) as ei:
            ctx.compute_root_posterior_rot(_pa_exp(R), bad, u)
        assert ei.value.status == pa.PA_ERR_INVALID
    two = dict(tree, parent=tree["parent"].copy())
    two["parent"][3] = 1  # part 1 (an upper leg) now has two children
    with pytest.raises(pa.PaError) as ei:
        ctx.compute_root_posterior_rot(_pa_exp(R), two, u)
    assert ei.value.status == pa.PA_ERR_UNSUPPORTED
    with pytest.raises(pa.PaError) as ei:
        ctx.compute_root_posterior_rot(_pa_exp(1), tree, u[:, :1])
    assert ei.value.status == pa.PA_ERR_INVALID
    # several scales with min == max: value_from_index asserts (partapp_aux.hpp:48-52)
    with pytest.raises(pa.PaError) as ei:
        ctx.compute_root_posterior_rot(_pa_exp(R, n_scales=2), tree, np.stack([u, u], axis=1))
    assert ei.value.status == pa.PA_ERR_INVALID
    # the --find_obj entries score one scale of descriptors
    img = synth.make_image(3, R=R, H=32, W=48, n_stumps=20, D=32)
    cls = ctx.classifiers(img["models"])
    with pytest.raises(pa.PaError) as ei:
        ctx.find_obj(_pa_exp(R, n_scales=2, scale_range=(0.5, 1.5)), img["tree"], cls,
                     img["desc"], img["Tig"], 32, 48)
    assert ei.value.status == pa.PA_ERR_UNSUPPORTED


# ------------------------------------------------------- uneven batches
@pytest.mark.parametrize("device", [False, True])
def test_find_obj_multi_uneven_sizes(ctx, orc, device):
    """Images of different sizes and rotation counts in one call: grouped
    images run as a batch and must equal one-image calls bit for bit; every
    image matches the oracle."""
    import torch

    shapes = [(12, 48, 64), (12, 48, 64), (12, 40, 56), (16, 48, 64), (8, 32, 48), (12, 48, 64)]
    imgs = [synth.make_image(700 + i, R=R, H=H, W=W, n_stumps=60, D=96, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i, (R, H, W) in enumerate(shapes)]
    models = imgs[0]["models"]
    cls = ctx.classifiers(models)
    todev = (lambda a: torch.from_numpy(a).cuda()) if device else (lambda a: a)
    batch = [dict(exp=_pa_exp(im["R"]), tree=im["tree"], desc=todev(im["desc"]), Tig=im["Tig"],
                  H=im["H"], W=im["W"]) for im in imgs]
    got = ctx.find_obj_multi(batch, cls, want_marg=True)
    for i, im in enumerate(imgs):
        one = ctx.find_obj(_pa_exp(im["R"]), im["tree"], cls, todev(im["desc"]), im["Tig"],
                           im["H"], im["W"])
        assert np.array_equal(got[i]["best_conf"], one["best_conf"]), i
        assert np.array_equal(np.asarray(got[i]["log_z"]), np.asarray(one["log_z"])), i
        gm = got[i]["log_marg"]
        om = one["log_marg"]
        if device:
            gm, om = gm.cpu().numpy(), om.cpu().numpy()
        assert np.array_equal(gm, om), i
        e = orc.make_exp(R=im["R"])
        want = orc.find_obj(e, im["tree"], models, im["desc"], im["Tig"], im["H"], im["W"])
        compare_ps(dict(got[i], log_marg=gm), want,
                   oracle64(orc, e, im["tree"], want["log_unary"]))
