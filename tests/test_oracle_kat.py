"""Known-answer tests that pin the CPU oracle.

The reference ships no golden vectors for this path, so each test here builds
an input whose correct output follows analytically from the reference's
definition (cited per test) and checks the oracle against a numpy derivation
written independently of oracle.cpp.
"""
import math

import numpy as np
import pytest

LOG_ZERO = np.float32(-1e6)


def gauss_taps(sigma):
    """boost_math.cpp:104-117, unnormalised."""
    k = int(math.floor(3 * sigma + 0.5))
    f = np.array([math.exp(-(i * i) / (2 * sigma * sigma)) for i in range(-k, k + 1)])
    f[k] = 1.0
    return f


def rot_value(R, r):
    """partapp_aux.hpp:45-58 with min=-180, max=180."""
    return -180.0 + (360.0 / R) * (0.5 + r)


def joint_shift(R, r, o, scale=1.0):
    """The rotated joint offset of objectdetect_findrot.cpp:348-351."""
    alpha = float(np.float32(rot_value(R, r) * math.pi / 180.0))
    ca, sa = math.cos(alpha), math.sin(alpha)
    return (ca * scale) * o[0] + ((-sa) * scale) * o[1], (sa * scale) * o[0] + (ca * scale) * o[1]


def test_gaussian_taps(orc):
    for sigma in (0.2, 0.9, 1.0, 2.5, 7.9, 12.0):
        np.testing.assert_allclose(orc.gaussian_filter(sigma), gauss_taps(sigma), rtol=0, atol=0)


def test_stump_tie_and_polarity(orc):
    """AdaBoost.h:147-159: (v*p < theta*p) ? alpha : -alpha.  At v == theta
    both polarities vote -alpha."""
    D = 4
    v = np.array([[0.25, 0.5, 0.75, 1.0]], dtype=np.float32)
    f = np.array([0, 1, 2, 3, 0, 2], dtype=np.int32)
    theta = np.array([0.25, 0.6, 0.75, 0.9, 0.3, 0.7], dtype=np.float32)
    p = np.array([1, 1, -1, -1, -1, 1], dtype=np.float32)
    alpha = np.array([0.5, 0.25, 0.125, 1.0, 2.0, 4.0], dtype=np.float32)
    # decisions: tie(-), 0.5<0.6(+), tie(-), 1.0>0.9(+), 0.25>0.3? no(-), 0.75<0.7? no(-)
    expect = -0.5 + 0.25 - 0.125 + 1.0 - 2.0 - 4.0
    out = orc.adaboost_eval(f, p, theta, alpha, v, normalize=False)
    assert out[0] == np.float32(expect)
    sa = orc.sum_alpha(alpha)
    assert sa == np.float32(7.875)
    outn = orc.adaboost_eval(f, p, theta, alpha, v, normalize=True)
    assert outn[0] == np.float32(np.float32(expect) / np.float32(7.875))


def test_sum_alpha_is_sequential_float(orc):
    a = np.array([1e8, 1.0, -1e8, 1.0], dtype=np.float32)
    # float: ((1e8 + 1) - 1e8) + 1 = 0 + 1 = 1
    assert orc.sum_alpha(a) == np.float32(1.0)


@pytest.mark.parametrize("R,k,rs", [(8, 0, 1.3), (8, 1, 2.0), (12, -2, 2.7), (7, 1, 1.5)])
def test_delta_message_is_analytic_gaussian(orc, R, k, rs):
    """objectdetect_findrot.cpp:292-456 on a single-cell child: the message
    is log of (rotation taps x spatial taps) around the shifted cell."""
    H, W = 40, 48
    r0, y0, x0 = 3, 21, 25
    child = np.full((R, H, W), LOG_ZERO, dtype=np.float32)
    child[r0, y0, x0] = 0.0
    oc, op = np.array([3.3, -2.6]), np.array([-1.7, 4.4])
    sx, sy = 1.6, 2.3
    step = float(np.float32(360.0) / np.float32(R)) * (math.pi / 180.0)
    rot_mean, rot_sigma = k * step, rs * step
    e = orc.make_exp(R=R)
    out = orc.rot_joint_marginal(e, child, oc, op, np.diag([sx * sx, sy * sy]), rot_mean, rot_sigma)

    # numpy derivation
    kidx = int(math.floor(-rot_mean / step + 0.5))
    rm = r0 + kidx
    dx, dy = joint_shift(R, r0, oc)
    # log_joint_10 cell that reads (y0, x0)
    xs = [x for x in range(W) if math.floor((x - dx) + 0.5) == x0]
    ys = [y for y in range(H) if math.floor((y - dy) + 0.5) == y0]
    assert len(xs) == 1 and len(ys) == 1
    x1, y1 = xs[0], ys[0]
    fr = gauss_taps(rot_sigma / step)
    if len(fr) >= R:
        c = len(fr) // 2
        L = R - 2 if R % 2 else R - 1
        fr = fr[c - L // 2: c - L // 2 + L]
    nr = (len(fr) - 1) // 2
    fx, fy = gauss_taps(sx), gauss_taps(sy)
    kx, ky = (len(fx) - 1) // 2, (len(fy) - 1) // 2
    j01 = np.full((R, H, W), -1e6)
    for r in range(R):
        d = (r - rm) % R
        wr = None
        for t in range(-nr, nr + 1):
            if (t % R) == d:
                wr = fr[t + nr]
        if wr is None:
            continue
        for y in range(max(0, y1 - ky), min(H, y1 + ky + 1)):
            for x in range(max(0, x1 - kx), min(W, x1 + kx + 1)):
                j01[r, y, x] = math.log(wr * fx[x - x1 + kx] * fy[y - y1 + ky])
    expect = np.full((R, H, W), -1e6)
    for r in range(R):
        ddx, ddy = joint_shift(R, r, op)
        for y in range(H):
            iy = math.floor((y + ddy) + 0.5)
            if not 0 <= iy < H:
                continue
            for x in range(W):
                ix = math.floor((x + ddx) + 0.5)
                if 0 <= ix < W:
                    expect[r, y, x] = j01[r, iy, ix]
    finite = expect > -1e5
    assert np.array_equal(out > -1e5, finite)
    np.testing.assert_array_equal(out[~finite], LOG_ZERO)
    np.testing.assert_allclose(out[finite], expect[finite], rtol=0, atol=2e-5)


def test_all_log_zero_child_plateau(orc):
    """A child that is LOG_ZERO everywhere has in_M = LOG_ZERO, so every
    exp() is 1 and the message is log(sum of the in-grid taps) + LOG_ZERO."""
    R, H, W = 6, 30, 36
    child = np.full((R, H, W), LOG_ZERO, dtype=np.float32)
    oc, op = np.array([2.0, 1.0]), np.array([-3.0, 2.5])
    sx, sy = 1.2, 0.8
    step = float(np.float32(360.0) / np.float32(R)) * (math.pi / 180.0)
    e = orc.make_exp(R=R)
    out = orc.rot_joint_marginal(e, child, oc, op, np.diag([sx * sx, sy * sy]), 0.0, 1.0 * step)
    fr = gauss_taps(1.0)
    fx, fy = gauss_taps(sx), gauss_taps(sy)
    kx, ky = (len(fx) - 1) // 2, (len(fy) - 1) // 2
    Sx = np.array([fx[max(0, kx - x):kx + (W - x)].sum() for x in range(W)])
    Sy = np.array([fy[max(0, ky - y):ky + (H - y)].sum() for y in range(H)])
    base = np.log(fr.sum() * Sy[:, None] * Sx[None, :]) - 1e6
    for r in range(R):
        ddx, ddy = joint_shift(R, r, op)
        for y in range(H):
            iy = math.floor((y + ddy) + 0.5)
            for x in range(W):
                ix = math.floor((x + ddx) + 0.5)
                if 0 <= iy < H and 0 <= ix < W:
                    assert abs(float(out[r, y, x]) - base[iy, ix]) <= 0.0625
                else:
                    assert out[r, y, x] == LOG_ZERO


def test_rotation_tap_clipping(orc):
    """objectdetect_findrot.cpp:385-399: a rotation kernel longer than R is
    clipped to R-1 (even R) or R-2 (odd R) taps, centred."""
    for R in (4, 5, 6):
        H, W = 5, 5
        child = np.full((R, H, W), LOG_ZERO, dtype=np.float32)
        child[0, 2, 2] = 0.0
        step = float(np.float32(360.0) / np.float32(R)) * (math.pi / 180.0)
        e = orc.make_exp(R=R)
        # tiny spatial sigma: 1 tap; zero offsets: no shift
        out = orc.rot_joint_marginal(e, child, np.zeros(2), np.zeros(2), np.diag([0.01, 0.01]), 0.0,
                                     5.0 * step)
        col = out[:, 2, 2]
        L = R - 2 if R % 2 else R - 1
        reached = np.sum(col > -1e5)
        assert reached == L


def test_bilinear_exact_hit_and_edge(orc):
    """multi_array_transform.hpp:210-231: exact hits copy the cell, the last
    grid row/column is not interpolated (stays at the default)."""
    g = np.arange(12, dtype=np.float32).reshape(3, 4) + 1
    T = np.array([[2.0, 0, 0], [0, 2.0, 0], [0, 0, 1]])
    out = orc.transform_grid(g, (6, 8), T, 0.0, 1)
    for y in range(6):
        for x in range(8):
            gx, gy = x / 2.0, y / 2.0
            ix, iy = int(math.floor(gx)), int(math.floor(gy))
            a, b = np.float32(gx - ix), np.float32(gy - iy)
            if a < 1.1920929e-06 and b < 1.1920929e-06:
                assert out[y, x] == g[iy, ix]
            elif ix < 3 and iy < 2:
                v = ((1 - b) * (1 - a) * g[iy, ix] + (1 - b) * a * g[iy, ix + 1]
                     + b * (1 - a) * g[iy + 1, ix] + b * a * g[iy + 1, ix + 1])
                assert out[y, x] == np.float32(v)
            else:
                assert out[y, x] == 0.0
    # direct: forward-mapped cells only
    outd = orc.transform_grid(g, (6, 8), T, 0.0, 2)
    assert np.count_nonzero(outd) == 12
    assert outd[4, 6] == g[2, 3]


def test_direct_transform_last_writer_wins(orc):
    """TM_DIRECT (multi_array_transform.hpp:173-193) loops x1 outer, y1 inner and
    writes every cell != default: where a half-pixel grid puts several cells on
    one pixel, the last of them in that loop order stays."""
    g = np.arange(1, 1 + 4 * 5, dtype=np.float32).reshape(4, 5)  # [ny][nx], no zeros
    T = np.array([[0.5, 0.0, 0.0], [0.0, 0.5, 0.0], [0, 0, 1]])
    out = orc.transform_grid(g, (3, 3), T, 0.0, 2)
    want = np.zeros((3, 3), np.float32)
    for x1 in range(5):
        for y1 in range(4):
            x3, y3 = math.floor(0.5 * x1 + 0.5), math.floor(0.5 * y1 + 0.5)
            if x3 < 3 and y3 < 3:
                want[y3, x3] = g[y1, x1]
    assert np.array_equal(out, want)
    assert out[1, 1] == g[2, 2]  # cells (1, 1), (1, 2), (2, 1), (2, 2) land on (1, 1)
    g[2, 2] = 0.0  # a default cell writes nothing: the previous writer stays
    out = orc.transform_grid(g, (3, 3), T, 0.0, 2)
    assert out[1, 1] == g[1, 2]


def test_clip_log(orc):
    g = np.array([-0.5, 0.0, 0.25, 1.0], dtype=np.float32)
    out = orc.clip_log(g)
    assert out[0] == np.float32(math.log(np.float32(1e-4)))
    assert out[1] == LOG_ZERO
    assert out[2] == np.float32(math.log(0.25))
    assert out[3] == 0.0


def test_local_max_rules_and_ties(orc):
    """objectdetect_aux.cpp:193-264: a cell is a maximum unless a 3x3
    neighbour is strictly greater and the adjacent scale (rotation) is
    strictly smaller; plateaus are all maxima; enumeration is x-major."""
    g = np.zeros((2, 4, 5), dtype=np.float32)
    g[0, 1, 1] = 5.0
    g[1, 1, 1] = 5.0  # equal across rotations: neither is a maximum
    g[0, 2, 3] = 3.0
    g[1, 3, 4] = 4.0
    lm = orc.find_local_max(g, 100)
    coords = [(int(s), int(x), int(y)) for s, x, y, _ in lm]
    assert (0, 1, 1) not in coords and (1, 1, 1) not in coords
    assert (0, 3, 2) in coords and (1, 4, 3) in coords
    top = orc.find_local_max(g, 1)
    assert (int(top[0][1]), int(top[0][2])) == (4, 3)


def test_argmax_first_maximum(orc):
    """objectdetect_findrot.cpp:261-277: the first strict maximum in flat
    [R][H][W] order wins ties."""
    R, H, W = 4, 6, 7
    e = orc.make_exp(R=R, use_pairwise=False, max_local_max=10)
    tree = dict(n_parts=1, root=0, is_upright=np.zeros(1, np.int32),
                child=np.zeros(0, np.int32), parent=np.zeros(0, np.int32),
                offset_c=np.zeros((0, 2)), offset_p=np.zeros((0, 2)), C=np.zeros((0, 4)),
                rot_mean=np.zeros(0), rot_sigma=np.zeros(0))
    u = np.full((1, R, H, W), -3.0, dtype=np.float32)
    u[0, 2, 4, 1] = 1.0
    u[0, 1, 5, 6] = 1.0
    u[0, 3, 0, 0] = 1.0
    out = orc.ps_infer(e, tree, u)
    b = out["best_conf"][0]
    assert (b[2], b[4], b[5], b[6]) == (1.0, 6.0, 5.0, 1.0)
    assert b[3] == np.float32(rot_value(R, 1))


def test_upright_mask_and_root_rotations(orc):
    """objectdetect_findrot.cpp:509-523,694-716: upright parts keep |rot| <
    15 deg; an upright root keeps the rotations at +-1e-6 deg."""
    e = orc.make_exp(R=24, use_pairwise=False)
    tree = dict(n_parts=1, root=0, is_upright=np.ones(1, np.int32),
                child=np.zeros(0, np.int32), parent=np.zeros(0, np.int32),
                offset_c=np.zeros((0, 2)), offset_p=np.zeros((0, 2)), C=np.zeros((0, 4)),
                rot_mean=np.zeros(0), rot_sigma=np.zeros(0))
    u = np.zeros((1, 24, 3, 3), dtype=np.float32)
    out = orc.ps_infer(e, tree, u)
    m = out["log_marg"][0]
    kept = [r for r in range(24) if m[r, 0, 0] == 0.0]
    assert kept == [11, 12]


# -------------------------------------------------------- full covariance
def test_eig2d_known_answers(orc):
    V, E = orc.eig2d([[2.0, 1.0], [1.0, 2.0]])
    assert np.allclose(E, [1.0, 3.0])
    s = 1 / np.sqrt(2)
    assert np.allclose(V, [[-s, -s], [s, -s]])  # columns: eigenvectors of 1 and 3
    V, E = orc.eig2d([[4.0, 0.0], [0.0, 1.0]])
    assert np.allclose(E, [1.0, 4.0]) and np.allclose(V, [[0, -1], [1, 0]])
    V, E = orc.eig2d([[1.0, 0.0], [0.0, 4.0]])
    assert np.allclose(E, [1.0, 4.0]) and np.allclose(V, [[1, 0], [0, 1]])


def test_full_covariance_near_diagonal_matches_diagonal(orc):
    """C with a 1e-12 off-diagonal term takes gaussFilter2dOffset: the
    eigenbasis is the axes rotated by 90 degrees, the rotated grid is an exact
    transpose (bilinear exact hits), so away from the border the message
    equals the diagonal filter's; the rotated grid's adaptive size
    (ceil(max - min)) drops the last row and column, which the reference
    leaves at 0 (LOG_ZERO after the log)."""
    rng = np.random.default_rng(5)
    R, H, W = 4, 20, 24
    child = rng.uniform(-3.0, 0.0, (R, H, W)).astype(np.float32)
    band = 6
    child[:, :band, :] = child[:, -band:, :] = LOG_ZERO
    child[:, :, :band] = child[:, :, -band:] = LOG_ZERO
    e = orc.make_exp(R=R)
    z = np.zeros(2)
    diag = orc.rot_joint_marginal(e, child, z, z, np.array([[2.25, 0.0], [0.0, 1.0]]), 0.0, 0.0)
    full = orc.rot_joint_marginal(e, child, z, z, np.array([[2.25, 1e-12], [1e-12, 1.0]]), 0.0, 0.0)
    a, b = diag[:, :H - 1, :W - 1], full[:, :H - 1, :W - 1]
    live = a > -1e5
    assert np.array_equal(live, b > -1e5)
    assert np.max(np.abs(a[live] - b[live])) <= 1e-5
    assert np.all(full[:, H - 1, :] == LOG_ZERO) and np.all(full[:, :, W - 1] == LOG_ZERO)


def test_multi_scale_is_independent_passes(orc):
    """computeRootPosteriorRot over num_scale_steps = 3 (objectdetect_findrot.cpp:
    503-678): every scale is a pass with the joints at scale_from_index(s) =
    min + (max - min)/S * (s + 0.5) (partapp_aux.hpp:54-66); best_conf and the
    part maxima are the last scale's, with scaleidx S - 1 on the argmax and 0
    on the local maxima (:276-283, objectdetect_aux.cpp:300-304); the root
    maxima come from the stacked [S][H][W] posterior with scale neighbours."""
    from partapp_gb300 import synth

    rng = np.random.default_rng(77)
    R, H, W, S = 8, 24, 30, 3
    tree = synth.make_tree(rng, R=R, offset_range=(2.0, 6.0), sigma_range=(1.0, 2.0))
    u = synth.random_log_unary(rng, 10 * S, R, H, W).reshape(10, S, R, H, W)
    lo, hi = 0.5, 2.0  # scales 0.75, 1.25, 1.75: exact in float and double
    multi = orc.ps_infer(orc.make_exp(R=R, n_scales=S, scale_range=(lo, hi), max_local_max=50),
                         tree, u)
    roots = []
    for s in range(S):
        sc = lo + (hi - lo) / S * (s + 0.5)
        one = orc.ps_infer(orc.make_exp(R=R, scale=sc, max_local_max=50), tree, u[:, s])
        assert np.array_equal(multi["log_marg"][:, s], one["log_marg"]), s
        assert np.array_equal(multi["root_post"][s], one["root_post"]), s
        roots.append(one["root_post"])
        if s == S - 1:
            assert np.array_equal(multi["best_conf"][:, [2, 3, 4, 5, 6]],
                                  one["best_conf"][:, [2, 3, 4, 5, 6]])
            assert (multi["best_conf"][:, 0] == S - 1).all()
            assert np.allclose(multi["best_conf"][:, 1], np.float32(sc))
            assert np.array_equal(multi["n_part_hyps"], one["n_part_hyps"])
            assert (multi["part_hyps"][:, :, 0] == 0).all()
    lm = orc.find_local_max(np.stack(roots), 1000)
    n = multi["n_root_hyps"]
    assert n == len(lm) and n > 0
    scales = (lo + (hi - lo) / S * (lm[:, 0] + 0.5)).astype(np.float32)
    assert np.array_equal(multi["root_hyps"][:n, 0], scales)
    assert np.array_equal(multi["root_hyps"][:n, 1:], lm[:, 1:].astype(np.float32))
    # a maximum must beat both scale neighbours (objectdetect_aux.cpp:223-229)
    stack = np.stack(roots)
    for s, x, y in lm[:, :3].astype(int):
        for t in (s - 1, s + 1):
            if 0 <= t < S:
                assert stack[t, y, x] < stack[s, y, x]
