"""The poselet-conditioned extra unary terms of findObjectImageRotJoints
(libPictStruct/objectdetect_findrot.cpp:915-948): rotation score, position
score around the root detection, torso position prior.

The oracle (oracle/oracle.cpp, orc_extra_unary) restates the reference's
three functions with their float/double typing; it is pinned by analytic
values (a term is log 1 = 0 at its mean, weight * log 1e-4 far from it,
log(weight) at the torso prior's mean).  The GPU kernel must match the oracle
within 4e-7 * max(1, |v|): CUDA's exp/logf and the host's can differ in the
last bit.
"""
import math

import numpy as np
import pytest

import oracle as orc_mod

LOG_CLIP = float(np.log(np.float32(1e-4)))


@pytest.fixture(scope="module")
def orc():
    orc_mod.build()
    return orc_mod


def test_rotation_term_pins(orc):
    R = 12
    e = orc.make_exp(R=R)
    P, H, W = 3, 2, 3
    u = np.zeros((P, R, H, W), np.float32)
    # part 0 centred on the rotation of bin 4, tiny variance: bin 4 -> log 1, others clipped
    rot4 = np.float32((-180.0 + 30.0 * 4.5) / 180 * math.pi)
    params = np.array([[float(rot4), 1e-6], [0.0, 1e9], [0.0, 1.0]])
    got = orc.extra_unary(e, u, root=2, rot=(2.0, params), is_detect=[1, 1, 0])
    assert np.all(got[0, 4] == 0.0)
    assert np.allclose(got[0, [0, 1, 2, 3, 5, 6, 7, 8, 9, 10, 11]], 2.0 * LOG_CLIP, rtol=0, atol=1e-6)
    assert np.allclose(got[1], 0.0, atol=1e-6)   # huge variance: log(~1)
    assert np.all(got[2] == 0.0)                # not detected: weight * 0


def test_position_and_torso_pins(orc):
    R, H, W = 2, 9, 11
    e = orc.make_exp(R=R)
    P, root = 3, 1
    u = np.zeros((P, R, H, W), np.float32)
    pos = np.array([[2.0, -1.0, 0.5, 0.5], [0.0, 0.0, 1.0, 1.0], [100.0, 100.0, 1.0, 1.0]])
    det = (4.0, 5.0)
    torso = np.array([1.5, -0.5, 1e-3, 1e-3])
    got = orc.extra_unary(e, u, root=root, pos=(3.0, pos, det), torso=(0.25, torso))
    # part 0 peaks at (det_x + 2, det_y - 1) = (6, 4)
    assert got[0, 0, 4, 6] == 0.0 and got[0, 1, 4, 6] == 0.0
    assert np.isclose(got[0, 0, 0, 0], 3.0 * LOG_CLIP, atol=1e-5)
    # part 2 is far away everywhere
    assert np.allclose(got[2], 3.0 * LOG_CLIP, atol=1e-5)
    # the root gets the torso prior only: log(0.25) where W/2 - x = 1.5, H/2 - y = -0.5
    assert np.isclose(got[1, 0, 5, 4], np.log(np.float32(0.25)), atol=1e-6)
    assert np.isclose(got[1, 1, 0, 0], LOG_CLIP, atol=1e-5)


def _case(rng, P=10, S=2, R=12, H=37, W=53):
    u = rng.uniform(-9.0, 0.0, (P, S, R, H, W)).astype(np.float32)
    u[rng.random(u.shape) < 0.02] = np.float32(-1e6)
    rot = np.stack([rng.uniform(-math.pi, math.pi, P), rng.uniform(0.05, 1.0, P) ** 2], 1)
    pos = np.stack([rng.uniform(-15, 15, P), rng.uniform(-15, 15, P), rng.uniform(10, 80, P),
                    rng.uniform(10, 80, P)], 1)
    torso = np.array([rng.uniform(-5, 5), rng.uniform(-5, 5), 200.0, 300.0])
    det = (float(rng.integers(0, W)), float(rng.integers(0, H)))
    is_det = (rng.random(P) < 0.8).astype(np.int32)
    return u, rot, pos, torso, det, is_det


@pytest.mark.gpu
@pytest.mark.parametrize("device", [True, False])
def test_gpu_matches_oracle(orc, device):
    import torch

    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    rng = np.random.default_rng(7 if device else 8)
    u, rot, pos, torso, det, is_det = _case(rng)
    P, S, R, H, W = u.shape
    root = 3
    e = orc.make_exp(R=R, n_scales=S, scale_range=(0.8, 1.2))
    want = orc.extra_unary(e, u, root, rot=(1.5, rot), pos=(0.7, pos, det), torso=(0.9, torso),
                           is_detect=is_det)
    ctx = pa.Context(0)
    try:
        pe = pa.exp_param(R=R, n_scales=S, scale_range=(0.8, 1.2))
        if device:
            g = torch.from_numpy(u).cuda()
            ctx.add_extra_unaries(pe, g, root, rot=(1.5, rot), pos=(0.7, pos, det),
                                  torso=(0.9, torso), is_detect=is_det)
            got = g.cpu().numpy()
        else:
            got = u.copy()
            ctx.add_extra_unaries(pe, got, root, rot=(1.5, rot), pos=(0.7, pos, det),
                                  torso=(0.9, torso), is_detect=is_det)
    finally:
        ctx.close()
    tol = 4e-7 * np.maximum(1.0, np.abs(want))
    assert np.all(np.abs(got - want) <= tol)
    # a pixel whose position or torso term differs in the last bit differs
    # in every rotation and scale (0.5 % of the cells measured)
    assert np.mean(got == want) > 0.98


@pytest.mark.gpu
def test_cli_adds_the_terms_from_prediction_files(tmp_path):
    """`--find_obj --scoregrid_dir ... --pred_dir ... --torso_prior ...`: the
    prediction files as the reference's loaders read them (deviations squared
    into variances, the torso detection truncated to int) -> the same
    best_conf and log Z as the C-ABI composition unary maps -> extra terms ->
    PS through the Python mirror."""
    import os
    import subprocess

    import torch

    sio = pytest.importorskip("scipy.io")
    import partapp_gb300 as pa
    from partapp_gb300 import build
    from test_mat_io import make_scoregrid_experiment

    assert torch.cuda.is_available()
    build.build()
    d = str(tmp_path)
    rng = np.random.default_rng(11)
    tree, scores, tigs, Rr, H, W, P = make_scoregrid_experiment(d, rng)
    root = int(tree["root"])
    rot = np.stack([rng.uniform(-math.pi, math.pi, P), rng.uniform(0.2, 1.0, P)], 1)
    pos = np.stack([rng.uniform(-10, 10, P), rng.uniform(-10, 10, P), rng.uniform(3, 9, P),
                    rng.uniform(3, 9, P)], 1)
    best = np.zeros((P, 7))
    best[:, 4] = rng.uniform(0, W, P)
    best[:, 5] = rng.uniform(0, H, P)
    torso = np.array([[1.5, -2.0, 150.0, 90.0]])
    os.makedirs(os.path.join(d, "pred"))
    os.makedirs(os.path.join(d, "det"))
    sio.savemat(os.path.join(d, "pred", "testlist_params_rot_imgidx_0.mat"), {"rot_test": rot})
    sio.savemat(os.path.join(d, "pred", "testlist_params_pos_imgidx_0.mat"), {"pos_test": pos})
    sio.savemat(os.path.join(d, "det", "pose_est_imgidx0000.mat"), {"best_conf": best})
    sio.savemat(os.path.join(d, "torso_pos_prior.mat"), {"params": torso})
    r = subprocess.run([build.CLI, "--find_obj", "--expdir", d, "--scoregrid_dir",
                        os.path.join(d, "sg"), "--pred_dir", os.path.join(d, "pred"),
                        "--pred_rot_weight", "0.5", "--pred_pos_weight", "0.25",
                        "--torso_det_dir", os.path.join(d, "det"), "--torso_prior",
                        os.path.join(d, "torso_pos_prior.mat"), "--torso_prior_weight", "0.8"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ctx = pa.Context(0)
    try:
        e = pa.exp_param(R=Rr, local_max=50, interpolate=True)
        lu = np.stack([ctx.unary_maps(scores[p][None], tigs[p][None], H, W, interpolate=True)[0]
                       for p in range(P)])
        det = (float(int(best[root, 4])), float(int(best[root, 5])))
        rv = rot.copy()
        rv[:, 1] = rv[:, 1] ** 2
        pv = pos.copy()
        pv[:, 2:] = pv[:, 2:] ** 2
        ctx.add_extra_unaries(e, lu, root, rot=(0.5, rv), pos=(0.25, pv, det),
                              torso=(0.8, torso[0]))
        want = ctx.compute_root_posterior_rot(e, tree, lu, is_sparse=True)
    finally:
        ctx.close()
    got = np.loadtxt(tmp_path / "best_conf_0.txt", dtype=np.float64).astype(np.float32)
    assert np.array_equal(got, want["best_conf"])
    lz = np.loadtxt(tmp_path / "log_z_0.txt", dtype=np.float64)
    assert np.array_equal(lz, np.asarray(want["log_z"], dtype=np.float64))
