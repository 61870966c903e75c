"""The DPM score terms of findObjectImageRotJoints
(libPictStruct/objectdetect_findrot.cpp:883-914): the torso grid on the root
part (computeLogGrid + addDPMScore), the head grid on one part and the
per-part unary grids (addLoadDPMScore, objectdetect_icps.cpp:445-522).

The oracle (oracle/oracle.cpp, orc_dpm_score) restates the two functions with
their float/double typing; it is pinned by analytic values (a grid value of 1
adds weight * log 1 = 0, a torso value of 0 adds weight * LOG_ZERO, a loaded
value at or below 1e-4 adds log(1e-4) whatever the weight, parts that are not
detected get no loaded term).  The GPU kernel must match the oracle within
4e-7 * max(1, |v|): CUDA's logf and the host's can differ in the last bit.
"""
import math

import numpy as np
import pytest

import oracle as orc_mod


@pytest.fixture(scope="module")
def orc():
    orc_mod.build()
    return orc_mod


def test_pins(orc):
    P, R, H, W = 3, 4, 2, 3
    e = orc.make_exp(R=R)
    u = np.zeros((P, R, H, W), np.float32)
    torso = np.ones((H, W), np.float32)
    torso[0, 0] = 0.0
    head = np.ones((H, W), np.float32)
    head[1, 2] = 1e-5
    head[0, 1] = np.float32(math.exp(2.0))
    unary = np.ones((P, R, H, W), np.float32)
    unary[2, 3, 1, 1] = 1e-4  # not above 1e-4 (float 1e-4 < double 1e-4)
    got = orc.dpm_score(e, u, 0, torso=(0.5, torso), head=(3.0, 1, head), unary=(2.0, unary),
                        is_detect=[1, 1, 0])
    assert np.all(got[0, :, 0, 0] == np.float32(0.5) * np.float32(-1e6))
    assert np.all(got[0].reshape(R, -1)[:, 1:] == 0.0)
    assert np.all(got[1, :, 1, 2] == np.float32(math.log(1e-4)))
    assert np.allclose(got[1, :, 0, 1], 6.0, atol=2e-6)
    assert np.all(got[1, :, 0, 0] == 0.0)
    assert np.all(got[2] == 0.0)  # not detected: neither the head nor the unary term
    got2 = orc.dpm_score(e, u, 0, unary=(2.0, unary))
    assert got2[2, 3, 1, 1] == np.float32(math.log(1e-4))
    assert np.count_nonzero(got2) == 1


def _case(rng, P=10, S=2, R=12, H=37, W=53, unary_rot=True):
    u = rng.uniform(-9.0, 0.0, (P, S, R, H, W)).astype(np.float32)
    u[rng.random(u.shape) < 0.02] = np.float32(-1e6)

    def grid(shape):
        g = rng.uniform(0.0, 1.5, shape).astype(np.float32)
        g[rng.random(shape) < 0.05] = 0.0
        g[rng.random(shape) < 0.05] = np.float32(1e-4)
        return g
    torso, head = grid((H, W)), grid((H, W))
    unary = grid((P, R if unary_rot else 1, H, W))
    is_det = (rng.random(P) < 0.8).astype(np.int32)
    is_det[5] = 1
    return u, torso, head, unary, is_det


@pytest.mark.gpu
@pytest.mark.parametrize("device,unary_rot", [(True, True), (False, True), (True, False)])
def test_gpu_matches_oracle(orc, device, unary_rot):
    import torch

    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    rng = np.random.default_rng(11 + 2 * device + unary_rot)
    u, torso, head, unary, is_det = _case(rng, unary_rot=unary_rot)
    P, S, R, H, W = u.shape
    root = 3
    terms = dict(torso=(1.2, torso), head=(0.8, 5, head), unary=(0.6, unary), is_detect=is_det)
    e = orc.make_exp(R=R, n_scales=S, scale_range=(0.8, 1.2))
    want = orc.dpm_score(e, u, root, **terms)
    ctx = pa.Context(0)
    try:
        pe = pa.exp_param(R=R, n_scales=S, scale_range=(0.8, 1.2))
        if device:
            g = torch.from_numpy(u).cuda()
            ctx.add_dpm_scores(pe, g, root, **terms)
            got = g.cpu().numpy()
        else:
            got = u.copy()
            ctx.add_dpm_scores(pe, got, root, **terms)
    finally:
        ctx.close()
    tol = 4e-7 * np.maximum(1.0, np.abs(want))
    assert np.all(np.abs(got - want) <= tol)
    assert np.mean(got == want) > 0.98


@pytest.mark.gpu
def test_cli_adds_the_dpm_grids(tmp_path):
    """`--find_obj --scoregrid_dir ... --dpm_torso_dir ... --dpm_unary_dir ...
    --use_dpm_head --use_dpm_unary --dpm_rot --torso_prior ...`: the DPM grids
    where loadDPMScoreGrid finds them (imgidx_0001.mat, variable scoregrid, a
    plain array for the torso, cells per rotation for the head and the parts)
    -> the same best_conf and log Z as the C-ABI composition unary maps -> DPM
    terms -> torso prior -> PS through the Python mirror."""
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
    rng = np.random.default_rng(21)
    tree, scores, tigs, Rr, H, W, P = make_scoregrid_experiment(d, rng)
    root = int(tree["root"])

    def grid(shape):
        g = rng.uniform(0.0, 1.5, shape).astype(np.float32)
        g[rng.random(shape) < 0.05] = 0.0
        return g

    def cell(gs):
        c = np.empty((len(gs), 1), dtype=object)
        for r, g in enumerate(gs):
            c[r, 0] = g
        return c
    torso_g, head_g = grid((H, W)), grid((H, W))
    unary_g = grid((P, Rr, H, W))
    for sub in ("torso", "unary/head"):
        os.makedirs(os.path.join(d, sub))
    sio.savemat(os.path.join(d, "torso", "imgidx_0001.mat"), {"scoregrid": torso_g})
    sio.savemat(os.path.join(d, "unary", "head", "imgidx_0001.mat"), {"scoregrid": cell([head_g])})
    for p in range(P):
        os.makedirs(os.path.join(d, "unary", f"pidx_{p:04d}"))
        sio.savemat(os.path.join(d, "unary", f"pidx_{p:04d}", "imgidx_0001.mat"),
                    {"scoregrid": cell(list(unary_g[p]))}, do_compression=True)
    torso = np.array([[1.5, -2.0, 150.0, 90.0]])
    sio.savemat(os.path.join(d, "torso_pos_prior.mat"), {"params": torso})
    r = subprocess.run([build.CLI, "--find_obj", "--expdir", d, "--scoregrid_dir",
                        os.path.join(d, "sg"), "--dpm_torso_dir", os.path.join(d, "torso"),
                        "--dpm_torso_weight", "0.7", "--dpm_unary_dir", os.path.join(d, "unary"),
                        "--use_dpm_head", "--dpm_head_weight", "1.3", "--use_dpm_unary",
                        "--dpm_unary_weight", "0.4", "--dpm_rot", "--torso_prior",
                        os.path.join(d, "torso_pos_prior.mat"), "--torso_prior_weight", "0.8"],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ctx = pa.Context(0)
    try:
        e = pa.exp_param(R=Rr, local_max=50, interpolate=True)
        lu = np.stack([ctx.unary_maps(scores[p][None], tigs[p][None], H, W, interpolate=True)[0]
                       for p in range(P)])
        ctx.add_dpm_scores(e, lu, root, torso=(0.7, torso_g), head=(1.3, 5, head_g),
                           unary=(0.4, unary_g))
        ctx.add_extra_unaries(e, lu, root, torso=(0.8, torso[0]))
        want = ctx.compute_root_posterior_rot(e, tree, lu, is_sparse=True)
    finally:
        ctx.close()
    got = np.loadtxt(tmp_path / "best_conf_0.txt", dtype=np.float64).astype(np.float32)
    assert np.array_equal(got, want["best_conf"])
    lz = np.loadtxt(tmp_path / "log_z_0.txt", dtype=np.float64)
    assert np.array_equal(lz, np.asarray(want["log_z"], dtype=np.float64))


@pytest.mark.gpu
def test_invalid_arguments_are_errors():
    import partapp_gb300 as pa
    from partapp_gb300 import build

    build.build()
    u = np.zeros((3, 4, 5, 6), np.float32)
    g = np.ones((5, 6), np.float32)
    ctx = pa.Context(0)
    try:
        pe = pa.exp_param(R=4)
        for kw in (dict(head=(1.0, 3, g)), dict(head=(1.0, -1, g))):
            with pytest.raises(pa.PaError):
                ctx.add_dpm_scores(pe, u, 0, **kw)
        with pytest.raises(pa.PaError):
            ctx.add_dpm_scores(pe, u, 3, torso=(1.0, g))
        with pytest.raises(ValueError):
            ctx.add_dpm_scores(pe, u, 0, unary=(1.0, np.ones((3, 2, 5, 6), np.float32)))
        for kw in (dict(torso=(1.0, np.ones((4, 6), np.float32))),
                   dict(head=(1.0, 1, np.ones((5, 7), np.float32)))):
            with pytest.raises(ValueError):  # torso and head grids are [H][W]
                ctx.add_dpm_scores(pe, u, 0, **kw)
        assert np.all(u == 0.0)  # nothing written by a refused call
        bad = g.copy()
        bad[2, 3] = -0.5  # computeLogGrid's domain is data >= 0
        with pytest.raises(pa.PaError):
            ctx.add_dpm_scores(pe, u.copy(), 0, torso=(1.0, bad))
        ctx.add_dpm_scores(pe, u, 0, torso=(1.0, g))  # the context still works
        assert np.all(u == 0.0)
    finally:
        ctx.close()
