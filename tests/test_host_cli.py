"""The C++ host layer (partapp_gb300/host) and its `partapp_find_obj
--find_obj` CLI: the reference-shaped entry points over the C-ABI."""
import os
import subprocess

import numpy as np
import pytest

from partapp_gb300 import build, synth

R, H, W, STRIDE, D = 12, 48, 64, 4, 96


def cli():
    build.build()
    return build.CLI


@pytest.fixture(scope="module")
def ctx():
    import torch

    import partapp_gb300 as pa

    build.build()
    assert torch.cuda.is_available(), "GPU tests need a CUDA device"
    c = pa.Context(0)
    yield c
    c.close()


def write_classifier(path, models, c):
    """The reference's text model format (AdaBoost.cc:295-338)."""
    n = models["f"].shape[1]
    with open(path, "w") as fh:
        fh.write(f"{models['D']}\n{n}\n")
        for i in range(n):
            fh.write("%d %.9g %.9g %.9g %.9g\n" % (models["f"][c, i], models["p"][c, i],
                                                   models["alpha"][c, i], 0.0,
                                                   models["theta"][c, i]))


def write_joints(path, tree):
    P = int(tree["n_parts"])
    with open(path, "w") as fh:
        fh.write(f"{P} {int(tree['root'])}\n")
        fh.write(" ".join(str(int(u)) for u in tree["is_upright"]) + "\n")
        for j in range(P - 1):
            vals = [tree["offset_c"][j][0], tree["offset_c"][j][1], tree["offset_p"][j][0],
                    tree["offset_p"][j][1], *tree["C"][j], tree["rot_mean"][j],
                    tree["rot_sigma"][j]]
            fh.write(f"{int(tree['child'][j])} {int(tree['parent'][j])} " +
                     " ".join("%.17g" % v for v in vals) + "\n")


def make_experiment(d, n_images=3):
    imgs = [synth.make_image(500 + i, R=R, H=H, W=W, n_stumps=60, D=D, offset_range=(3, 8),
                             sigma_range=(1, 2.5)) for i in range(n_images)]
    models = imgs[0]["models"]
    with open(os.path.join(d, "exp.txt"), "w") as fh:
        for k, v in (("num_rotation_steps", R), ("min_part_rotation", -180),
                     ("max_part_rotation", 180), ("object_scale", 1),
                     ("strip_border_detections", 0), ("roi_save_num_samples", 50),
                     ("use_pairwise", 1), ("interpolate", 1), ("height", H), ("width", W),
                     ("grid_ny", H // STRIDE), ("grid_nx", W // STRIDE), ("dim", D),
                     ("n_classifiers", models["f"].shape[0]), ("n_images", n_images)):
            fh.write(f"{k} {v}\n")
    with open(os.path.join(d, "tig.txt"), "w") as fh:
        fh.write(" ".join("%.17g" % t for t in imgs[0]["Tig"].reshape(9)) + "\n")
    write_joints(os.path.join(d, "joints.txt"), imgs[0]["tree"])
    for i, im in enumerate(imgs):
        write_joints(os.path.join(d, f"joints_{i}.txt"), im["tree"])
        im["desc"].astype(np.float32).tofile(os.path.join(d, f"desc_{i}.bin"))
    for c in range(models["f"].shape[0]):
        write_classifier(os.path.join(d, f"class_{c}.txt"), models, c)
    return imgs


def test_cli_builds_and_prints_usage():
    r = subprocess.run([cli(), "--help"], capture_output=True, text=True)
    assert r.returncode == 0 and "--find_obj" in r.stdout


def test_detection_masks_load_as_the_reference_reads_them(tmp_path):
    """detection_mask_imgidx<NNNNN>.mat (NNNNN = imgidx + 1), variable
    detection_mask [S'][H][W] (mat_load_multi_array keeps MATLAB's dims):
    the first S scales come back as [S][H][W]; a file of another image size
    is refused."""
    sio = pytest.importorskip("scipy.io")
    rng = np.random.default_rng(4)
    S, H, W = 3, 5, 7
    mask = rng.integers(0, 3, (S + 1, H, W)).astype(np.float32) * 0.5
    sio.savemat(str(tmp_path / "detection_mask_imgidx00003.mat"), {"detection_mask": mask})
    r = subprocess.run([cli(), "--mask_dump", str(S), str(H), str(W), "--detection_masks_dir",
                        str(tmp_path), "--first", "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    got, cur = [], None
    for line in r.stdout.splitlines():
        if line.startswith("scale"):
            cur = []
            got.append(cur)
        else:
            cur.append([float(v) for v in line.split()])
    assert np.array_equal(np.array(got, np.float32), mask[:S])
    r = subprocess.run([cli(), "--mask_dump", str(S), str(H + 1), str(W), "--detection_masks_dir",
                        str(tmp_path), "--first", "2"], capture_output=True, text=True)
    assert r.returncode == 1 and "detection_mask is not" in r.stderr
    r = subprocess.run([cli(), "--mask_dump", str(S), str(H), str(W), "--detection_masks_dir",
                        str(tmp_path), "--first", "0"], capture_output=True, text=True)
    assert r.returncode == 1  # no file for image 0


def test_cli_reports_a_missing_experiment(tmp_path):
    r = subprocess.run([cli(), "--find_obj", "--expdir", str(tmp_path / "none")],
                       capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("batch", [1, 3])
def test_cli_find_obj_matches_c_abi(tmp_path, ctx, orc, batch):
    """best_conf and log Z from the C++ CLI equal the C-ABI call through the
    Python mirror bit for bit, and match the oracle's argmax."""
    import partapp_gb300 as pa

    imgs = make_experiment(str(tmp_path))
    r = subprocess.run([cli(), "--find_obj", "--expdir", str(tmp_path), "--batch", str(batch)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cls = ctx.classifiers(imgs[0]["models"])
    e = pa.exp_param(R=R, local_max=50, interpolate=True)
    ref = ctx.find_obj_batch(e, [im["tree"] for im in imgs], cls,
                             np.stack([im["desc"] for im in imgs]), imgs[0]["Tig"], H, W)
    oe = orc.make_exp(R=R, max_local_max=50)
    for i, im in enumerate(imgs):
        got = np.loadtxt(tmp_path / f"best_conf_{i}.txt", dtype=np.float64).astype(np.float32)
        assert np.array_equal(got, ref[i]["best_conf"])
        lz = np.loadtxt(tmp_path / f"log_z_{i}.txt", dtype=np.float64)
        assert np.array_equal(lz, np.asarray(ref[i]["log_z"], dtype=np.float64))
        want = orc.find_obj(oe, im["tree"], imgs[0]["models"], im["desc"], im["Tig"], H, W)
        for p in range(got.shape[0]):
            assert tuple(got[p, [2, 4, 5]]) == tuple(want["best_conf"][p, [2, 4, 5]]), (i, p)


@pytest.mark.gpu
def test_cli_writes_reference_mat_files(tmp_path, ctx):
    """pose_est_imgidx<NNNN>.mat (best_conf) and log_part_posterior_final_*.mat
    (log_prob_grid, [R][H][W] as MATLAB sees it), read back with scipy."""
    sio = pytest.importorskip("scipy.io")
    import partapp_gb300 as pa

    imgs = make_experiment(str(tmp_path), n_images=2)
    r = subprocess.run([cli(), "--find_obj", "--expdir", str(tmp_path), "--batch", "2",
                        "--save_marginals"], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cls = ctx.classifiers(imgs[0]["models"])
    e = pa.exp_param(R=R, local_max=50, interpolate=True)
    ref = ctx.find_obj_batch(e, [im["tree"] for im in imgs], cls,
                             np.stack([im["desc"] for im in imgs]), imgs[0]["Tig"], H, W,
                             want_marg=True)
    for i in range(2):
        bc = sio.loadmat(str(tmp_path / f"pose_est_imgidx{i:04d}.mat"))["best_conf"]
        assert bc.shape == (10, 7) and bc.dtype == np.float32
        assert np.array_equal(bc, ref[i]["best_conf"])
        for p in (0, 4, 9):
            g = sio.loadmat(str(tmp_path / f"log_part_posterior_final_imgidx{i}_scaleidx0_o0_pidx{p}.mat"))
            assert np.array_equal(g["log_prob_grid"], ref[i]["log_marg"][p])


@pytest.mark.gpu
def test_cli_find_obj_from_images(tmp_path, ctx):
    """`--find_obj --from_images`: grey PGM images -> partdetect on the GPU ->
    PS with bIsSparse; best_conf equals the C-ABI path (pa_partdetect +
    pa_ps_infer) through the Python mirror bit for bit."""
    import partapp_gb300 as pa

    rng = np.random.default_rng(8)
    Rr, h, w, n_cls = 6, 56, 72, 10
    windows = [(4, 16, 2.0, 8.0)] * n_cls
    models = dict(f=rng.integers(0, 960, (n_cls, 80)).astype(np.int32),
                  p=np.where(rng.random((n_cls, 80)) < 0.5, -1.0, 1.0).astype(np.float32),
                  theta=rng.uniform(0, 60, (n_cls, 80)).astype(np.float32),
                  alpha=rng.uniform(0, 1, (n_cls, 80)).astype(np.float32), D=960)
    tree = synth.make_tree(rng, R=Rr, offset_range=(3.0, 8.0), sigma_range=(1.0, 2.5))
    d = str(tmp_path)
    imgs = []
    for i in range(2):
        g = np.clip(rng.uniform(0, 255, (h, w)), 0, 255)
        k = np.ones(5) / 5.0
        g = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 0, g)
        g = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 1, g)
        g[:, w // 2:] += 70.0
        g8 = np.clip(g, 0, 255).astype(np.uint8)
        with open(os.path.join(d, f"img_{i}.pgm"), "wb") as fh:
            fh.write(f"P5\n# synthetic\n{w} {h}\n255\n".encode())
            fh.write(g8.tobytes())
        imgs.append(g8.astype(np.float32))
    with open(os.path.join(d, "exp.txt"), "w") as fh:
        for k_, v in (("num_rotation_steps", Rr), ("min_part_rotation", -180),
                      ("max_part_rotation", 180), ("object_scale", 1),
                      ("strip_border_detections", 0), ("roi_save_num_samples", 50),
                      ("use_pairwise", 1), ("interpolate", 0), ("n_classifiers", n_cls),
                      ("n_images", 2), ("desc_step", 4), ("desc_size", 10),
                      ("window_desc_step_ratio", 1)):
            fh.write(f"{k_} {v}\n")
    with open(os.path.join(d, "windows.txt"), "w") as fh:
        for wx, wy, ox, oy in windows:
            fh.write(f"{wx} {wy} {ox} {oy}\n")
    write_joints(os.path.join(d, "joints.txt"), tree)
    for c in range(n_cls):
        write_classifier(os.path.join(d, f"class_{c}.txt"), models, c)
    r = subprocess.run([cli(), "--find_obj", "--from_images", "--expdir", d], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    cls = ctx.classifiers(models)
    e = pa.exp_param(R=Rr, local_max=50, interpolate=False)
    for i in range(2):
        lu = ctx.partdetect(e, imgs[i], cls, windows, 4, 10, 1.0)
        ref = ctx.compute_root_posterior_rot(e, tree, lu[:10], is_sparse=True)
        got = np.loadtxt(os.path.join(d, f"best_conf_{i}.txt"), dtype=np.float64).astype(np.float32)
        assert np.array_equal(got, ref["best_conf"]), i


@pytest.mark.gpu
def test_cli_from_images_masks_and_two_scales(tmp_path, ctx):
    """`--from_images --detection_masks_dir DIR` at two scales: the masks
    come from detection_mask_imgidx<NNNNN>.mat ([S][H][W], as
    partdetect_dense loads them) and best_conf equals pa_partdetect_masked +
    pa_ps_infer through the Python mirror."""
    sio = pytest.importorskip("scipy.io")
    import partapp_gb300 as pa

    rng = np.random.default_rng(18)
    Rr, h, w, n_cls = 4, 56, 72, 10
    windows = [(4, 16, 2.0, 8.0)] * n_cls
    models = dict(f=rng.integers(0, 960, (n_cls, 80)).astype(np.int32),
                  p=np.where(rng.random((n_cls, 80)) < 0.5, -1.0, 1.0).astype(np.float32),
                  theta=rng.uniform(0, 60, (n_cls, 80)).astype(np.float32),
                  alpha=rng.uniform(0, 1, (n_cls, 80)).astype(np.float32), D=960)
    tree = synth.make_tree(rng, R=Rr, offset_range=(3.0, 8.0), sigma_range=(1.0, 2.5))
    d = str(tmp_path)
    masks_dir = os.path.join(d, "masks")
    os.makedirs(masks_dir)
    g = np.clip(rng.uniform(0, 255, (h, w)), 0, 255)
    k = np.ones(5) / 5.0
    g = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 0, g)
    g = np.apply_along_axis(lambda v: np.convolve(v, k, mode="same"), 1, g)
    g[h // 3:, :] += 60.0
    img = np.clip(g, 0, 255).astype(np.uint8)
    with open(os.path.join(d, "img_0.pgm"), "wb") as fh:
        fh.write(f"P5\n{w} {h}\n255\n".encode())
        fh.write(img.tobytes())
    mask = np.zeros((3, h, w), np.float32)  # one more scale than used: the first two are read
    mask[0, 6:50, 10:60] = 1.0
    mask[1, :, 20:] = 0.5
    mask[2] = 1.0
    sio.savemat(os.path.join(masks_dir, "detection_mask_imgidx00001.mat"), {"detection_mask": mask})
    with open(os.path.join(d, "exp.txt"), "w") as fh:
        for k_, v in (("num_rotation_steps", Rr), ("min_part_rotation", -180),
                      ("max_part_rotation", 180), ("num_scale_steps", 2),
                      ("min_object_scale", 0.875), ("max_object_scale", 1.125),
                      ("strip_border_detections", 0), ("roi_save_num_samples", 50),
                      ("use_pairwise", 1), ("interpolate", 0), ("n_classifiers", n_cls),
                      ("n_images", 1), ("desc_step", 4), ("desc_size", 10),
                      ("window_desc_step_ratio", 1)):
            fh.write(f"{k_} {v}\n")
    with open(os.path.join(d, "windows.txt"), "w") as fh:
        for wx, wy, ox, oy in windows:
            fh.write(f"{wx} {wy} {ox} {oy}\n")
    write_joints(os.path.join(d, "joints.txt"), tree)
    for c in range(n_cls):
        write_classifier(os.path.join(d, f"class_{c}.txt"), models, c)
    r = subprocess.run([cli(), "--find_obj", "--from_images", "--expdir", d,
                        "--detection_masks_dir", masks_dir], capture_output=True, text=True,
                       timeout=600)
    assert r.returncode == 0, r.stderr
    cls = ctx.classifiers(models)
    e = pa.exp_param(R=Rr, local_max=50, interpolate=False, n_scales=2,
                     scale_range=(0.875, 1.125))
    lu = ctx.partdetect(e, img.astype(np.float32), cls, windows, 4, 10, 1.0, mask=mask[:2])
    full = ctx.partdetect(e, img.astype(np.float32), cls, windows, 4, 10, 1.0)
    assert not np.array_equal(lu, full)  # the masks removed detections
    ref = ctx.compute_root_posterior_rot(e, tree, lu[:10], is_sparse=True)
    got = np.loadtxt(os.path.join(d, "best_conf_0.txt"), dtype=np.float64).astype(np.float32)
    assert np.array_equal(got, ref["best_conf"])


# ------------------------------------------- the reference's joint files
def write_part_conf(path, tree, n_joint_types=1):
    """PartConfig (libPartDetect/PartConfig.proto) in protobuf text format,
    with fields this path does not read mixed in."""
    P = int(tree["n_parts"])
    root = int(tree["root"])
    with open(path, "w") as fh:
        fh.write("# part configuration\n")
        for p in range(P):
            fh.write("part {\n  part_id: %d\n  part_pos: %d\n  part_pos: %d\n" % (p + 1, 2 * p, 2 * p + 1))
            if p == root:
                fh.write("  is_root: true\n")
            fh.write("  is_upright: %s\n  ext_x_pos: 2.5\n}\n" %
                     ("true" if tree["is_upright"][p] else "false"))
        for j in range(P - 1):
            fh.write('joint { child_idx: %d parent_idx: %d type: "RotGaussian" joint_pos: 3 '
                     'num_joint_types: %d }\n' % (int(tree["child"][j]) + 1,
                                                  int(tree["parent"][j]) + 1, n_joint_types))
        fh.write("app_group { part_id: 1 part_id: 2 }\n")


def write_joint_files(spatial, tree, suffix="", scale=1.0):
    """joint_<child>_<parent><suffix>.mat as the reference's save_joint writes
    them (objectdetect_learnparam.cpp:66-90): doubles, vectors as columns."""
    sio = pytest.importorskip("scipy.io")
    os.makedirs(spatial, exist_ok=True)
    for j in range(int(tree["n_parts"]) - 1):
        c, p = int(tree["child"][j]) + 1, int(tree["parent"][j]) + 1
        sio.savemat(os.path.join(spatial, f"joint_{c}_{p}{suffix}.mat"), {
            "type": 2.0, "child_idx": float(c), "parent_idx": float(p),
            "offset_c": (scale * np.asarray(tree["offset_c"][j], np.float64)).reshape(2, 1),
            "offset_p": (scale * np.asarray(tree["offset_p"][j], np.float64)).reshape(2, 1),
            "C": np.asarray(tree["C"][j], np.float64).reshape(2, 2),
            "rot_mean": float(tree["rot_mean"][j]), "rot_sigma": float(tree["rot_sigma"][j])})


def parse_dump(text):
    blocks, cur = [], None
    for line in text.splitlines():
        f = line.split()
        if f[0] == "parts":
            cur = dict(P=int(f[1]), root=int(f[3]), upright=[int(v) for v in f[5:]], joints=[])
            blocks.append(cur)
        elif f[0] == "joint":
            cur["joints"].append([int(f[1]), int(f[2])] + [float(v) for v in f[3:]])
    return blocks


def tree_rows(tree, scale=1.0):
    return [[int(tree["child"][j]), int(tree["parent"][j]),
             *(scale * np.asarray(tree["offset_c"][j])), *(scale * np.asarray(tree["offset_p"][j])),
             *tree["C"][j], tree["rot_mean"][j], tree["rot_sigma"][j]]
            for j in range(int(tree["n_parts"]) - 1)]


def test_joints_from_reference_files(tmp_path):
    """load_joint (objectdetect_learnparam.cpp:92-180) + loadJoints' id ->
    index conversion (objectdetect_aux.cpp:54-141) over scipy-written joint
    files and a text-format part configuration."""
    tree = synth.make_tree(np.random.default_rng(3), R=R, upright=[2, 7])
    write_part_conf(tmp_path / "parts.txt", tree)
    write_joint_files(str(tmp_path / "spatial"), tree)
    r = subprocess.run([cli(), "--joints_dump", "--part_conf", str(tmp_path / "parts.txt"),
                        "--spatial_dir", str(tmp_path / "spatial")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    (b,) = parse_dump(r.stdout)
    assert b["P"] == 10 and b["root"] == int(tree["root"])
    assert b["upright"] == [int(u) for u in tree["is_upright"]]
    assert b["joints"] == tree_rows(tree)


def test_joint_mixtures_from_prediction_files(tmp_path):
    """num_joint_types > 1: the mixture component of each joint comes from
    clusidx_test of testlist_pred_pwise_imgidx_<i>.mat and selects
    joint_<c>_<p>_tidx_<t>.mat (objectdetect_aux.cpp:73-92)."""
    sio = pytest.importorskip("scipy.io")
    tree = synth.make_tree(np.random.default_rng(4), R=R)
    write_part_conf(tmp_path / "parts.txt", tree, n_joint_types=3)
    sp = str(tmp_path / "spatial")
    write_joint_files(sp, tree)
    for t in range(3):
        write_joint_files(sp, tree, suffix=f"_tidx_{t}", scale=1.0 + t)
    pred = tmp_path / "pred"
    pred.mkdir()
    clus = np.array([[t % 3 for t in range(9)], [2] * 9], np.float64)
    for i in range(2):
        sio.savemat(str(pred / f"testlist_pred_pwise_imgidx_{i}.mat"),
                    {"clusidx_test": clus[i].reshape(9, 1)})
    r = subprocess.run([cli(), "--joints_dump", "--part_conf", str(tmp_path / "parts.txt"),
                        "--spatial_dir", sp, "--pred_dir", str(pred), "--first", "0",
                        "--numimgs", "2"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    base, img0, img1 = parse_dump(r.stdout)
    assert base["joints"] == tree_rows(tree)
    assert img1["joints"] == tree_rows(tree, 3.0)
    for j in range(9):
        assert img0["joints"][j] == tree_rows(tree, 1.0 + j % 3)[j]


def test_joint_file_errors(tmp_path):
    """What load_joint asserts on is an error: ids that differ from the part
    configuration, a missing joint file, a missing mixture file of a rotation
    joint."""
    sio = pytest.importorskip("scipy.io")
    tree = synth.make_tree(np.random.default_rng(5), R=R)
    write_part_conf(tmp_path / "parts.txt", tree)
    sp = str(tmp_path / "spatial")
    write_joint_files(sp, tree)
    args = [cli(), "--joints_dump", "--part_conf", str(tmp_path / "parts.txt"), "--spatial_dir", sp]
    c, p = int(tree["child"][4]) + 1, int(tree["parent"][4]) + 1
    f = os.path.join(sp, f"joint_{c}_{p}.mat")
    good = sio.loadmat(f)
    good = {k: v for k, v in good.items() if not k.startswith("__")}
    sio.savemat(f, dict(good, child_idx=float(c + 1)))
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 1 and "differ" in r.stderr
    os.remove(f)
    r = subprocess.run(args, capture_output=True, text=True)
    assert r.returncode == 1 and "cannot open" in r.stderr
    sio.savemat(f, good)
    write_part_conf(tmp_path / "parts.txt", tree, n_joint_types=2)
    pred = tmp_path / "pred"
    pred.mkdir()
    sio.savemat(str(pred / "testlist_pred_pwise_imgidx_0.mat"), {"clusidx_test": np.ones((9, 1))})
    r = subprocess.run(args + ["--pred_dir", str(pred), "--numimgs", "1"], capture_output=True,
                       text=True)
    assert r.returncode == 1 and "mixture" in r.stderr


@pytest.mark.gpu
def test_cli_find_obj_from_reference_joint_files(tmp_path):
    """--part_conf / --spatial_dir give the same results as the same joints
    in joints.txt."""
    imgs = make_experiment(str(tmp_path), n_images=2)
    for i in range(2):
        os.remove(tmp_path / f"joints_{i}.txt")
    write_part_conf(tmp_path / "parts.txt", imgs[0]["tree"])
    write_joint_files(str(tmp_path / "spatial"), imgs[0]["tree"])
    out_a, out_b = tmp_path / "a", tmp_path / "b"
    out_a.mkdir()
    out_b.mkdir()
    base = [cli(), "--find_obj", "--expdir", str(tmp_path), "--batch", "2"]
    r = subprocess.run(base + ["--outdir", str(out_a)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    r = subprocess.run(base + ["--outdir", str(out_b), "--part_conf", str(tmp_path / "parts.txt"),
                               "--spatial_dir", str(tmp_path / "spatial")],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    for i in range(2):
        for name in (f"best_conf_{i}.txt", f"log_z_{i}.txt"):
            assert (out_a / name).read_text() == (out_b / name).read_text()
