"""MAT-file reading (partapp_gb300/host/mat_io.hpp + inflate.hpp) and the
--find_obj branch that loads the part detector's saved score grids
(PartApp::loadScoreGrid, libPartApp/partapp.cpp:830-903).

The reader is checked against files written by scipy.io.savemat (an
independent writer of the format), compressed and not, and against
miCOMPRESSED elements built with Python's zlib at every block type
(stored, fixed Huffman, dynamic Huffman).  Values must come back exactly.
"""
import os
import struct
import subprocess
import zlib

import numpy as np
import pytest

from partapp_gb300 import build, synth

sio = pytest.importorskip("scipy.io")


def cli():
    build.build()
    return build.CLI


def dump(path):
    """Variables printed by `partapp_find_obj --mat_dump`: name -> dict."""
    r = subprocess.run([cli(), "--mat_dump", str(path)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    lines = r.stdout.split("\n")
    pos = 0

    def one(indent):
        nonlocal pos
        head = lines[pos][len(indent):].split()
        pos += 1
        assert head[0] == "var"
        name, cls, dims = head[1], int(head[3]), [int(x) for x in head[5:]]
        if cls == 1:
            cells = [one(indent + "  ") for _ in range(int(np.prod(dims)))]
            return dict(name=name, cls=cls, dims=dims, cells=cells)
        vals = np.array([float(x) for x in lines[pos].split()], dtype=np.float64)
        pos += 1
        return dict(name=name, cls=cls, dims=dims, values=vals)

    out = {}
    while pos < len(lines) and lines[pos].startswith("var"):
        v = one("")
        out[v["name"]] = v
    return out


def fortran(a):
    return np.asarray(a, dtype=np.float64).reshape(-1, order="F")


def score_grid_vars(rng, S=2, R=3):
    cells = np.empty((S, R), dtype=object)
    for s in range(S):
        for r in range(R):
            cells[s, r] = rng.uniform(-1, 1, (5 + s, 7 + 2 * s)).astype(np.float32)
    return {"cell_scoregrid": cells,
            "transform_Ti2": rng.uniform(-3, 3, (S, R, 3, 3)).astype(np.float32),
            "transform_T2g": rng.uniform(-3, 3, (S, R, 3, 3)).astype(np.float32)}


@pytest.mark.parametrize("compressed", [True, False])
def test_reads_scipy_cells_and_arrays(tmp_path, compressed):
    rng = np.random.default_rng(1)
    v = score_grid_vars(rng)
    v["ints"] = rng.integers(-100, 100, (4, 3)).astype(np.int16)
    v["bytes"] = rng.integers(0, 255, (2, 5)).astype(np.uint8)
    v["dbl"] = rng.standard_normal((3, 2))
    path = tmp_path / "v.mat"
    sio.savemat(str(path), v, do_compression=compressed)
    got = dump(path)
    c = got["cell_scoregrid"]
    assert c["cls"] == 1 and c["dims"] == [2, 3]
    for s in range(2):
        for r in range(3):
            e = c["cells"][s + 2 * r]  # cells in Fortran order
            want = v["cell_scoregrid"][s, r]
            assert e["dims"] == list(want.shape) and e["cls"] == 7
            assert np.array_equal(e["values"], fortran(want))
    for k in ("transform_Ti2", "transform_T2g", "ints", "bytes", "dbl"):
        assert got[k]["dims"] == list(v[k].shape)
        assert np.array_equal(got[k]["values"], fortran(v[k])), k


def _elements(buf):
    """(type, payload) of the top-level data elements after the header."""
    out, off = [], 128
    while off + 8 <= len(buf):
        t, n = struct.unpack_from("<II", buf, off)
        out.append((t, buf[off + 8:off + 8 + n]))
        off += 8 + (n if t == 15 else (n + 7) // 8 * 8)
    return out


@pytest.mark.parametrize("mode", ["stored", "fixed", "dynamic", "best", "rle"])
def test_inflate_block_types(tmp_path, mode):
    rng = np.random.default_rng(2)
    v = {"a": rng.uniform(0, 1, (40, 30)).astype(np.float32),
         "b": np.repeat(np.arange(50, dtype=np.float32), 20).reshape(25, 40)}
    plain = tmp_path / "plain.mat"
    sio.savemat(str(plain), v, do_compression=False)
    buf = plain.read_bytes()
    out = bytearray(buf[:128])
    for t, payload in _elements(buf):
        raw = struct.pack("<II", t, len(payload)) + payload + bytes((-len(payload)) % 8)
        if mode == "stored":
            z = zlib.compress(raw, 0)
        elif mode == "fixed":
            co = zlib.compressobj(6, zlib.DEFLATED, 15, 9, zlib.Z_FIXED)
            z = co.compress(raw) + co.flush()
        elif mode == "rle":
            co = zlib.compressobj(6, zlib.DEFLATED, 15, 9, zlib.Z_RLE)
            z = co.compress(raw) + co.flush()
        else:
            z = zlib.compress(raw, 6 if mode == "dynamic" else 9)
        out += struct.pack("<II", 15, len(z)) + z
    path = tmp_path / f"{mode}.mat"
    path.write_bytes(bytes(out))
    got = dump(path)
    for k in v:
        assert np.array_equal(got[k]["values"], fortran(v[k])), (mode, k)


def test_corrupt_stream_is_an_error(tmp_path):
    v = {"a": np.arange(100, dtype=np.float32).reshape(10, 10)}
    path = tmp_path / "c.mat"
    sio.savemat(str(path), v, do_compression=True)
    buf = bytearray(path.read_bytes())
    buf[-2] ^= 0x5A  # inside the Adler-32 trailer
    path.write_bytes(bytes(buf))
    r = subprocess.run([cli(), "--mat_dump", str(path)], capture_output=True, text=True)
    assert r.returncode == 1 and "inflate" in r.stderr


def make_scoregrid_experiment(d, rng, Rr=8, H=40, W=56, P=10):
    """exp.txt, joints.txt and per-part compressed score-grid files under d/sg
    as partdetect saves them; returns (tree, scores[p] [R][ny][nx], Tig[p]
    [R][3][3] computed as the host does, Rr, H, W, P)."""
    from test_host_cli import write_joints

    tree = synth.make_tree(rng, R=Rr, offset_range=(3.0, 8.0), sigma_range=(1.0, 2.5))
    with open(os.path.join(d, "exp.txt"), "w") as fh:
        for k, val in (("num_rotation_steps", Rr), ("min_part_rotation", -180),
                       ("max_part_rotation", 180), ("object_scale", 1),
                       ("strip_border_detections", 0), ("roi_save_num_samples", 50),
                       ("use_pairwise", 1), ("interpolate", 1), ("height", H), ("width", W),
                       ("n_images", 1)):
            fh.write(f"{k} {val}\n")
    write_joints(os.path.join(d, "joints.txt"), tree)
    os.makedirs(os.path.join(d, "sg"))
    scores, tigs = [], []
    for p in range(P):
        ny, nx = 9 + p % 3, 13 + p % 2  # squeezed grids differ per part
        cells = np.empty((1, Rr), dtype=object)
        ti2 = np.zeros((1, Rr, 3, 3), np.float32)
        t2g = np.zeros((1, Rr, 3, 3), np.float32)
        tig = np.zeros((Rr, 3, 3))
        for r in range(Rr):
            cells[0, r] = rng.uniform(-0.5, 1.0, (ny, nx)).astype(np.float32)
            a = np.deg2rad(-180 + 360 / Rr * (r + 0.5))
            ti2[0, r] = [[np.cos(a), -np.sin(a), W / 2], [np.sin(a), np.cos(a), H / 2], [0, 0, 1]]
            t2g[0, r] = [[4, 0, -2 * nx], [0, 4, -2 * ny], [0, 0, 1]]
            a64, b64 = ti2[0, r].astype(np.float64), t2g[0, r].astype(np.float64)
            for i in range(3):  # prod(Ti2, T2g), summed in order as the host does
                for j in range(3):
                    acc = 0.0
                    for q in range(3):
                        acc += float(a64[i, q]) * float(b64[q, j])
                    tig[r, i, j] = acc
        sio.savemat(os.path.join(d, "sg", f"imgidx0-pidx{p}-o0-scoregrid.mat"),
                    {"cell_scoregrid": cells, "transform_Ti2": ti2, "transform_T2g": t2g},
                    do_compression=True)
        scores.append(np.stack([cells[0, r] for r in range(Rr)]))
        tigs.append(tig)
    return tree, scores, tigs, Rr, H, W, P


# ------------------------------------------------------------------ GPU
@pytest.mark.gpu
def test_find_obj_from_saved_score_grids(tmp_path):
    """`--find_obj --scoregrid_dir`: per part the saved cell_scoregrid with
    per-rotation Ti2, T2g (compressed, as partdetect saves them) -> Tig = Ti2
    T2g -> pa_unary_maps -> pa_ps_infer (bIsSparse); best_conf and log Z equal
    the same composition through the Python mirror bit for bit."""
    import torch

    import partapp_gb300 as pa

    assert torch.cuda.is_available()
    d = str(tmp_path)
    tree, scores, tigs, Rr, H, W, P = make_scoregrid_experiment(d, np.random.default_rng(5))
    r = subprocess.run([cli(), "--find_obj", "--expdir", d, "--scoregrid_dir",
                        os.path.join(d, "sg")], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ctx = pa.Context(0)
    try:
        e = pa.exp_param(R=Rr, local_max=50, interpolate=True)
        lu = np.stack([ctx.unary_maps(scores[p][None], tigs[p][None], H, W, interpolate=True)[0]
                       for p in range(P)])
        want = ctx.compute_root_posterior_rot(e, tree, lu, is_sparse=True)
    finally:
        ctx.close()
    got = np.loadtxt(tmp_path / "best_conf_0.txt", dtype=np.float64).astype(np.float32)
    assert np.array_equal(got, want["best_conf"])
    lz = np.loadtxt(tmp_path / "log_z_0.txt", dtype=np.float64)
    assert np.array_equal(lz, np.asarray(want["log_z"], dtype=np.float64))


@pytest.mark.parametrize("compressed", [True, False])
def test_corrupt_files_fail_cleanly(tmp_path, compressed):
    """Mutated and truncated files: the reader reports an error or reads
    something, but never crashes or hangs (every offset and size is checked
    against the buffer; the inflater checks its input and distances)."""
    rng = np.random.default_rng(17 if compressed else 18)
    v = score_grid_vars(rng)
    good = tmp_path / "good.mat"
    sio.savemat(str(good), v, do_compression=compressed)
    buf = good.read_bytes()
    for trial in range(60):
        b = bytearray(buf)
        if trial % 3 == 0:
            b = b[:int(rng.integers(1, len(b)))]
        else:
            for _ in range(int(rng.integers(1, 6))):
                b[int(rng.integers(128, len(b)))] = int(rng.integers(0, 256))
        path = tmp_path / f"bad{trial}.mat"
        path.write_bytes(bytes(b))
        r = subprocess.run([cli(), "--mat_dump", str(path)], capture_output=True, timeout=60)
        assert r.returncode in (0, 1), (trial, r.returncode, r.stderr[-300:])
