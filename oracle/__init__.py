"""ctypes binding of the CPU restatement of partapp's inference hot path.

TEST INFRASTRUCTURE ONLY.  The product (the ``partapp_gb300`` package and its
CUDA library) never imports this module.  It is used by ``tests/``, by
``__graft_entry__.smoke()`` as the checker, and by ``bench.py`` for the timed
CPU baseline / reference arm.

The C++ sources next to this file restate the reference functions cited in
``oracle.h``; ``build()`` compiles them with the committed Makefile into
``oracle/_build/liboracle.so``.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "liboracle.so")
_lib = None
_lock = threading.Lock()

LOG_ZERO = -1e6
NO_CLASS_VALUE = 0.0


class OrcExp(C.Structure):
    _fields_ = [
        ("num_rotation_steps", C.c_int),
        ("min_part_rotation", C.c_float),
        ("max_part_rotation", C.c_float),
        ("min_object_scale", C.c_float),
        ("max_object_scale", C.c_float),
        ("strip_border_detections", C.c_float),
        ("max_local_max", C.c_int),
        ("use_pairwise", C.c_int),
        ("sparse_up", C.c_int),
        ("num_scale_steps", C.c_int),
    ]


class OrcTree(C.Structure):
    _fields_ = [
        ("n_parts", C.c_int),
        ("root", C.c_int),
        ("is_upright", C.POINTER(C.c_int)),
        ("n_joints", C.c_int),
        ("child", C.POINTER(C.c_int)),
        ("parent", C.POINTER(C.c_int)),
        ("offset_c", C.POINTER(C.c_double)),
        ("offset_p", C.POINTER(C.c_double)),
        ("C", C.POINTER(C.c_double)),
        ("rot_mean", C.POINTER(C.c_double)),
        ("rot_sigma", C.POINTER(C.c_double)),
    ]


class OrcModels(C.Structure):
    _fields_ = [
        ("n_parts", C.c_int),
        ("n_stumps", C.c_int),
        ("f", C.POINTER(C.c_int32)),
        ("p", C.POINTER(C.c_float)),
        ("theta", C.POINTER(C.c_float)),
        ("alpha", C.POINTER(C.c_float)),
        ("sum_alpha", C.POINTER(C.c_float)),
    ]


def build(force: bool = False) -> str:
    """Compile liboracle.so with the Makefile beside this file."""
    with _lock:
        if force or not os.path.exists(_LIB_PATH) or _stale():
            subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


def _stale() -> bool:
    t = os.path.getmtime(_LIB_PATH)
    return any(os.path.getmtime(os.path.join(_HERE, f)) > t for f in ("oracle.cpp", "oracle.h"))


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(_LIB_PATH)
        _declare(_lib)
    return _lib


def _p(a, ct):
    return a.ctypes.data_as(C.POINTER(ct)) if a is not None else None


def _declare(L):
    fp, ip, dp = C.POINTER(C.c_float), C.POINTER(C.c_int), C.POINTER(C.c_double)
    L.orc_adaboost_eval.argtypes = [C.POINTER(C.c_int32), fp, fp, fp, C.c_int, C.c_float, fp,
                                    C.c_int64, C.c_int, C.c_int, fp]
    L.orc_adaboost_eval.restype = None
    L.orc_sum_alpha.argtypes = [fp, C.c_int]
    L.orc_sum_alpha.restype = C.c_float
    L.orc_score_grid_window.argtypes = [C.POINTER(C.c_int32), fp, fp, fp, C.c_int, C.c_float, fp,
                                        C.POINTER(C.c_uint8), C.c_int, C.c_int, C.c_int, C.c_int,
                                        C.c_int, C.c_double, C.c_int, fp]
    L.orc_score_grid_window.restype = None
    L.orc_squeeze_bbox.argtypes = [fp, C.c_int, C.c_int, ip]
    L.orc_squeeze_bbox.restype = C.c_int
    L.orc_transform_grid.argtypes = [fp, C.c_int, C.c_int, fp, C.c_int, C.c_int, dp, C.c_float,
                                     C.c_int]
    L.orc_transform_grid.restype = None
    L.orc_clip_log.argtypes = [fp, C.c_int64]
    L.orc_clip_log.restype = None
    L.orc_gaussian_filter.argtypes = [C.c_double, dp]
    L.orc_gaussian_filter.restype = C.c_int
    L.orc_eig2d.argtypes = [dp, dp, dp]
    L.orc_eig2d.restype = None
    for suf, t in (("f32", fp), ("f64", dp)):
        fn = getattr(L, "orc_rot_joint_marginal_" + suf)
        fn.argtypes = [C.POINTER(OrcExp), t, t, C.c_int, C.c_int, C.c_int, dp, dp, dp, C.c_double,
                       C.c_double, C.c_double]
        fn.restype = C.c_int
        fn = getattr(L, "orc_ps_infer_" + suf)
        fn.argtypes = [C.POINTER(OrcExp), C.POINTER(OrcTree), t, C.c_int, C.c_int, t, fp, t, fp, ip,
                       fp, ip]
        fn.restype = C.c_int
    L.orc_find_local_max.argtypes = [fp, C.c_int, C.c_int, C.c_int, C.c_int, dp]
    L.orc_find_local_max.restype = C.c_int
    L.orc_extra_unary.argtypes = [C.POINTER(OrcExp), C.c_int, C.c_int, C.c_float, dp, C.c_float,
                                  dp, C.c_double, C.c_double, C.c_float, dp, C.POINTER(C.c_int),
                                  fp, C.c_int, C.c_int, C.c_int]
    L.orc_extra_unary.restype = C.c_int
    L.orc_dpm_score.argtypes = [C.POINTER(OrcExp), C.c_int, C.c_int, C.c_float, fp, C.c_float,
                                C.c_int, fp, C.c_float, C.c_int, fp, C.POINTER(C.c_int), fp,
                                C.c_int, C.c_int, C.c_int]
    L.orc_dpm_score.restype = C.c_int
    L.orc_nms_recursive.argtypes = [C.c_int, fp, fp, fp, fp, C.c_double, C.c_double,
                                    C.POINTER(C.c_int)]
    L.orc_nms_recursive.restype = C.c_int
    L.orc_rect_from_hyp.argtypes = [C.c_float, C.c_float, C.c_float, C.c_double, C.c_double, dp]
    L.orc_rect_from_hyp.restype = None
    L.orc_nms_rects.argtypes = [C.c_int, dp, dp, C.c_double, C.POINTER(C.c_int)]
    L.orc_nms_rects.restype = C.c_int
    L.orc_find_obj_f32.argtypes = [C.POINTER(OrcExp), C.POINTER(OrcTree), C.POINTER(OrcModels), fp,
                                   C.c_int, C.c_int, C.c_int, dp, C.c_int, C.c_int, C.c_int, fp, fp,
                                   fp, fp, fp, ip, fp, ip]
    L.orc_find_obj_f32.restype = C.c_int
    L.orc_find_obj_batch_f32.argtypes = [C.POINTER(OrcExp), C.POINTER(OrcTree),
                                         C.POINTER(OrcModels), C.c_int, C.POINTER(fp), C.c_int,
                                         C.c_int, C.c_int, dp, C.c_int, C.c_int, C.c_int, fp,
                                         C.c_int]
    L.orc_find_obj_batch_f32.restype = C.c_int
    L.orc_ps_from_scores_batch_f32.argtypes = [C.POINTER(OrcExp), C.POINTER(OrcTree), C.c_int,
                                               C.POINTER(fp), C.c_int, C.c_int, dp, C.c_int,
                                               C.c_int, C.c_int, fp, C.c_int]
    L.orc_ps_from_scores_batch_f32.restype = C.c_int


# ---------------------------------------------------------------------------
# Python-facing helpers.  Arrays are numpy, C-contiguous.
# ---------------------------------------------------------------------------

def make_exp(R=24, min_rot=-180.0, max_rot=180.0, scale=1.0, strip=0.0, max_local_max=1000,
             use_pairwise=True, sparse=False, n_scales=1, scale_range=None) -> OrcExp:
    """sparse: bIsSparse of the upward messages (and of rot_joint_marginal);
    the --find_obj path (find_obj) always uses True, as
    findObjectImageRotJoints does.  n_scales > 1 needs scale_range =
    (min_object_scale, max_object_scale) with min < max."""
    lo, hi = (scale, scale) if scale_range is None else scale_range
    return OrcExp(int(R), float(min_rot), float(max_rot), float(lo), float(hi), float(strip),
                  int(max_local_max), int(bool(use_pairwise)), int(bool(sparse)), int(n_scales))


class _TreeHolder:
    """Keeps the numpy arrays behind an OrcTree alive."""

    def __init__(self, tree):
        P = int(tree["n_parts"])
        self.is_upright = np.ascontiguousarray(tree["is_upright"], dtype=np.int32)
        self.child = np.ascontiguousarray(tree["child"], dtype=np.int32)
        self.parent = np.ascontiguousarray(tree["parent"], dtype=np.int32)
        self.offset_c = np.ascontiguousarray(tree["offset_c"], dtype=np.float64)
        self.offset_p = np.ascontiguousarray(tree["offset_p"], dtype=np.float64)
        self.C = np.ascontiguousarray(tree["C"], dtype=np.float64)
        self.rot_mean = np.ascontiguousarray(tree["rot_mean"], dtype=np.float64)
        self.rot_sigma = np.ascontiguousarray(tree["rot_sigma"], dtype=np.float64)
        self.s = OrcTree(P, int(tree["root"]), _p(self.is_upright, C.c_int), len(self.child),
                         _p(self.child, C.c_int), _p(self.parent, C.c_int),
                         _p(self.offset_c, C.c_double), _p(self.offset_p, C.c_double),
                         _p(self.C, C.c_double), _p(self.rot_mean, C.c_double),
                         _p(self.rot_sigma, C.c_double))


class _ModelsHolder:
    def __init__(self, models):
        self.f = np.ascontiguousarray(models["f"], dtype=np.int32)
        self.p = np.ascontiguousarray(models["p"], dtype=np.float32)
        self.theta = np.ascontiguousarray(models["theta"], dtype=np.float32)
        self.alpha = np.ascontiguousarray(models["alpha"], dtype=np.float32)
        P, S = self.f.shape
        self.sum_alpha = np.array([sum_alpha(self.alpha[i]) for i in range(P)], dtype=np.float32)
        self.s = OrcModels(P, S, _p(self.f, C.c_int32), _p(self.p, C.c_float),
                           _p(self.theta, C.c_float), _p(self.alpha, C.c_float),
                           _p(self.sum_alpha, C.c_float))


def sum_alpha(alpha) -> float:
    a = np.ascontiguousarray(alpha, dtype=np.float32)
    return float(lib().orc_sum_alpha(_p(a, C.c_float), len(a)))


def adaboost_eval(f, p, theta, alpha, desc, normalize=True, sum_alpha_value=None):
    f = np.ascontiguousarray(f, dtype=np.int32)
    p = np.ascontiguousarray(p, dtype=np.float32)
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    alpha = np.ascontiguousarray(alpha, dtype=np.float32)
    desc = np.ascontiguousarray(desc, dtype=np.float32)
    D = desc.shape[-1]
    n = desc.size // D
    sa = sum_alpha(alpha) if sum_alpha_value is None else float(sum_alpha_value)
    out = np.empty(desc.shape[:-1], dtype=np.float32)
    lib().orc_adaboost_eval(_p(f, C.c_int32), _p(p, C.c_float), _p(theta, C.c_float),
                            _p(alpha, C.c_float), len(f), sa, _p(desc, C.c_float), n, D,
                            int(normalize), _p(out, C.c_float))
    return out


def score_grid_window(f, p, theta, alpha, cells, valid, gx, gy, grid_step, normalize=True):
    f = np.ascontiguousarray(f, dtype=np.int32)
    p = np.ascontiguousarray(p, dtype=np.float32)
    theta = np.ascontiguousarray(theta, dtype=np.float32)
    alpha = np.ascontiguousarray(alpha, dtype=np.float32)
    cells = np.ascontiguousarray(cells, dtype=np.float32)
    valid = np.ascontiguousarray(valid, dtype=np.uint8)
    ny, nx, Dc = cells.shape
    out = np.empty((ny, nx), dtype=np.float32)
    lib().orc_score_grid_window(_p(f, C.c_int32), _p(p, C.c_float), _p(theta, C.c_float),
                                _p(alpha, C.c_float), len(f), sum_alpha(alpha),
                                _p(cells, C.c_float), _p(valid, C.c_uint8), ny, nx, Dc, int(gx),
                                int(gy), float(grid_step), int(normalize), _p(out, C.c_float))
    return out


def squeeze_bbox(grid):
    g = np.ascontiguousarray(grid, dtype=np.float32)
    bbox = np.zeros(4, dtype=np.int32)
    crop = lib().orc_squeeze_bbox(_p(g, C.c_float), g.shape[0], g.shape[1], _p(bbox, C.c_int))
    return bool(crop), bbox


def transform_grid(grid_in, out_shape, T21, default=0.0, method=1):
    g = np.ascontiguousarray(grid_in, dtype=np.float32)
    T = np.ascontiguousarray(T21, dtype=np.float64).reshape(9)
    out = np.empty(out_shape, dtype=np.float32)
    lib().orc_transform_grid(_p(g, C.c_float), g.shape[0], g.shape[1], _p(out, C.c_float),
                             out_shape[0], out_shape[1], _p(T, C.c_double), float(default),
                             int(method))
    return out


def clip_log(grid):
    g = np.array(grid, dtype=np.float32, copy=True, order="C")
    lib().orc_clip_log(_p(g, C.c_float), g.size)
    return g


def eig2d(M):
    """boost_math::eig2d of a symmetric 2x2 matrix: (V, E) with V's columns
    the eigenvectors and E = (smallest, largest) eigenvalue."""
    m = np.ascontiguousarray(M, dtype=np.float64).reshape(4)
    V = np.zeros(4)
    E = np.zeros(2)
    lib().orc_eig2d(_p(m, C.c_double), _p(V, C.c_double), _p(E, C.c_double))
    return V.reshape(2, 2), E


def gaussian_filter(sigma):
    buf = np.zeros(int(2 * np.floor(3 * sigma + 0.5) + 1) + 8, dtype=np.float64)
    n = lib().orc_gaussian_filter(float(sigma), _p(buf, C.c_double))
    return buf[:n].copy()


def rot_joint_marginal(exp: OrcExp, child, offset_c, offset_p, Cmat, rot_mean, rot_sigma,
                       scale=1.0, f64=False):
    dt, ct = (np.float64, C.c_double) if f64 else (np.float32, C.c_float)
    child = np.ascontiguousarray(child, dtype=dt)
    R, H, W = child.shape
    out = np.empty_like(child)
    oc = np.ascontiguousarray(offset_c, dtype=np.float64)
    op = np.ascontiguousarray(offset_p, dtype=np.float64)
    Cm = np.ascontiguousarray(Cmat, dtype=np.float64).reshape(4)
    fn = lib().orc_rot_joint_marginal_f64 if f64 else lib().orc_rot_joint_marginal_f32
    rc = fn(C.byref(exp), _p(child, ct), _p(out, ct), R, H, W, _p(oc, C.c_double),
            _p(op, C.c_double), _p(Cm, C.c_double), float(rot_mean), float(rot_sigma),
            float(scale))
    if rc:
        raise ValueError(f"orc_rot_joint_marginal failed: {rc}")
    return out


def ps_infer(exp: OrcExp, tree, log_unary, f64=False, want_marg=True, want_hyps=True):
    """Returns dict(log_marg, best_conf, root_post, part_hyps, n_part_hyps, root_hyps,
    n_root_hyps)."""
    dt, ct = (np.float64, C.c_double) if f64 else (np.float32, C.c_float)
    u = np.ascontiguousarray(log_unary, dtype=dt)
    multi = u.ndim == 5  # [P][S][R][H][W]
    P, S, R, H, W = u.shape if multi else (u.shape[0], 1) + u.shape[1:]
    if S != max(1, exp.num_scale_steps):
        raise ValueError("log_unary has a different number of scales than exp")
    th = _TreeHolder(tree)
    K = exp.max_local_max
    marg = np.empty_like(u) if want_marg else None
    best = np.zeros((P, 7), dtype=np.float32)
    rp = np.empty((S, H, W) if multi else (H, W), dtype=dt)
    ph = np.zeros((P, K, 7), dtype=np.float32) if want_hyps else None
    nph = np.zeros(P, dtype=np.int32)
    rh = np.zeros((1000, 4), dtype=np.float32) if want_hyps else None
    nrh = np.zeros(1, dtype=np.int32)
    fn = lib().orc_ps_infer_f64 if f64 else lib().orc_ps_infer_f32
    rc = fn(C.byref(exp), C.byref(th.s), _p(u, ct), H, W, _p(marg, ct), _p(best, C.c_float),
            _p(rp, ct), _p(ph, C.c_float), _p(nph, C.c_int), _p(rh, C.c_float), _p(nrh, C.c_int))
    if rc:
        raise ValueError(f"orc_ps_infer failed: {rc}")
    return dict(log_marg=marg, best_conf=best, root_post=rp, part_hyps=ph, n_part_hyps=nph,
                root_hyps=rh, n_root_hyps=int(nrh[0]))


def find_local_max(grid, max_n):
    g = np.ascontiguousarray(grid, dtype=np.float32)
    S, H, W = g.shape
    out = np.zeros((max(max_n, 1), 4), dtype=np.float64)
    n = lib().orc_find_local_max(_p(g, C.c_float), S, H, W, int(max_n), _p(out, C.c_double))
    return out[:n].copy()


def extra_unary(exp: OrcExp, log_unary, root, rot=None, pos=None, torso=None, is_detect=None):
    """findObjectImageRotJoints' extra unary terms on a copy of log_unary
    [P][S][R][H][W] (or [P][R][H][W]).  rot = (weight, params [P][2]);
    pos = (weight, params [P][4], (det_x, det_y)); torso = (weight, params[4])."""
    u = np.array(log_unary, dtype=np.float32, copy=True)
    shape = u.shape
    if u.ndim == 4:
        u = u[:, None]
    P, S, R, H, W = u.shape
    u = np.ascontiguousarray(u)
    keep = []
    def arr(a):
        if a is None:
            return None
        a = np.ascontiguousarray(a, dtype=np.float64)
        keep.append(a)
        return _p(a, C.c_double)
    rw, rp = (0.0, None) if rot is None else (rot[0], arr(rot[1]))
    pw, pp, det = (0.0, None, (0.0, 0.0)) if pos is None else (pos[0], arr(pos[1]), pos[2])
    tw, tp = (0.0, None) if torso is None else (torso[0], arr(torso[1]))
    isd = None
    if is_detect is not None:
        isd_a = np.ascontiguousarray(is_detect, dtype=np.int32)
        keep.append(isd_a)
        isd = _p(isd_a, C.c_int)
    rc = lib().orc_extra_unary(C.byref(exp), P, int(root), float(rw), rp, float(pw), pp,
                               float(det[0]), float(det[1]), float(tw), tp, isd,
                               _p(u, C.c_float), S, H, W)
    if rc:
        raise ValueError(f"orc_extra_unary failed: {rc}")
    return u.reshape(shape)


def dpm_score(exp: OrcExp, log_unary, root, torso=None, head=None, unary=None, is_detect=None):
    """findObjectImageRotJoints' DPM terms on a copy of log_unary [P][S][R][H][W]
    (or [P][R][H][W]).  torso = (weight, grid [H][W]); head = (weight, part,
    grid [H][W]); unary = (weight, grids [P][R or 1][H][W]); raw scores."""
    u = np.array(log_unary, dtype=np.float32, copy=True)
    shape = u.shape
    if u.ndim == 4:
        u = u[:, None]
    P, S, R, H, W = u.shape
    u = np.ascontiguousarray(u)
    keep = []

    def arr(a):
        a = np.ascontiguousarray(a, dtype=np.float32)
        keep.append(a)
        return _p(a, C.c_float)
    tw, tg = (0.0, None) if torso is None else (torso[0], arr(torso[1]))
    hw, hp, hg = (0.0, 0, None) if head is None else (head[0], head[1], arr(head[2]))
    uw, ur, ug = 0.0, 0, None
    if unary is not None:
        g = np.asarray(unary[1])
        uw, ur, ug = unary[0], int(g.shape[1] == R and R > 1), arr(g)
    isd = None
    if is_detect is not None:
        isd_a = np.ascontiguousarray(is_detect, dtype=np.int32)
        keep.append(isd_a)
        isd = _p(isd_a, C.c_int)
    rc = lib().orc_dpm_score(C.byref(exp), P, int(root), float(tw), tg, float(hw), int(hp), hg,
                             float(uw), ur, ug, isd, _p(u, C.c_float), S, H, W)
    if rc:
        raise ValueError(f"orc_dpm_score failed: {rc}")
    return u.reshape(shape)


def nms_recursive(x, y, scale, score, train_w, train_h):
    """Suppressed flags (bool [n]) of hypotheses sorted by descending score."""
    a = [np.ascontiguousarray(v, dtype=np.float32) for v in (x, y, scale, score)]
    n = len(a[0])
    out = np.zeros(max(n, 1), np.int32)
    rc = lib().orc_nms_recursive(n, *[_p(v, C.c_float) for v in a], float(train_w),
                                 float(train_h), _p(out, C.c_int))
    if rc:
        raise ValueError(f"orc_nms_recursive failed: {rc}")
    return out[:n].astype(bool)


def rect_from_hyp(x, y, scale, reference_height, reference_width):
    """libNms rect_from_hyp: corners [4][2] (double) of one hypothesis."""
    out = np.zeros(8, np.float64)
    lib().orc_rect_from_hyp(float(np.float32(x)), float(np.float32(y)), float(np.float32(scale)),
                            float(reference_height), float(reference_width), _p(out, C.c_double))
    return out.reshape(4, 2)


def nms_rects(rects, scores, ellipse_size=0.5):
    """libNms nms_recursive on rectangles [n][4][2]: suppressed flags (bool [n])."""
    r = np.ascontiguousarray(rects, dtype=np.float64).reshape(-1, 8)
    sc = np.ascontiguousarray(scores, dtype=np.float64)
    n = len(sc)
    out = np.zeros(max(n, 1), np.int32)
    rc = lib().orc_nms_rects(n, _p(r, C.c_double), _p(sc, C.c_double), float(ellipse_size),
                             _p(out, C.c_int))
    if rc:
        raise ValueError(f"orc_nms_rects failed: {rc}")
    return out[:n].astype(bool)


def find_obj(exp: OrcExp, tree, models, desc, Tig, H, W, interpolate=True):
    """Whole --find_obj path for one image; desc is [R][ny][nx][D]."""
    desc = np.ascontiguousarray(desc, dtype=np.float32)
    R, ny, nx, D = desc.shape
    th, mh = _TreeHolder(tree), _ModelsHolder(models)
    P = th.s.n_parts
    K = exp.max_local_max
    T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(9)
    lu = np.empty((P, R, H, W), dtype=np.float32)
    marg = np.empty((P, R, H, W), dtype=np.float32)
    best = np.zeros((P, 7), dtype=np.float32)
    rp = np.empty((H, W), dtype=np.float32)
    ph = np.zeros((P, K, 7), dtype=np.float32)
    nph = np.zeros(P, dtype=np.int32)
    rh = np.zeros((1000, 4), dtype=np.float32)
    nrh = np.zeros(1, dtype=np.int32)
    fp = C.c_float
    rc = lib().orc_find_obj_f32(C.byref(exp), C.byref(th.s), C.byref(mh.s), _p(desc, fp), ny, nx,
                                D, _p(T, C.c_double), int(interpolate), H, W, _p(lu, fp),
                                _p(marg, fp), _p(best, fp), _p(rp, fp), _p(ph, fp),
                                _p(nph, C.c_int), _p(rh, fp), _p(nrh, C.c_int))
    if rc:
        raise ValueError(f"orc_find_obj failed: {rc}")
    return dict(log_unary=lu, log_marg=marg, best_conf=best, root_post=rp, part_hyps=ph,
                n_part_hyps=nph, root_hyps=rh, n_root_hyps=int(nrh[0]))


def find_obj_batch(exp: OrcExp, tree, models, descs, Tig, H, W, interpolate=True, n_threads=1):
    """CPU baseline: many images over n_threads threads; returns best_conf [n][P][7]."""
    th, mh = _TreeHolder(tree), _ModelsHolder(models)
    descs = [np.ascontiguousarray(d, dtype=np.float32) for d in descs]
    R, ny, nx, D = descs[0].shape
    arr = (C.POINTER(C.c_float) * len(descs))(*[_p(d, C.c_float) for d in descs])
    best = np.zeros((len(descs), th.s.n_parts, 7), dtype=np.float32)
    T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(9)
    rc = lib().orc_find_obj_batch_f32(C.byref(exp), C.byref(th.s), C.byref(mh.s), len(descs), arr,
                                      ny, nx, D, _p(T, C.c_double), int(interpolate), H, W,
                                      _p(best, C.c_float), int(n_threads))
    if rc:
        raise ValueError(f"orc_find_obj_batch failed: {rc}")
    return best


def ps_from_scores_batch(exp: OrcExp, trees, scores, Tig, H, W, interpolate=True, n_threads=1):
    """The PS half of --find_obj for many images from their score grids:
    scores is a list of [P][R][ny][nx] float32 arrays (the tree's parts),
    trees one tree dict per image (one topology); returns best_conf
    [n][P][7].  Images run on n_threads host threads."""
    ths = [_TreeHolder(t) for t in trees]
    arr_t = (OrcTree * len(ths))(*[t.s for t in ths])
    sc = [np.ascontiguousarray(a, dtype=np.float32) for a in scores]
    P, R, ny, nx = sc[0].shape
    if any(a.shape != sc[0].shape for a in sc) or len(sc) != len(ths):
        raise ValueError("one [P][R][ny][nx] score array per tree, all of one shape")
    ptrs = (C.POINTER(C.c_float) * len(sc))(*[_p(a, C.c_float) for a in sc])
    best = np.zeros((len(sc), P, 7), dtype=np.float32)
    T = np.ascontiguousarray(Tig, dtype=np.float64).reshape(9)
    rc = lib().orc_ps_from_scores_batch_f32(C.byref(exp), arr_t, len(sc), ptrs, ny, nx,
                                            _p(T, C.c_double), int(interpolate), H, W,
                                            _p(best, C.c_float), int(n_threads))
    if rc:
        raise ValueError(f"orc_ps_from_scores_batch failed: {rc}")
    return best


# ---------------------------------------------------------------- SHAPEv5
PATCH = 21
SHAPE_DIM = 96


def _desc_decl(L):
    if getattr(L, "_desc_declared", False):
        return L
    fp, dp, ip = C.POINTER(C.c_float), C.POINTER(C.c_double), C.POINTER(C.c_int)
    L.orc_patch_tables.argtypes = [fp, dp, dp]
    L.orc_patch_tables.restype = None
    L.orc_shape_descriptor.argtypes = [fp, fp]
    L.orc_shape_descriptor.restype = None
    L.orc_feature_grid.argtypes = [C.c_int, C.c_int, dp, dp, C.c_double, dp, ip, ip]
    L.orc_feature_grid.restype = None
    L.orc_descriptor_grid.argtypes = [fp, C.c_int, C.c_int, dp, dp, C.c_double, C.c_int, fp,
                                      C.POINTER(C.c_uint8)]
    L.orc_descriptor_grid.restype = C.c_int
    L.orc_descriptor_grid_ex.argtypes = [fp, C.c_int, C.c_int, dp, dp, C.c_double, C.c_int, fp,
                                         ip, fp, C.POINTER(C.c_uint8)]
    L.orc_descriptor_grid_ex.restype = C.c_int
    L.orc_smooth.argtypes = [fp, C.c_int, C.c_int, C.c_float, fp]
    L.orc_smooth.restype = C.c_int
    L.orc_add_border.argtypes = [fp, C.c_int, C.c_int, C.c_int, fp]
    L.orc_add_border.restype = C.c_int
    L.orc_partdetect.argtypes = [C.c_void_p, C.c_void_p, ip, dp, C.c_int, C.c_int, C.c_double,
                                 fp, C.c_int, C.c_int, C.c_int, fp]
    L.orc_partdetect.restype = C.c_int
    L.orc_partdetect_masked.argtypes = [C.c_void_p, C.c_void_p, ip, dp, C.c_int, C.c_int,
                                        C.c_double, fp, C.c_int, C.c_int, C.c_int, fp, fp]
    L.orc_partdetect_masked.restype = C.c_int
    L._desc_declared = True
    return L


def patch_tables():
    """(mask [21][21] f32, lcpos [21][21] f64, lrpos [21][21] f64)."""
    L = _desc_decl(lib())
    m = np.zeros((PATCH, PATCH), np.float32)
    lc = np.zeros((PATCH, PATCH), np.float64)
    lr = np.zeros((PATCH, PATCH), np.float64)
    L.orc_patch_tables(_p(m, C.c_float), _p(lc, C.c_double), _p(lr, C.c_double))
    return m, lc, lr


def shape_descriptor(patch):
    """KMAcomputeShape of one normalised [21][21] patch -> 96 floats."""
    L = _desc_decl(lib())
    p = np.ascontiguousarray(patch, dtype=np.float32).reshape(PATCH, PATCH)
    v = np.zeros(SHAPE_DIM, np.float32)
    L.orc_shape_descriptor(_p(p, C.c_float), _p(v, C.c_float))
    return v


def _axes(x_axis, y_axis):
    return (np.ascontiguousarray(x_axis, dtype=np.float64).reshape(2),
            np.ascontiguousarray(y_axis, dtype=np.float64).reshape(2))


def feature_grid(img_w, img_h, x_axis, y_axis, desc_step):
    """(rect [4], nx, ny) of FeatureGrid's rotated grid."""
    L = _desc_decl(lib())
    ax, ay = _axes(x_axis, y_axis)
    rect = np.zeros(4, np.float64)
    nx, ny = C.c_int(), C.c_int()
    L.orc_feature_grid(int(img_w), int(img_h), _p(ax, C.c_double), _p(ay, C.c_double),
                       float(desc_step), _p(rect, C.c_double), C.byref(nx), C.byref(ny))
    return rect, nx.value, ny.value


def descriptor_grid(image, x_axis, y_axis, desc_step, desc_size, mask=None, roi=None):
    """computeDescriptorGrid (SHAPEv5): (cells [ny][nx][96] f32, valid [ny][nx] u8).
    mask: detection mask [h][w] or None; roi: (x, y, width, height) as
    QRect(x, y, width, height), or None for QRect(0, 0, w - 1, h - 1)."""
    L = _desc_decl(lib())
    img = np.ascontiguousarray(image, dtype=np.float32)
    h, w = img.shape
    _, nx, ny = feature_grid(w, h, x_axis, y_axis, desc_step)
    ax, ay = _axes(x_axis, y_axis)
    cells = np.zeros((ny, nx, SHAPE_DIM), np.float32)
    valid = np.zeros((ny, nx), np.uint8)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    if mk is not None and mk.shape != (h, w):
        raise ValueError("the detection mask must have the image's shape")
    rr = None if roi is None else np.ascontiguousarray(roi, dtype=np.int32)
    rc = L.orc_descriptor_grid_ex(_p(img, C.c_float), h, w, _p(ax, C.c_double),
                                  _p(ay, C.c_double), float(desc_step), int(desc_size),
                                  None if mk is None else _p(mk, C.c_float),
                                  None if rr is None else _p(rr, C.c_int), _p(cells, C.c_float),
                                  _p(valid, C.c_uint8))
    if rc:
        raise ValueError(f"orc_descriptor_grid failed: {rc}")
    return cells, valid


def smooth(image, sigma):
    """libKMA2's recursive Gaussian smooth(image, out, sigma): along y, then x."""
    L = _desc_decl(lib())
    img = np.ascontiguousarray(image, dtype=np.float32)
    out = np.empty_like(img)
    if L.orc_smooth(_p(img, C.c_float), img.shape[0], img.shape[1], float(sigma),
                    _p(out, C.c_float)):
        raise ValueError("orc_smooth needs an image of at least 5 x 5")
    return out


def add_border(image, b):
    """add_image_border2: mirrored border; returns (bordered image, border used)."""
    L = _desc_decl(lib())
    img = np.ascontiguousarray(image, dtype=np.float32)
    h, w = img.shape
    bb = b if (b < w and b < h) else min(w, h) - 1
    out = np.zeros((h + 2 * bb, w + 2 * bb), np.float32)
    used = L.orc_add_border(_p(img, C.c_float), h, w, int(b), _p(out, C.c_float))
    return out, used


def partdetect(exp: OrcExp, models, windows, desc_step, desc_size, ratio, image, flip=False,
               mask=None):
    """partdetect_dense (one image, in-memory path) + clip/log: windows =
    [(window_size_x, window_size_y, pos_offset_x, pos_offset_y)] per
    classifier; mask: detection masks [S][h][w] or None; returns log
    unaries [n][R][h][w], or [n][S][R][h][w] for num_scale_steps = S > 1."""
    L = _desc_decl(lib())
    mh = _ModelsHolder(models)
    n = mh.s.n_parts
    img = np.ascontiguousarray(image, dtype=np.float32)
    h, w = img.shape
    ws = np.ascontiguousarray([[int(a[0]), int(a[1])] for a in windows], dtype=np.int32)
    po = np.ascontiguousarray([[float(a[2]), float(a[3])] for a in windows], dtype=np.float64)
    S = max(1, exp.num_scale_steps)
    out = np.zeros((n, S, exp.num_rotation_steps, h, w), np.float32)
    mk = None if mask is None else np.ascontiguousarray(mask, dtype=np.float32)
    if mk is not None and mk.shape != (S, h, w):
        raise ValueError("detection masks must be [S][h][w]")
    rc = L.orc_partdetect_masked(C.addressof(exp), C.addressof(mh.s), _p(ws, C.c_int),
                                 _p(po, C.c_double), int(desc_step), int(desc_size),
                                 float(ratio), _p(img, C.c_float), h, w, int(bool(flip)),
                                 None if mk is None else _p(mk, C.c_float), _p(out, C.c_float))
    if rc:
        raise ValueError(f"orc_partdetect failed: {rc}")
    return out if S > 1 else out[:, 0]
