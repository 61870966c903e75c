"""Seeded synthetic inputs with the shapes and value distributions of the
partapp --find_obj workloads.

The LSP images, trained classifiers and learned joints of the original
experiments are not available, so every workload runs on synthetic data drawn
here from a seeded numpy Generator (PCG64 keyed by the seed):

* descriptor fields: one field per rotation (the reference recomputes the
  descriptor grid per rotation, libPartDetect/partdetect_test.cpp:171-192),
  960-dim vectors at stride 4 px, entries ~ Gamma(k=0.5, theta=1) -- drawn as
  z**2/2 with z ~ N(0, 1) -- then L2-normalised per location;
* AdaBoost classifiers: feature index ~ U{0..D-1}, threshold ~ U(0, 0.1),
  polarity +-1, weight ~ U(0, 1);
* the 10-part kinematic tree rooted at the torso, with per-edge offsets
  ~ U(lo, hi) px with random sign, diagonal Gaussian sigma_x, sigma_y
  ~ U(s_lo, s_hi) px, rotation sigma ~ U(1, 3) rotation bins and rotation mean
  k * step with k ~ U{-2..2}.
"""
from __future__ import annotations

import math

import numpy as np

# Part order of the 10-part model: lower/upper legs, lower/upper arms, head,
# torso (root).  Joints are (child, parent) pairs in this order.
PART_NAMES = ("r_lower_leg", "r_upper_leg", "l_upper_leg", "l_lower_leg", "r_lower_arm",
              "r_upper_arm", "l_upper_arm", "l_lower_arm", "head", "torso")
ROOT = 9
JOINTS = ((0, 1), (1, 9), (2, 9), (3, 2), (4, 5), (5, 9), (6, 9), (7, 6), (8, 9))


def rot_step_rad(R: int, min_rot: float = -180.0, max_rot: float = 180.0) -> float:
    """Rotation bin width in radians as computeRotJointMarginal forms it
    (float division of the float range by the step count, then * pi/180)."""
    step = np.float32(np.float32(max_rot) - np.float32(min_rot)) / np.float32(R)
    return float(step) * (math.pi / 180.0)


def make_tree(rng: np.random.Generator, R: int = 24, offset_range=(10.0, 40.0),
              sigma_range=(2.0, 8.0), rot_sigma_bins=(1.0, 3.0), rot_mean_k=(-2, 2),
              upright=None) -> dict:
    """Random 10-part tree with diagonal-covariance rotation joints."""
    J = len(JOINTS)
    step = rot_step_rad(R)
    lo, hi = offset_range
    sign = lambda n: np.where(rng.random(n) < 0.5, -1.0, 1.0)
    offset_c = rng.uniform(lo, hi, (J, 2)) * sign((J, 2))
    offset_p = rng.uniform(lo, hi, (J, 2)) * sign((J, 2))
    sig = rng.uniform(sigma_range[0], sigma_range[1], (J, 2))
    Cm = np.zeros((J, 4))
    Cm[:, 0] = sig[:, 0] ** 2
    Cm[:, 3] = sig[:, 1] ** 2
    rot_sigma = rng.uniform(rot_sigma_bins[0], rot_sigma_bins[1], J) * step
    k = rng.integers(rot_mean_k[0], rot_mean_k[1] + 1, J)
    rot_mean = k * step
    is_upright = np.zeros(len(PART_NAMES), dtype=np.int32)
    if upright:
        for p in upright:
            is_upright[p] = 1
    return dict(n_parts=len(PART_NAMES), root=ROOT, is_upright=is_upright,
                child=np.array([c for c, _ in JOINTS], dtype=np.int32),
                parent=np.array([p for _, p in JOINTS], dtype=np.int32),
                offset_c=offset_c, offset_p=offset_p, C=Cm, rot_mean=rot_mean.astype(np.float64),
                rot_sigma=rot_sigma.astype(np.float64))


def make_models(rng: np.random.Generator, n_parts: int = 10, n_stumps: int = 500,
                D: int = 960) -> dict:
    """n_parts AdaBoost classifiers of n_stumps decision stumps each."""
    f = rng.integers(0, D, (n_parts, n_stumps)).astype(np.int32)
    theta = rng.uniform(0.0, 0.1, (n_parts, n_stumps)).astype(np.float32)
    p = np.where(rng.random((n_parts, n_stumps)) < 0.5, -1.0, 1.0).astype(np.float32)
    alpha = rng.uniform(0.0, 1.0, (n_parts, n_stumps)).astype(np.float32)
    return dict(f=f, p=p, theta=theta, alpha=alpha, D=D)


def make_descriptors(rng: np.random.Generator, R: int, ny: int, nx: int, D: int = 960,
                     dtype=np.float32) -> np.ndarray:
    """[R][ny][nx][D] Gamma(0.5, 1) vectors, L2-normalised per location."""
    z = rng.standard_normal((R, ny, nx, D), dtype=np.float32)
    g = 0.5 * z * z
    g /= np.sqrt(np.sum(g.astype(np.float64) ** 2, axis=-1, keepdims=True)).astype(np.float32)
    return g.astype(dtype, copy=False)


def grid_to_image(stride: float = 4.0, ox: float = 0.0, oy: float = 0.0) -> np.ndarray:
    """Tig of a stride-`stride` grid aligned with the image axes:
    image = stride * grid + offset."""
    return np.array([[stride, 0.0, ox], [0.0, stride, oy], [0.0, 0.0, 1.0]])


def make_image(seed: int, R: int = 24, H: int = 240, W: int = 320, n_parts: int = 10,
               n_stumps: int = 500, D: int = 960, stride: int = 4, offset_range=(10.0, 40.0),
               sigma_range=(2.0, 8.0)) -> dict:
    """Everything one synthetic --find_obj image needs."""
    rng = np.random.default_rng(seed)
    ny, nx = H // stride, W // stride
    tree = make_tree(rng, R=R, offset_range=offset_range, sigma_range=sigma_range)
    models = make_models(rng, n_parts=n_parts, n_stumps=n_stumps, D=D)
    desc = make_descriptors(rng, R, ny, nx, D)
    return dict(tree=tree, models=models, desc=desc, Tig=grid_to_image(stride), R=R, H=H, W=W,
                ny=ny, nx=nx, D=D)


def random_log_unary(rng: np.random.Generator, P: int, R: int, H: int, W: int,
                     zero_frac: float = 0.0) -> np.ndarray:
    """Log unaries with the value range the AdaBoost path produces: log of
    scores in (1e-4, 1], with an optional fraction of exact LOG_ZERO cells."""
    s = rng.uniform(-1.0, 1.0, (P, R, H, W)).astype(np.float32)
    s = np.where(s < 0, np.float32(1e-4), s)
    u = np.log(s.astype(np.float64)).astype(np.float32)
    if zero_frac > 0:
        u[rng.random(u.shape) < zero_frac] = np.float32(-1e6)
    return u
