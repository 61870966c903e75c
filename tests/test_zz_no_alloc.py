"""The allocation-free message entry point, pa_rot_joint_marginal_noalloc.

It exists for callers that may not allocate device memory on their call
path; its scratch is a fixed static device array shared by all calls.  This
file is collected last so that a failure here stops a `-x` run only after
every other test has run.  The test calls the entry point through the C-ABI
twice in a row (a larger message, then a smaller one, so stale contents of
the shared array from the first call must not leak into the second) and
compares each result with the allocating entry point within the tolerance of
the other message tests (per-cell max-normalised 1e-5, out-of-grid cells
exactly LOG_ZERO).
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _maxnorm_err(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.abs(np.exp(a - a.max()) - np.exp(b - b.max())).max())


def test_noalloc_matches_allocating_entry_point_twice():
    import torch

    from partapp_gb300 import build

    build.build()
    import partapp_gb300 as pa
    from partapp_gb300 import synth

    assert torch.cuda.is_available()
    lib = pa.load_library()
    ctx = pa.Context(0)
    rng = np.random.default_rng(77)
    dp = lambda a: np.ascontiguousarray(a, dtype=np.float64).reshape(-1)
    pd = lambda a: a.ctypes.data_as(C.POINTER(C.c_double))
    cases = [(24, 120, 160, 1, 2.2, (7.5, -3.0), (-4.25, 6.0), (3.5, 2.0)),
             (12, 40, 56, -2, 1.4, (2.0, 2.5), (1.5, -3.5), (1.2, 2.7))]
    for R, H, W, k, rs, oc, op, sig in cases:
        assert R * H * W <= pa.NOALLOC_MAX_CELLS
        child = torch.from_numpy(synth.random_log_unary(rng, 1, R, H, W, 0.01)[0]).cuda()
        step = synth.rot_step_rad(R)
        exp = pa.exp_param(R=R)
        ocv, opv, Cm = dp(oc), dp(op), dp(np.diag([sig[0] ** 2, sig[1] ** 2]))
        want = ctx.rot_joint_marginal(exp, child, ocv, opv, Cm, k * step, rs * step)
        got = torch.full_like(child, 123.0)
        st = lib.pa_rot_joint_marginal_noalloc(C.byref(exp), C.c_void_p(child.data_ptr()),
                                               C.c_void_p(got.data_ptr()), R, H, W, pd(ocv),
                                               pd(opv), pd(Cm), float(k * step),
                                               float(rs * step), 1.0, None)
        assert st == pa.PA_OK
        g, w = got.cpu().numpy(), want.cpu().numpy()
        oob = w == np.float32(-1e6)
        assert np.array_equal(g[oob], w[oob])
        assert _maxnorm_err(g, w) <= 1e-5
    # a message larger than the static scratch is refused before any work
    big = torch.zeros((48, 240, 320), dtype=torch.float32, device="cuda")
    exp = pa.exp_param(R=48)
    st = lib.pa_rot_joint_marginal_noalloc(C.byref(exp), C.c_void_p(big.data_ptr()),
                                           C.c_void_p(big.data_ptr()), 48, 240, 320,
                                           pd(dp((1, 1))), pd(dp((1, 1))),
                                           pd(dp(np.eye(2).reshape(-1))), 0.0, 0.1, 1.0, None)
    assert st == pa.PA_ERR_NOMEM
    # host memory is not a device buffer of the current device
    hb = np.zeros((12, 40, 56), np.float32)
    st = lib.pa_rot_joint_marginal_noalloc(C.byref(pa.exp_param(R=12)), hb.ctypes.data_as(C.c_void_p),
                                           hb.ctypes.data_as(C.c_void_p), 12, 40, 56,
                                           pd(dp((1, 1))), pd(dp((1, 1))),
                                           pd(dp(np.eye(2).reshape(-1))), 0.0, 0.1, 1.0, None)
    assert st == pa.PA_ERR_INVALID
    ctx.close()
