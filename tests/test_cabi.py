"""C-ABI boundary checks that need no GPU: the library builds for sm_103a,
loads, and exports exactly the entry points include/partapp_gb300.h declares."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def lib():
    from partapp_gb300 import build

    build.build()
    import partapp_gb300

    return partapp_gb300.load_library()


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "partapp_gb300.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(pa_[a-z_0-9]+)\s*\(", text)))


def test_header_and_binding_agree():
    import partapp_gb300

    assert declared_symbols() == sorted(partapp_gb300.EXPORTS)


def test_library_exports_every_declared_symbol(lib):
    for name in declared_symbols():
        assert hasattr(lib, name), name


def test_status_strings_and_defaults(lib):
    import ctypes

    import partapp_gb300 as pa

    assert lib.pa_status_string(0) == b"ok"
    assert lib.pa_status_string(2) == b"unsupported"
    e = pa.ExpParam()
    lib.pa_exp_param_default(ctypes.byref(e))
    assert (e.num_rotation_steps, e.min_part_rotation, e.max_part_rotation) == (48, -180.0, 180.0)
    assert (e.roi_save_num_samples, e.use_pairwise, e.interpolate) == (1000, 1, 0)


def test_null_context_is_rejected(lib):
    # no GPU work: every entry point validates its context first
    assert lib.pa_ctx_synchronize(None) == 1
    assert lib.pa_score_grids(None, None, 0, None, 0, 0, 0, 0, 0, None, 0) == 1
