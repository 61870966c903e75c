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


def test_null_context_is_rejected_by_the_image_entries(lib):
    # the descriptor, detection and multi-scale entries check the context
    # before anything else (no GPU is touched)
    assert lib.pa_descriptor_grid_masked(None, None, 0, 0, None, None, 0.0, 0, None, None, None,
                                         None, 0) == 1
    assert lib.pa_partdetect_masked(None, None, None, 0, 0, 0, None, 0, None, None, None, None,
                                    0) == 1
    assert lib.pa_find_obj_scales(None, None, None, 0, None, 0, None, 0, 0, None, 0) == 1
    assert lib.pa_nms_rects(None, 0, None, None, 0.5, None, 0) == 1


def test_mask_buffers_follow_the_image(lib):
    """A numpy detection mask beside a host image stays a host buffer of the
    checked shape; a wrong shape is refused before any call."""
    import numpy as np

    import partapp_gb300 as pa

    img = pa._Buf(np.zeros((6, 8), np.float32), np.float32)
    m = pa._mask_buf(np.ones((6, 8), np.float64), img, (6, 8))
    assert m.mem == pa.PA_MEM_HOST and m.arr.dtype == np.float32 and m.arr.shape == (6, 8)
    assert pa._mask_buf(None, img, (6, 8)) is None
    with pytest.raises(ValueError):
        pa._mask_buf(np.ones((2, 6, 8), np.float32), img, (6, 8))
