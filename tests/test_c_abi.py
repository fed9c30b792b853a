"""The drop-in boundary: libegsgpu.so loads without a GPU, exports every entry
point declared in include/egsgpu.h, and reports errors through its status
codes (no exit, no fallback)."""
import ctypes as C
import os
import re

import pytest

import egsnrc_gb300 as eg

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    text = open(os.path.join(ROOT, "include", "egsgpu.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(egsgpu_[a-z_0-9]+)\s*\(", text)))


@pytest.fixture(scope="module")
def L():
    if not os.path.exists(eg.library_path()):
        from egsnrc_gb300 import build
        build.build_engine()
    return eg.load_library()


def test_every_declared_symbol_is_exported(L):
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(L, n), n


def test_default_config_is_the_reference_profile(L):
    c = eg.default_config()
    assert (c.ecut, c.pcut, c.estepe, c.ximax, c.skindepth, c.precision) == (0.521, 0.010, 0.25, 0.5, 3.0, 32)


def test_create_reports_missing_device_or_bad_args(L):
    h = C.c_void_p()
    c = eg.default_config()
    c.precision = 16
    assert L.egsgpu_create(C.byref(c), C.byref(h)) == 1          # EGSGPU_ERR_ARG
    c.precision = 32
    rc = L.egsgpu_create(C.byref(c), C.byref(h))
    import torch
    if not torch.cuda.is_available():
        assert rc == 4 and not h.value                            # EGSGPU_ERR_CUDA, no handle
    else:
        assert rc == 0
        L.egsgpu_destroy(h)


def test_null_handle_calls_fail_cleanly(L):
    assert L.egsgpu_run(None, 0, 10, 1, 1, None) == 1
    assert L.egsgpu_get_tallies(None, None, None, None) == 7
    assert L.egsgpu_last_error(None) == b"null handle"
