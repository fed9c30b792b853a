"""The drop-in boundary: libegsgpu.so loads without a GPU, exports every entry
point declared in include/egsgpu.h, and reports errors through its status
codes (no exit, no fallback)."""
import ctypes as C
import os
import re
import subprocess

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


def test_config_keywords_name_fields_of_the_c_struct(L):
    c = eg.default_config(inter_batch=12, fp64_near_faces=1, capacity=1 << 20)
    assert (c.inter_batch, c.fp64_near_faces, c.capacity) == (12, 1, 1 << 20)
    # a misspelt name must not pass silently as a Python attribute
    with pytest.raises(TypeError):
        eg.default_config(inter_bach=12)


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


def blob(nv, hist, batches, sums, sum2s, dep=1.0, esc=2.0):
    """A checkpoint in the layout egsgpu_checkpoint writes."""
    import numpy as np
    hdr = np.array([0x45475347505531, nv, hist, batches], dtype=np.int64).tobytes()
    en = np.array([dep, esc], dtype=np.float64).tobytes()
    cnt = np.arange(8, dtype=np.uint64).tobytes()
    return hdr + en + cnt + np.asarray(sums, np.float64).tobytes() + np.asarray(sum2s, np.float64).tobytes()


def test_combine_checkpoints_adds_shards(L):
    import numpy as np
    rng = np.random.default_rng(1)
    nv = 37
    a = blob(nv, 1000, 10, rng.random(nv), rng.random(nv), 5.0, 1.0)
    b = blob(nv, 500, 5, rng.random(nv), rng.random(nv), 3.0, 2.0)
    c = eg.checkpoint_arrays(eg.combine_checkpoints(a, b))
    A, B = eg.checkpoint_arrays(a), eg.checkpoint_arrays(b)
    assert c["histories"] == 1500 and c["batches"] == 15
    assert c["deposited"] == 8.0 and c["escaped"] == 3.0
    assert np.array_equal(c["counters"], 2 * np.arange(8, dtype=np.uint64))
    assert np.array_equal(c["sum"], A["sum"] + B["sum"]) and np.array_equal(c["sum2"], A["sum2"] + B["sum2"])


def test_combine_checkpoints_refuses_mismatches(L):
    import numpy as np
    a = blob(4, 100, 10, np.ones(4), np.ones(4))
    with pytest.raises(eg.EGSError):              # another phantom size
        eg.combine_checkpoints(a, blob(5, 100, 10, np.ones(5), np.ones(5)))
    with pytest.raises(eg.EGSError):              # other histories per batch
        eg.combine_checkpoints(a, blob(4, 100, 5, np.ones(4), np.ones(4)))
    with pytest.raises(eg.EGSError):              # truncated
        eg.combine_checkpoints(a, a[:-8])
    n = C.c_size_t(0)
    assert L.egsgpu_combine_checkpoints(a, len(a), a, len(a), None, C.byref(n)) == 0 and n.value == len(a)


C_CALLER = r"""
#include <stdio.h>
#include "egsgpu.h"
int main(void) {
    egsgpu_config c;
    egsgpu_handle *h = 0;
    int rc;
    egsgpu_default_config(&c);
    if (c.precision != 32) return 10;
    c.precision = 16;
    rc = egsgpu_create(&c, &h);
    if (rc != EGSGPU_ERR_ARG || h) return 11;
    if (!egsgpu_last_error(0)) return 12;
    printf("%d\n", rc);
    return 0;
}
"""


def test_header_is_plain_c_and_links(L, tmp_path):
    # the boundary is usable from C (the language of cgo, JNI and FFI
    # bindings): the header compiles as strict C99 and a C program links
    # against the library and calls it
    src = tmp_path / "caller.c"
    src.write_text(C_CALLER)
    exe = tmp_path / "caller"
    lib_dir = os.path.dirname(eg.library_path())
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Wextra", "-pedantic", "-Werror", "-I",
                        os.path.join(ROOT, "include"), str(src), "-o", str(exe), "-L" + lib_dir, "-legsgpu",
                        "-Wl,-rpath," + lib_dir], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == "1", (r.returncode, r.stdout, r.stderr)
