"""The transport kernels' generator window (Rng::ahead) on the host: every
number drawn through the window equals the lazily computed Philox stream's,
through any order of look-aheads, draws, copies and restored copies, and a
look-ahead of k numbers leaves nothing to compute at the next k draws.  The
check program (rng_window_check.cu) includes the engine's own header and is
compiled here with nvcc as host code; it needs no GPU."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_generator_window_matches_the_lazy_stream(tmp_path):
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(nvcc):
        pytest.skip("nvcc not found")
    exe = tmp_path / "rng_window_check"
    r = subprocess.run([nvcc, "-std=c++17", "-O2", "-I", os.path.join(ROOT, "egsnrc_gb300", "csrc"),
                        os.path.join(ROOT, "tests", "rng_window_check.cu"), "-o", str(exe)],
                       capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-3000:]
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.startswith("ok")
    n, covered = int(r.stdout.split()[1]), int(r.stdout.split()[3])
    assert n > 500000 and covered > 100000
