"""Input errors of the egs++ driver (egs_gpu_app), found before it touches a GPU.

The driver reads the whole input (run control, transport parameters,
geometry, source) before it creates the engine, so a bad source block stops it
with a message on a machine without a GPU too.  Each case edits one line of a
valid phase-space input.
"""
import gzip
import os
import shutil
import subprocess

import numpy as np
import pytest

from egsnrc_gb300 import formats
from test_gpu_app import APP, HERE, PHSP


@pytest.fixture(scope="module")
def phsp_file(tmp_path_factory):
    d = tmp_path_factory.mktemp("appin")
    path = d / "EX16MVp.egsphsp1"
    with gzip.open(os.path.join(HERE, "golden", "EX16MVp.egsphsp1.gz"), "rb") as a, open(path, "wb") as b:
        shutil.copyfileobj(a, b)
    p, _ = formats.read_egsphsp(str(path))
    formats.write_iaea_phsp(str(d / "planes"), p[:4], 4, z=np.array([0.0, 1.0, 2.0, 3.0], dtype=np.float32))
    return path, d


def run(tmp_path, text):
    if not os.path.exists(APP):
        pytest.skip("egs_gpu_app not built")
    f = tmp_path / "case.egsinp"
    f.write_text(text)
    return subprocess.run([APP, "-i", str(f), "-p", "521icru", "-o", str(tmp_path / "case")], capture_output=True,
                          text=True, timeout=120)


CASES = {
    "zero rotation vector": (("translation = 0 0 -0.5", "translation = 0 0 -0.5\n            rotation vector = 0 0 0"),
                             "rotation vector of length 0"),
    "latch filter type 2": (("particle type = all", "particle type = all\n        filter type = 2\n"
                             "        latch setting = 0011"), "filter type = 0"),
    "unequal recycling": (("recycle electrons = 1", "recycle electrons = 2"), "different recycle numbers"),
    "unknown particle type": (("particle type = all", "particle type = neutrons"), "unknown particle type"),
    "missing file": (("PHSPFILE", "PHSPFILE.missing"), "cannot read phase-space file"),
}


@pytest.mark.parametrize("case", sorted(CASES))
def test_bad_phase_space_source_input(tmp_path, phsp_file, case):
    path, _ = phsp_file
    (old, new), msg = CASES[case]
    text = PHSP.replace(old, new).replace("PHSPFILE", str(path))
    r = run(tmp_path, text)
    assert r.returncode != 0 and msg in r.stderr, r.stderr


def test_iaea_particles_on_several_planes_refused(tmp_path, phsp_file):
    _, d = phsp_file
    text = PHSP.replace("egs_phsp_source", "iaea_phsp_source").replace(
        "phase space file = PHSPFILE", "iaea phase space file = " + str(d / "planes"))
    r = run(tmp_path, text)
    assert r.returncode != 0 and "not on one plane" in r.stderr, r.stderr


def test_rotated_parallel_beam_refused(tmp_path):
    text = PHSP.replace("library   = egs_phsp_source", "library   = egs_parallel_beam").replace(
        "translation = 0 0 -0.5", "translation = 0 0 -0.5\n            rotation = 0.1 0.2 0.3")
    r = run(tmp_path, text)
    assert r.returncode != 0 and "phase-space sources only" in r.stderr, r.stderr
