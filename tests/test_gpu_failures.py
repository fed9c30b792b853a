"""Failure detection without a GPU fault: every failure here is made on the
host (bad data) or by a device loop running out of its iteration cap, which
the kernel turns into an error status; the context stays usable.

* Device caps (egsgpu_config.loop_cap, .step_cap; the reference's analogues
  are simulateSingleShower's 100000-try limit, egs++/egs_application.cpp:
  925-930, and loopMax, egs++/egs_functions.h:96): a cap of one rejection-loop
  iteration, or of two transport steps per particle, makes the run return
  EGSGPU_ERR_LOOP; a new engine on the same device then runs normally.
* Data (HATCH's file reading, src/egsnrc.mortran:1828-2152): a missing data
  directory is EGSGPU_ERR_DATA, a PEGS4 file cut inside a medium's block and a
  medium absent from the file are EGSGPU_ERR_MEDIUM; nothing exits.
"""
import os

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

ERR_DATA, ERR_MEDIUM, ERR_LOOP = 2, 3, 6


def run_with(**cfg):
    wl = W.water128e(16)
    e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=32, **cfg)
    e.set_geometry(wl["geometry"])
    e.set_source(wl["source"])
    try:
        e.run(2000, nbatch=1, seed=3)
        return 0, e
    except eg.EGSError as ex:
        return ex.code, e


@pytest.mark.parametrize("cap", [{"loop_cap": 1}, {"step_cap": 2}])
def test_device_cap_returns_loop_error_and_the_device_stays_usable(cap):
    code, e = run_with(**cap)
    e.close()
    assert code == ERR_LOOP
    code, e = run_with()
    assert code == 0
    t = e.totals()
    assert abs(t["deposited"] + t["escaped"] - 2000 * 20.0) < 2e-4 * 2000 * 20.0
    e.close()


def test_missing_data_directory_is_a_data_error(tmp_path):
    with pytest.raises(eg.EGSError) as ex:
        eg.DoseEngine([W.WATER], data_dir=str(tmp_path / "nowhere"))
    assert ex.value.code == ERR_DATA


def test_truncated_pegs4_block_is_a_medium_error(tmp_path):
    text = open(eg.PEGS_FILE).read()
    i = text.index(" MEDIUM=H2O521ICRU")
    cut = tmp_path / "cut.pegs4dat"
    cut.write_text(text[:i + 20000])          # inside the water block's tables
    with pytest.raises(eg.EGSError) as ex:
        eg.DoseEngine([W.WATER], pegs_file=str(cut))
    assert ex.value.code == ERR_MEDIUM and "H2O521ICRU" in str(ex.value)


def test_medium_missing_from_the_pegs4_file(tmp_path):
    with pytest.raises(eg.EGSError) as ex:
        eg.DoseEngine(["NOSUCHMEDIUM"])
    assert ex.value.code == ERR_MEDIUM
