"""The CUDA engine on BEAMnrc's EXslabs example, through the C ABI.

EXslabs is the reference's own run of 20 MeV electrons through a 100 cm air
slab (AIR700ICRU, ECUT 1.0, PCUT 0.01, SMAX 5 cm); its listing gives the
energy deposited in the slab per incident electron, 0.2296 MeV +- 0.9%.
tests/test_oracle_exslabs.py holds the oracle to the same listing.  Here:
  * FP64, history by history against the oracle (700 keV media and the SMAX
    step limit on both sides);
  * FP32 and FP64, the deposited energy of 1e6 histories against the listing.
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from oracle.oracle_binding import Oracle
from test_oracle_exslabs import PEGS700, deposit_reference, exslabs_case

pytestmark = pytest.mark.gpu


def engine(precision):
    g, src = exslabs_case()
    e = eg.DoseEngine(["AIR700ICRU"], pegs_file=PEGS700, ecut=1.0, pcut=0.01, smax=5.0, precision=precision)
    e.set_geometry(g)
    e.set_source(src)
    return e


def test_history_by_history_fp64():
    n = 2000
    e = engine(64)
    g, src = exslabs_case()
    o = Oracle(["AIR700ICRU"], ecut=1.0, pcut=0.01, pegs_file=PEGS700)
    o.set_geometry(g)
    o.set_source(src)
    o.set_smax(5.0)
    e.set_history_tally(0, n)
    o.set_history_tally(0, n)
    e.run(n, nbatch=2, seed=13)
    o.run(n, nbatch=2, seed=13)
    hg, ho = e.history_tally(), o.history_tally()
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    assert np.mean(rel < 1e-6) >= 0.97
    # the same step count: SMAX reached the kernels
    assert e.totals()["electron_steps"] == pytest.approx(o.tallies()[2][6], rel=0.02)
    e.close()
    o.close()


@pytest.mark.parametrize("precision", [32, 64])
def test_energy_deposit_matches_reference_run(precision):
    n, nb = 1000000, 20
    e = engine(precision)
    e.run(n, nbatch=nb, seed=2004)
    s, s2, t = e.tallies()
    m = s[0] / nb
    sig = np.sqrt(max(s2[0] / nb - m * m, 0) / (nb - 1)) * nb / n
    dep = s[0] / n
    ref, sref = deposit_reference()
    assert abs(dep - ref) < 3 * np.hypot(sref, sig), (dep, sig, ref, sref)
    tot = e.totals()
    assert tot["deposited"] + tot["escaped"] == pytest.approx(20.0 * n, rel=1e-6)
    e.close()
