"""The oracle against a run of the reference itself: BEAMnrc's EXslabs example.

EXslabs (omega/beamnrc/BEAMnrc_examples/EXslabs/EXslabs.egsinp) sends a pencil
beam of 20 MeV electrons along z through a 100 cm slab of AIR700ICRU whose
square outer boundary has a half-width of 10 cm (ECUT 1.0, PCUT 0.01, SMAX 5 cm,
ESTEPE 0.25, XIMAX 0.5, PRESTA-II), 1000 histories.  Its listing
(EXslabs.egslst) gives the energy deposited in the slab per incident electron
with its uncertainty, and the fluence of the particles that leave through the
back face; its phase-space file (EXslabs.egsphsp1) holds those particles.
Both are fixtures here (tests/golden/beamnrc_examples.json, generated from the
listing by tests/golden/make_fixtures.py, and EXslabs.egsphsp1.gz).

The reference ran with spin effects on (not restated: the spin data file is
not part of the reference) and the PRESTA-I boundary-crossing algorithm.  The
listing's deposit and fluences are compared for both boundary-crossing
algorithms of the restatement, EXACT and PRESTA-I: in a thin, homogeneous slab
they are set by stopping powers, Moller/bremsstrahlung production and escape.
The step counts depend on the boundary-crossing algorithm and are compared for
PRESTA-I only, with the skin depth that PRESTA-I derives from ECUT.
"""
import json
import os

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import formats as F
from oracle.oracle_binding import Oracle

HERE = os.path.dirname(os.path.abspath(__file__))
GOLD = os.path.join(HERE, "golden")
PEGS700 = os.path.join(eg.DATA_DIR, "700icru.pegs4dat")
J_PER_MEV = 1.602176634e-13


def exslabs_case():
    """The EXslabs geometry (a 20 x 20 cm slab, z from 0.001 to 100.001 cm)
    and source (20 MeV electrons along +z through the origin)."""
    g = eg.XYZGeometry([-10.0, 10.0], [-10.0, 10.0], [0.001, 100.001], 0)
    src = eg.ParallelBeam(charge=-1, energy=20.0, position=(0.0, 0.0, 0.0))
    return g, src


def listing():
    with open(os.path.join(GOLD, "beamnrc_examples.json")) as f:
        return json.load(f)["EXslabs"]


def deposit_reference():
    """Energy deposited in the slab per incident electron (MeV) and its 1-sigma."""
    z = listing()["dose"][0]
    e = z["energy_j"] / J_PER_MEV
    return e, e * z["sigma_pct"] / 100


def exslabs_oracle(bca_algorithm):
    """The oracle set up as EXslabs ran: PRESTA-I takes the default skin depth."""
    return Oracle(["AIR700ICRU"], ecut=1.0, pcut=0.01, pegs_file=PEGS700, bca_algorithm=bca_algorithm,
                  skindepth=0.0 if bca_algorithm else 3.0)


@pytest.fixture(scope="module", params=[0, 1], ids=["exact", "presta1"])
def oracle_run(request):
    g, src = exslabs_case()
    o = exslabs_oracle(request.param)
    o.set_geometry(g)
    o.set_source(src)
    o.set_smax(5.0)
    o.set_escape_log(True)
    n, nb = 200000, 20
    o.run(n, nbatch=nb, seed=2004, threads=8)
    s, s2, tot = o.tallies()
    esc = o.escapes()
    run = (n, nb, s, s2, tot, esc)
    if request.param == 1:
        run += (o.charged_steps(), o.msdist_steps())
    o.close()
    return run


def test_listing_fixture():
    L = listing()
    assert L["histories"] == 1000
    assert L["dose"][0]["mass_g"] == pytest.approx(400 * 100 * 1.205e-3, rel=1e-3)   # the 20x20x100 cm slab
    e, se = deposit_reference()
    assert e == pytest.approx(0.22962, rel=1e-4) and se == pytest.approx(0.0020666, rel=1e-3)


def test_energy_deposit_matches_reference_run(oracle_run):
    n, nb, s, s2, tot, _ = oracle_run[:6]
    m = s[0] / nb
    sig = np.sqrt(max(s2[0] / nb - m * m, 0) / (nb - 1)) * nb / n
    dep = s[0] / n
    e, se = deposit_reference()
    assert abs(dep - e) < 3 * np.hypot(se, sig), (dep, sig, e, se)
    # and the run conserves energy
    assert tot[2] + tot[3] == pytest.approx(20.0 * n, rel=1e-9)


def _back(esc):
    return esc[esc[:, 4] > 100.001 - 1e-6]


def test_back_plane_fluence_matches_listing(oracle_run):
    n, _, _, _, _, esc = oracle_run[:6]
    L = listing()
    r1 = L["plane_radii_cm"][0]
    b = _back(esc)
    el, ph = b[b[:, 0] == -1], b[b[:, 0] == 0]
    r = np.hypot(el[:, 2], el[:, 3])
    z1 = el[r < r1]

    def close(mine, sig_mine, ref):
        v, pct = ref
        return abs(mine - v) < 3 * np.hypot(v * pct / 100, sig_mine)

    pe = L["plane_electrons"]
    k = len(z1) / n
    assert close(k, np.sqrt(k * (1 - k) / n), pe["number"]), k
    assert close(len(el) / n, np.sqrt(len(el)) / n, pe["total_number"])
    emean = z1[:, 1].mean()
    assert close(emean, z1[:, 1].std() / np.sqrt(len(z1)), pe["energy_mev"]), emean
    ang = np.degrees(np.arccos(np.clip(z1[:, 7], -1, 1)))
    assert close(ang.mean(), ang.std() / np.sqrt(len(ang)), pe["angle_deg"]), ang.mean()
    pp = L["plane_photons"]
    assert close(len(ph) / n, np.sqrt(len(ph)) / n, pp["total_number"]), len(ph) / n


def test_exit_electrons_match_reference_phase_space(oracle_run):
    """The electrons leaving the back face against the reference's own phase
    space: the median energy loss (continuous restricted loss over 100 cm of
    air, a spike about 1e-4 MeV wide) to 1e-3, the fraction that lost more
    than 0.3 MeV (a Moller or bremsstrahlung event) within 3 sigma, and
    two-sample Kolmogorov-Smirnov tests of the radius and polar angle."""
    stats = pytest.importorskip("scipy.stats")
    n, _, _, _, _, esc = oracle_run[:6]
    ref, hdr = F.read_egsphsp(os.path.join(GOLD, "EXslabs.egsphsp1.gz"))
    assert hdr["incident"] == 1000
    re_ = ref[ref[:, 0] == -1]
    b = _back(esc)
    el = b[b[:, 0] == -1]
    loss_mine, loss_ref = 20 - np.median(el[:, 1]), 20 - np.median(re_[:, 1])
    assert loss_mine == pytest.approx(loss_ref, rel=1e-3)
    f_mine, f_ref = np.mean(el[:, 1] < 19.7), np.mean(re_[:, 1] < 19.7)
    assert abs(f_mine - f_ref) < 3 * np.sqrt(f_ref / len(re_) + f_mine / len(el))
    pairs = [
        (np.hypot(el[:, 2], el[:, 3]), np.hypot(re_[:, 2], re_[:, 3])),   # radius
        (np.hypot(el[:, 5], el[:, 6]), np.hypot(re_[:, 4], re_[:, 5])),   # sine of the polar angle
    ]
    for mine, theirs in pairs:
        assert stats.ks_2samp(mine, theirs).pvalue > 1e-3


def test_presta1_default_skindepth_is_the_listings():
    """PRESTA-I with no skin depth given: the old PRESTA minimum step from the
    lowest ECUT, which the listing prints (910.8 elastic MFPs)."""
    assert exslabs_oracle(1).skindepth() == pytest.approx(listing()["skindepth_mfp"], abs=0.05)
    assert exslabs_oracle(0).skindepth() == 3.0


def test_presta1_step_counts_match_listing(oracle_run):
    """Charged-particle steps per history (21.22 +- 0.3%) and their PRESTA-II
    fraction (0.859 +- 0.3%) as the reference counted them (AUSGAB(0) calls,
    msdist_pII calls).  The restatement gives 0.8-0.9% fewer of both, which
    this test allows: the listing comes from the EGSnrc of 2004 with spin
    effects on."""
    if len(oracle_run) < 8:
        pytest.skip("step counts are compared for PRESTA-I")
    n, steps, msdist = oracle_run[0], oracle_run[6], oracle_run[7]
    L = listing()
    assert steps / n == pytest.approx(L["charged_steps_per_history"]["value"], rel=0.015)
    assert msdist / steps == pytest.approx(L["presta2_step_fraction"]["value"], rel=0.015)
