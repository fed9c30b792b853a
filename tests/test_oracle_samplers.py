"""The restatement's photon-interaction samplers against the analytic
distributions they sample (chi-square goodness of fit, p > 1e-3).

The engine's FP64 build draws the same random numbers as the oracle and
follows it history by history (tests/test_gpu_parity.py), so these checks
pin the GPU samplers too.

* Klein-Nishina (COMPT's sampler without binding, src/egsnrc.mortran:552-640):
  epsilon = k'/k on [1/(1 + 2k), 1] with
  dsigma/depsilon ~ 1/epsilon + epsilon - sin^2(theta),
  cos(theta) = 1 - (1 - epsilon)/(k epsilon), k in electron rest energies;
  both sampling regimes (k <= 2 and k > 2).
* Sauter's K-shell photo-electron distribution ($SELECT-PHOTOELECTRON-
  DIRECTION, src/egsnrc.macros:1916-1955):
  dsigma/dcos ~ (1 - c^2)/(1 - beta c)^4 [1 + gamma (gamma - 1)(gamma - 2)(1 - beta c)/2].
* Bethe-Heitler pair energy split (PAIR, src/egsnrc.mortran:4518-4715):
  with b = (E- - m)/(E - 2m) folded to [0, 1/2] and delta = delcm E / (E- E+) as
  PAIR forms it, dsigma/db ~ (1 - 2m/E)^2 (1 - 2b)^2 A(delta) + B(delta), A and B the
  PEGS4 screening fits dl1..dl6 (l = 4, 5) of the medium, each taken as 0 where
  its fit is negative (large delta near threshold).
"""
import numpy as np
import pytest
from scipy import integrate
from scipy.stats import chi2 as chi2_dist

from oracle.oracle_binding import Oracle

RM = 0.5109989461
N = 200000


@pytest.fixture(scope="module")
def ora():
    o = Oracle(["H2O521ICRU", "ICRPBONE521ICRU"], ecut=0.521, pcut=0.01)
    yield o
    o.close()


def gof(samples, pdf, lo, hi, nbins=60):
    """Chi-square of the histogram of samples against pdf (unnormalised) on
    [lo, hi]; bins with fewer than 20 expected counts are merged."""
    edges = np.linspace(lo, hi, nbins + 1)
    w = np.array([integrate.quad(pdf, a, b, limit=200)[0] for a, b in zip(edges[:-1], edges[1:])])
    exp = w / w.sum() * len(samples)
    obs, _ = np.histogram(samples, bins=edges)
    assert obs.sum() == len(samples)
    oo, ee = [], []
    o_acc = e_acc = 0.0
    for o, e in zip(obs, exp):
        o_acc += o
        e_acc += e
        if e_acc >= 20:
            oo.append(o_acc)
            ee.append(e_acc)
            o_acc = e_acc = 0.0
    if e_acc > 0:
        oo[-1] += o_acc
        ee[-1] += e_acc
    oo, ee = np.array(oo), np.array(ee)
    stat = float(((oo - ee) ** 2 / ee).sum())
    dof = len(oo) - 1
    return stat, dof, float(chi2_dist.sf(stat, dof))


@pytest.mark.parametrize("energy", [0.1, 0.8, 5.0, 20.0])
def test_klein_nishina(ora, energy):
    k = energy / RM
    s = ora.sample_interaction(0, 0, energy, N, seed=3)
    eps, cost = s[:, 0], s[:, 1]
    emin = 1.0 / (1.0 + 2.0 * k)
    assert eps.min() >= emin * (1 - 1e-12) and eps.max() <= 1 + 1e-12
    # the photon direction follows from epsilon (the beam was along +z)
    assert np.allclose(cost, 1 - (1 - eps) / (k * eps), atol=1e-9)

    def pdf(e):
        c = 1 - (1 - e) / (k * e)
        return 1 / e + e - (1 - c * c)
    stat, dof, p = gof(eps, pdf, emin, 1.0)
    assert p > 1e-3, (energy, stat, dof, p)


@pytest.mark.parametrize("kinetic", [0.02, 0.1, 0.5, 2.0])
def test_sauter_photoelectron_direction(ora, kinetic):
    E = kinetic + RM
    gamma = E / RM
    beta = np.sqrt(1 - 1 / gamma ** 2)
    c = ora.sample_interaction(2, 0, E, N, seed=4)[:, 0]
    assert c.min() >= -1 - 1e-12 and c.max() <= 1 + 1e-12

    def pdf(x):
        return (1 - x * x) / (1 - beta * x) ** 4 * (1 + 0.5 * gamma * (gamma - 1) * (gamma - 2) * (1 - beta * x))
    stat, dof, p = gof(c, pdf, -1.0, 1.0, nbins=80)
    assert p > 1e-3, (kinetic, stat, dof, p)


@pytest.mark.parametrize("med,energy", [(0, 3.0), (0, 10.0), (1, 6.0), (1, 40.0)])
def test_bethe_heitler_pair_split(ora, med, energy):
    dl, delcm, bpar = ora.pair_constants(med)
    s = ora.sample_interaction(3, med, energy, N, seed=5)
    em, ep = s[:, 0], s[:, 1]
    assert np.allclose(em + ep, energy, rtol=1e-12)
    avail = energy - 2 * RM
    b = (em - RM) / avail
    b = np.minimum(b, 1 - b)   # PAIR samples the smaller share and assigns the charges at random
    # both shares occur as the electron's: the charge assignment is symmetric
    frac_low = np.mean((em - RM) / avail < 0.5)
    assert abs(frac_low - 0.5) < 5 * np.sqrt(0.25 / N)

    def screen(l, delta):
        if delta < 1:
            return dl[0][l] + delta * (dl[1][l] + delta * dl[2][l])
        return dl[3][l] + dl[4][l] * np.log(delta + dl[5][l])

    c = (1 - 2 * RM / energy) ** 2

    def pdf(x):
        e_minus = x * avail + RM
        delta = energy * delcm / (e_minus * (energy - e_minus))
        # a rejection sampler cannot produce negative density: where a fit
        # turns negative (large delta: asymmetric splits near threshold) that
        # part contributes nothing
        return c * (1 - 2 * x) ** 2 * max(screen(4, delta), 0.0) + max(screen(5, delta), 0.0)
    stat, dof, p = gof(b, pdf, 0.0, 0.5)
    assert p > 1e-3, (med, energy, stat, dof, p)


def test_bound_compton_limits(ora):
    # binding shifts energy to the shells and suppresses forward scattering,
    # but at 5 MeV the mean k'/k is Klein-Nishina's within 0.2%
    kn = ora.sample_interaction(0, 0, 5.0, N, seed=6)
    bd = ora.sample_interaction(1, 0, 5.0, N, seed=6)
    assert abs(bd[:, 0].mean() / kn[:, 0].mean() - 1) < 2e-3
    assert np.all(bd[:, 2] >= 0) and bd[:, 2].max() < 1e-3   # water: O K shell 0.54 keV
