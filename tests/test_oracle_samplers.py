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
* Moller (MOLLER, src/egsnrc.mortran:2599-2746), the energy fraction eps of
  the delta ray, eps in [te/T, 1/2], t = T/m:
  dsigma/deps ~ 1/eps^2 + 1/(1 - eps)^2 + (t/(t+1))^2 - (2t+1)/(t+1)^2 / (eps (1 - eps)).
* Bhabha (BHABHA, :229-307), the energy fraction eps of the electron before
  the swap, eps in [te/T, 1], y = 1/(gamma + 1):
  dsigma/deps ~ (1/eps^2) [1/beta^2 - B1 eps + B2 eps^2 - B3 eps^3 + B4 eps^4],
  B1 = 2 - y^2, B2 = (1 - 2y)(3 + y^2), B3 = (1 - 2y)^2 (2 - 2y), B4 = (1 - 2y)^3.
* Bethe-Heitler bremsstrahlung (BREMS, :312-524), photon energy k in [AP, T]:
  dsigma/dk ~ (1/k) [(1 + (E'/E)^2) phi1(delta) - (2/3)(E'/E) phi2(delta)],
  E' = E - k, delta = k delcm / (E E'), phi1, phi2 the PEGS4 screening fits
  of the medium (columns 0, 1 below 50 MeV, 2, 3 above); the bracket is
  taken as 0 where the fits make it negative (a rejection sampler cannot
  produce negative density).
* Two-photon annihilation in flight (ANNIH, :70-182; Heitler), positron of
  total energy gamma m on an electron at rest, photon energy fractions eps
  and 1 - eps of (gamma + 1) m, the smaller one folded to [eps0, 1/2]:
  dsigma/deps ~ S(eps) + S(1 - eps), S(e) = -(gamma+1)^2 + (gamma^2 + 4 gamma + 1)/e - 1/e^2,
  eps0 = (1 - sqrt((gamma - 1)/(gamma + 1)))/2.
* Rayleigh scattering (egs_rayleigh_sampling, src/egsnrc.mortran:8559-8590,
  prepare_rayleigh_data :8593-8726), photon of energy E:
  dsigma/dcos ~ (1 + cos^2) F^2(x), x = E sin(theta/2)/hc, with F^2 the
  independent-atom molecular form factor sum p_i F_i^2 of the medium's
  elements from pgs4form.dat, interpolated as a power law in x between the
  tabulated points as PEGS does.
Each is histogrammed in the variable in which its sampler's proposal is
uniform (1/eps, log k, or the cumulative of F^2 in x^2), so that the bins are
populated evenly.
"""
import os

import numpy as np
import pytest
from scipy import integrate
from scipy.stats import chi2 as chi2_dist

from oracle.oracle_binding import Oracle

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

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


@pytest.mark.parametrize("kinetic", [0.1, 1.0, 10.0])
def test_moller_delta_ray_energy(ora, kinetic):
    te, thmoll, _ = ora.thresholds(0)
    t = kinetic / RM
    e_min = te / kinetic
    eps = ora.sample_interaction(4, 0, kinetic + RM, N, seed=7)[:, 0]
    assert eps.min() >= e_min * (1 - 1e-12) and eps.max() <= 0.5 + 1e-12
    a = 1 / e_min - 2   # y = (1/e_min - 1/eps) / a is uniform under the 1/eps^2 proposal

    def pdf(y):
        e = 1 / (1 / e_min - a * y)
        f = 1 / e ** 2 + 1 / (1 - e) ** 2 + (t / (t + 1)) ** 2 - (2 * t + 1) / (t + 1) ** 2 / (e * (1 - e))
        return f * e * e
    stat, dof, p = gof((1 / e_min - 1 / eps) / a, pdf, 0.0, 1.0)
    assert p > 1e-3, (kinetic, stat, dof, p)


@pytest.mark.parametrize("kinetic", [0.1, 1.0, 10.0])
def test_bhabha_electron_energy(ora, kinetic):
    te, _, _ = ora.thresholds(0)
    gamma = kinetic / RM + 1
    beta2 = 1 - 1 / gamma ** 2
    y = 1 / (gamma + 1)
    b1, b2 = 2 - y * y, (1 - 2 * y) * (3 + y * y)
    b3, b4 = (1 - 2 * y) ** 2 * (2 - 2 * y), (1 - 2 * y) ** 3
    e_min = te / kinetic
    eps = ora.sample_interaction(5, 0, kinetic + RM, N, seed=8)[:, 0]
    assert eps.min() >= e_min * (1 - 1e-12) and eps.max() <= 1 + 1e-12
    a = 1 / e_min - 1

    def pdf(u):
        e = 1 / (1 / e_min - a * u)
        f = (1 / beta2 - b1 * e + b2 * e ** 2 - b3 * e ** 3 + b4 * e ** 4) / e ** 2
        return f * e * e
    stat, dof, p = gof((1 / e_min - 1 / eps) / a, pdf, 0.0, 1.0)
    assert p > 1e-3, (kinetic, stat, dof, p)


@pytest.mark.parametrize("med,kinetic", [(0, 1.0), (0, 5.0), (1, 20.0), (0, 60.0)])
def test_bremsstrahlung_photon_energy(ora, med, kinetic):
    dl, delcm, _ = ora.pair_constants(med)
    _, _, ap = ora.thresholds(med)
    E = kinetic + RM
    l, l1 = (0, 1) if E < 50 else (2, 3)
    k = ora.sample_interaction(6, med, E, N, seed=9)[:, 0]
    assert k.min() >= ap * (1 - 1e-12) and k.max() <= kinetic * (1 + 1e-12)
    span = np.log(kinetic / ap)   # y = log(k/ap)/span is uniform under the 1/k proposal

    def phi(col, delta):
        if delta < 1:
            return dl[0][col] + delta * (dl[1][col] + delta * dl[2][col])
        return dl[3][l] + dl[4][l] * np.log(delta + dl[5][l])

    def pdf(y):
        kk = ap * np.exp(y * span)
        ep = E - kk
        delta = kk * delcm / (E * ep)
        aux = ep / E
        return max((1 + aux * aux) * phi(l, delta) - 2 * aux * phi(l1, delta) / 3, 0.0)
    stat, dof, p = gof(np.log(k / ap) / span, pdf, 0.0, 1.0)
    assert p > 1e-3, (med, kinetic, stat, dof, p)


HC_INV = 80.65506856998   # 1/(hc) in 1/(MeV Angstrom), as egs_rayleigh_sampling has it
TWICE_HC2 = 0.000307444456


def molecular_form_factor(z, pz):
    """Grid x (1/Angstrom) and F(x) = sqrt(sum_i p_i F_i(x)^2) from the raw
    pgs4form.dat (100 x values, then 100 values per element Z = 1..100)."""
    vals = np.array(open(os.path.join(ROOT, "egsnrc_gb300", "data", "pgs4form.dat")).read().split(), dtype=float)
    x = vals[:100].copy()
    aff = vals[100:100 + 100 * 100].reshape(100, 100)
    f = np.sqrt(sum(p * aff[int(zz) - 1] ** 2 for zz, p in zip(z, pz)))
    if x[0] < 1e-6:
        x[0] = 1e-4
    f[f == 0] = 1e-30
    return x, f


@pytest.mark.parametrize("med,energy", [(0, 0.02), (0, 0.05), (0, 0.1), (0, 0.5), (1, 0.03), (1, 0.1)])
def test_rayleigh_angle(ora, med, energy):
    z, pz = ora.elements(med)
    x, f = molecular_form_factor(z, pz)
    b = np.log(f[1:] / f[:-1]) / np.log(x[1:] / x[:-1])   # F = f_i (x/x_i)^b_i on [x_i, x_i+1)
    coef = f[:-1] ** 2 * x[:-1] ** (-2 * b) / (b + 1)
    cum = np.concatenate([[0.0], np.cumsum(coef * (x[1:] ** (2 * b + 2) - x[:-1] ** (2 * b + 2)))])

    def cdf(xx):   # integral of F^2 d(x^2) from x_0 to xx
        i = np.clip(np.searchsorted(x, xx, side="right") - 1, 0, len(b) - 1)
        return cum[i] + coef[i] * (xx ** (2 * b[i] + 2) - x[i] ** (2 * b[i] + 2))

    def inverse(pp):
        i = np.clip(np.searchsorted(cum, pp, side="right") - 1, 0, len(b) - 1)
        return (x[i] ** (2 * b[i] + 2) + (pp - cum[i]) / coef[i]) ** (1 / (2 * b[i] + 2))

    xmax = HC_INV * energy
    ptot = cdf(xmax)
    c = ora.sample_interaction(7, med, energy, N, seed=10)[:, 0]
    assert c.min() >= -1 - 1e-12 and c.max() <= 1 + 1e-12
    xs = energy * np.sqrt(np.maximum(1 - c, 0) / TWICE_HC2)
    t = cdf(xs) / ptot   # uniform under the F^2 proposal

    def pdf(u):
        xx = inverse(u * ptot)
        cc = 1 - TWICE_HC2 * (xx / energy) ** 2
        return 1 + cc * cc
    stat, dof, p = gof(t, pdf, 0.0, 1.0)
    assert p > 1e-3, (med, energy, stat, dof, p)


@pytest.mark.parametrize("kinetic", [0.1, 1.0, 10.0])
def test_annihilation_in_flight_photon_energy(ora, kinetic):
    gamma = kinetic / RM + 1
    eps0 = 0.5 * (1 - np.sqrt((gamma - 1) / (gamma + 1)))
    eps = ora.sample_interaction(8, 0, kinetic + RM, N, seed=11)[:, 0]
    assert eps.min() >= eps0 * (1 - 1e-9) and eps.max() <= (1 - eps0) * (1 + 1e-9)
    e = np.minimum(eps, 1 - eps)
    span = np.log(0.5 / eps0)   # y = log(e/eps0)/span: the 1/e proposal, folded

    def s(v):
        return -(gamma + 1) ** 2 + (gamma ** 2 + 4 * gamma + 1) / v - 1 / v ** 2

    def pdf(y):
        v = eps0 * np.exp(y * span)
        return (s(v) + s(1 - v)) * v
    stat, dof, p = gof(np.log(e / eps0) / span, pdf, 0.0, 1.0)
    assert p > 1e-3, (kinetic, stat, dof, p)
