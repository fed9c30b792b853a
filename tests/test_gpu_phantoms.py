"""Several phantoms in one run (egsgpu_set_phantoms / egsgpu_run_phantoms).

Every phantom keeps its own geometry, source, Philox seed and history count,
so its tallies must equal those of a run of its own with the same seed,
histories and batch count: the histories consume the same random numbers in
the same local coordinates, and only the order of the FP64 atomic additions
differs.  The phantoms are small versions of the batched workload (Gaussian
random-field densities over four media, photon or electron beams of 1-18 MeV).
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def small_phantoms(n=5):
    ph = [W.batch_problem(k, edge=(8, 20), hist=(300, 3000)) for k in range(n)]
    # one phantom with a histogram spectrum and a pencil (point) beam
    edges = np.linspace(0.1, 6.0, 41)
    ph[1]["source"] = eg.ParallelBeam(charge=0, spectrum=(edges, 1.0 / edges[1:] * (1 - edges[1:] / 6.0 + 1e-3)),
                                      position=(0.05, -0.03, -1.0))
    return ph


def engine(precision):
    return eg.DoseEngine(W.BATCH_MEDIA, ecut=0.7, pcut=0.01, precision=precision)


@pytest.mark.parametrize("precision", [64, 32])
def test_phantoms_match_separate_runs(precision):
    ph = small_phantoms()
    nb = 3
    eng = engine(precision)
    eng.set_phantoms(ph)
    eng.run_phantoms(nbatch=nb)     # histories [0, n_k) of every phantom
    eng.run_phantoms(nbatch=nb)     # then [n_k, 2 n_k)
    tol = 1e-12 if precision == 64 else 2e-5
    for k, p in enumerate(ph):
        s, s2 = eng.phantom_tallies(k)
        one = engine(precision)
        one.set_geometry(p["geometry"])
        one.set_source(p["source"])
        one.run(p["histories"], nbatch=nb, seed=p["seed"])
        one.run(p["histories"], nbatch=nb, seed=p["seed"], first=p["histories"])
        r, r2, _ = one.tallies()
        assert r.sum() > 0
        assert np.allclose(s, r, rtol=tol, atol=tol * r.max()), (k, np.abs(s - r).max())
        assert np.allclose(s2, r2, rtol=tol, atol=tol * r2.max()), k
        d, sd = eng.phantom_dose(k)
        d1, sd1 = one.dose()
        assert np.allclose(d, d1, rtol=1e-9, atol=1e-9 * d1.max())
        assert np.allclose(sd, sd1, rtol=1e-6, atol=1e-6 * sd1.max() + 1e-300)
        one.close()
    eng.close()


def test_phantom_bookkeeping_and_modes():
    ph = small_phantoms(3)
    eng = engine(32)
    eng.set_phantoms(ph)
    off = 0
    for k, p in enumerate(ph):
        assert eng.phantom_info(k) == (off, p["geometry"].nvox, 0)
        off += p["geometry"].nvox
    eng.run_phantoms(nbatch=2)
    eng.run_phantoms(nbatch=2)
    assert [eng.phantom_info(k)[2] for k in range(3)] == [2 * p["histories"] for p in ph]
    # single-phantom calls are refused while several phantoms are set
    with pytest.raises(eg.EGSError) as ex:
        eng.run(100, nbatch=1)
    assert ex.value.code == 7
    with pytest.raises(eg.EGSError):
        eng.run_phantoms(nbatch=10 ** 6)     # more batches than histories
    # a single geometry switches back
    eng.set_geometry(ph[0]["geometry"])
    eng.set_source(ph[0]["source"])
    eng.run(200, nbatch=2, seed=3)
    assert eng.tallies()[0].sum() > 0
    eng.close()


def test_phantoms_energy_conservation():
    ph = [W.batch_problem(k, edge=(8, 16), hist=(500, 1500)) for k in range(4)]
    for p in ph:
        # a field inside the phantom's face, so that every source particle enters
        s = p["source"].s
        h = 0.4 * (p["geometry"].xb[-1] - p["geometry"].xb[0])
        p["source"] = eg.ParallelBeam(charge=s.charge, energy=s.energy, position=(0.0, 0.0, -1.0),
                                      rectangle=(-h, h, -h, h))
    eng = engine(64)
    eng.set_phantoms(ph)
    eng.run_phantoms(nbatch=2)
    t = eng.totals()
    e0 = sum(p["histories"] * (p["source"].s.energy + (2 * eg.RM if p["source"].s.charge > 0 else 0.0)) for p in ph)
    assert abs(t["deposited"] + t["escaped"] - e0) < 1e-9 * e0
    eng.close()
