"""The CUDA engine on BEAMnrc's EXslabs example, through the C ABI.

EXslabs is the reference's own run of 20 MeV electrons through a 100 cm air
slab (AIR700ICRU, ECUT 1.0, PCUT 0.01, SMAX 5 cm, PRESTA-I boundary crossing);
its listing gives the energy deposited in the slab per incident electron,
0.2296 MeV +- 0.9%.  tests/test_oracle_exslabs.py holds the oracle to the same
listing.  Here, for EXACT and PRESTA-I boundary crossing:
  * FP64, history by history against the oracle (700 keV media and the SMAX
    step limit on both sides);
  * FP32 and FP64, the deposited energy of 1e6 histories against the listing;
and PRESTA-I history by history in a voxel phantom, where most electron steps
end near a voxel face.
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle
from test_oracle_exslabs import PEGS700, deposit_reference, exslabs_case, exslabs_oracle

pytestmark = pytest.mark.gpu

BCA = pytest.mark.parametrize("bca", [0, 1], ids=["exact", "presta1"])


def engine(precision, bca):
    g, src = exslabs_case()
    e = eg.DoseEngine(["AIR700ICRU"], pegs_file=PEGS700, ecut=1.0, pcut=0.01, smax=5.0, precision=precision,
                      bca_algorithm=bca, skindepth=0.0 if bca else 3.0)
    e.set_geometry(g)
    e.set_source(src)
    return e


def by_history(e, o, n, seed):
    e.set_history_tally(0, n)
    o.set_history_tally(0, n)
    e.run(n, nbatch=2, seed=seed)
    o.run(n, nbatch=2, seed=seed)
    hg, ho = e.history_tally(), o.history_tally()
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    return np.mean(rel < 1e-6), ho


@BCA
def test_history_by_history_fp64(bca):
    n = 2000
    e = engine(64, bca)
    g, src = exslabs_case()
    o = exslabs_oracle(bca)
    o.set_geometry(g)
    o.set_source(src)
    o.set_smax(5.0)
    match, _ = by_history(e, o, n, seed=13)
    assert match >= 0.97
    # the same step count: SMAX and the boundary-crossing algorithm reached the kernels
    assert e.totals()["electron_steps"] == pytest.approx(o.tallies()[2][6], rel=0.02)
    e.close()
    o.close()


@BCA
@pytest.mark.parametrize("precision", [32, 64])
def test_energy_deposit_matches_reference_run(precision, bca):
    n, nb = 1000000, 20
    e = engine(precision, bca)
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


@pytest.mark.parametrize("charge,energy", [(-1, 5.0), (1, 3.0), (0, 6.0)])
def test_presta1_voxels_history_by_history_fp64(charge, energy):
    """PRESTA-I in 0.25 cm voxels of three media, default skin depth."""
    med = (np.arange(16 ** 3) % 3).astype(np.int32)
    g = W.centred_geometry(16, 0.25, med)
    src = eg.ParallelBeam(charge=charge, energy=energy, position=(0.1, -0.1, -1.0), direction=(0.2, 0.1, 1.0),
                          rectangle=(-1, 1, -1, 1))
    media = [W.WATER, W.LUNG, W.BONE]
    e = eg.DoseEngine(media, ecut=0.521, pcut=0.01, precision=64, bca_algorithm=1, skindepth=0.0)
    e.set_geometry(g)
    e.set_source(src)
    o = Oracle(media, ecut=0.521, pcut=0.01, bca_algorithm=1, skindepth=0.0)
    o.set_geometry(g)
    o.set_source(src)
    match, ho = by_history(e, o, 1000, seed=21)
    assert match >= 0.97 and ho.sum() > 0
    e.close()
    o.close()


def test_presta1_refused_where_it_has_no_kernel():
    e = eg.DoseEngine([W.WATER], ecut=0.521, pcut=0.01, bca_algorithm=1, skindepth=0.0)
    e.set_geometry(W.centred_geometry(8, 0.5))
    e.set_source(eg.ParallelBeam(charge=-1, energy=2.0, position=(0, 0, -1)))
    e.run(100, nbatch=1, seed=1)
    with pytest.raises(eg.EGSError) as ex:
        e.adjoint(np.ones(8 ** 3), 100, seed=1)
    assert "PRESTA-I" in str(ex.value)
    e.close()
    with pytest.raises(eg.EGSError):
        eg.DoseEngine([W.WATER], bca_algorithm=2)


def test_presta1_phantoms_match_separate_runs():
    """PRESTA-I with several phantoms per run: each equals a run of its own."""
    media = [W.WATER, W.LUNG, W.BONE]
    ps = []
    for k, (n, q, en) in enumerate(((10, -1, 4.0), (14, 0, 3.0))):
        g = W.centred_geometry(n, 0.3, (np.arange(n ** 3) % 3).astype(np.int32))
        src = eg.ParallelBeam(charge=q, energy=en, position=(0.0, 0.0, -1.0), rectangle=(-1, 1, -1, 1))
        ps.append(dict(geometry=g, source=src, seed=31 + k, histories=600))
    kw = dict(ecut=0.521, pcut=0.01, precision=64, bca_algorithm=1, skindepth=0.0)
    e = eg.DoseEngine(media, **kw)
    e.set_phantoms(ps)
    e.run_phantoms(nbatch=2)
    for k, p in enumerate(ps):
        s, s2 = e.phantom_tallies(k)
        one = eg.DoseEngine(media, **kw)
        one.set_geometry(p["geometry"])
        one.set_source(p["source"])
        one.run(p["histories"], nbatch=2, seed=p["seed"])
        r, r2, _ = one.tallies()
        assert r.sum() > 0
        assert np.allclose(s, r, rtol=1e-12, atol=1e-12 * r.max())
        assert np.allclose(s2, r2, rtol=1e-12, atol=1e-12 * r2.max())
        one.close()
    e.close()
