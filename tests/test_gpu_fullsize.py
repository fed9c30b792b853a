"""The configured workloads at their full phantom sizes (c1 water30 30^3, c2 slab64
64^3, c3 water128e 128^3, c4 batched64 with 64 phantoms of 32^3-160^3, c5
perturbed64 64^3), through the C ABI.

The parity tests compare with the oracle on reduced phantoms; here the full
phantoms are checked through properties that do not depend on the number of
histories:
  * FP64 history by history against the oracle for a few hundred histories.
    Neither side fuses multiply-adds, but log/exp can differ in the last ulp
    between the GPU and the host; steps limited by the distance to the
    nearest voxel face feed a position difference into the next step length,
    so a 20 MeV electron track in 0.2 cm voxels amplifies it by about 2% per
    step until a branch decision flips and the history forks.  In 128^3 voxels
    about 3% of the 20 MeV electron histories fork (none in 0.4 or 0.8 cm
    voxels); a forked history is as valid a sample as the oracle's, so the
    energy deposited per history must still agree on average;
  * energy conservation of an FP32 run: deposited + escaped = source energy;
  * the tallies do not depend on how histories are chunked into wavefronts;
  * (c4) every phantom of the batched run equals a run of its own.
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle

pytestmark = pytest.mark.gpu

FULL = ["water30", "slab64", "water128e", "perturbed64"]
NHIST = {"water30": 400, "slab64": 400, "water128e": 200, "perturbed64": 300}
MATCH = {"water30": 0.97, "slab64": 0.97, "water128e": 0.9, "perturbed64": 0.97}


def engine(wl, precision, **cfg):
    e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=precision, **cfg)
    e.set_geometry(wl["geometry"])
    e.set_source(wl["source"])
    return e


def source_energy(src):
    s = src.s
    return None if s.spectrum else s.energy + (2 * eg.RM if s.charge > 0 else 0.0)


@pytest.mark.parametrize("name", FULL)
def test_full_size_history_by_history_fp64(name):
    wl = W.WORKLOADS[name]()
    n = NHIST[name]
    e = engine(wl, 64)
    o = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
    o.set_geometry(wl["geometry"])
    o.set_source(wl["source"])
    e.set_history_tally(0, n)
    o.set_history_tally(0, n)
    e.run(n, nbatch=1, seed=17)
    o.run(n, nbatch=1, seed=17, threads=8)
    hg, ho = e.history_tally(), o.history_tally()
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    assert np.mean(rel < 1e-6) >= MATCH[name] and ho.sum() > 0
    assert hg.mean() == pytest.approx(ho.mean(), rel=0.02)
    e.close()
    o.close()


@pytest.mark.parametrize("name", FULL)
def test_full_size_energy_conservation_and_chunking_fp32(name):
    wl = W.WORKLOADS[name]()
    n = 200000 if name != "water128e" else 20000
    res = []
    for chunk in (0, n // 7 + 1):
        e = engine(wl, 32, chunk=chunk)
        e.run(n, nbatch=4, seed=5)
        s, s2, _ = e.tallies()
        t = e.totals()
        e0 = source_energy(wl["source"])
        if e0 is not None:
            assert t["deposited"] + t["escaped"] == pytest.approx(n * e0, rel=1e-6)
        assert s.sum() == pytest.approx(t["deposited"], rel=1e-6)
        res.append(s)
        e.close()
    # FP32 transport, FP64 tallies: chunking changes only the order of the atomic sums
    assert np.allclose(res[0], res[1], rtol=2e-5, atol=2e-5 * res[0].max())


def test_full_size_batched_phantoms_match_separate_runs():
    wl = W.batched64(scale=2e-4)
    ps = wl["problems"]
    e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=64)
    e.set_phantoms(ps)
    e.run_phantoms(nbatch=2)
    for k in (0, 17, 63):
        got, got2 = e.phantom_tallies(k)
        p = ps[k]
        one = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=64)
        one.set_geometry(p["geometry"])
        one.set_source(p["source"])
        one.run(p["histories"], nbatch=2, seed=p["seed"])
        want, want2, _ = one.tallies()
        assert np.allclose(got, want, rtol=1e-12, atol=1e-12 * want.max())
        assert np.allclose(got2, want2, rtol=1e-12, atol=1e-12 * want2.max())
        one.close()
    e.close()
