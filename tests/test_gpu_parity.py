"""GPU parity: the CUDA engine (through the C ABI) against the FP64 CPU oracle.

Three levels, following the reference's lack of transport golden values:
  * history by history: with Philox streams keyed by (seed, history) the FP64
    GPU build and the oracle consume identical random numbers, so per-history
    deposited energies agree to rounding except where a last-ulp difference in
    a transcendental flips a rejection test;
  * statistically (tests/test_gpu_statistical.py): voxel doses and total
    deposited energy against the oracle at the workloads' full sizes;
  * precision: FP32 against FP64 with common random numbers, paired batch
    by batch, so that a bias of the FP32 arithmetic shows at a level far
    below the statistical noise of either run;
  * exactly: energy conservation per run, and independence of the results
    from the chunking of histories into wavefronts.
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle

pytestmark = pytest.mark.gpu

RM = eg.RM


def make_pair(wl, precision=64, **cfg):
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=precision, **cfg)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    ora = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
    ora.set_geometry(wl["geometry"])
    ora.set_source(wl["source"])
    return eng, ora


def source_energy(src):
    s = src.s
    if s.spectrum:
        return None
    return s.energy + (2 * RM if s.charge > 0 else 0.0)


def small_cases():
    # reduced-size versions of the benchmark problems plus positron / bone cases
    g = W.centred_geometry(20, 1.0)
    yield "water_photon_2MeV", W.water30(20)
    yield "slab_spectrum", dict(W.slab64(32), histories=0)
    yield "water_electron_20MeV", dict(W.water128e(32), histories=0)
    yield "perturbed_photon_6MeV", dict(W.perturbed64(24), histories=0)
    yield "water_positron_5MeV", dict(name="pos", media=[W.WATER], ecut=0.521, pcut=0.01, geometry=g,
                                      source=eg.ParallelBeam(charge=1, energy=5.0, position=(0.2, -0.3, -1.0)))
    med = (np.arange(20 ** 3) % 4).astype(np.int32)
    yield "mixed_media_electron", dict(name="mix", media=[W.WATER, W.LUNG, W.BONE, W.TISSUE], ecut=0.521,
                                       pcut=0.01, geometry=W.centred_geometry(20, 0.5, med),
                                       source=eg.ParallelBeam(charge=-1, energy=3.0, position=(0.1, 0.1, -1.0),
                                                              direction=(0.1, 0.2, 1.0)))


CASES = list(small_cases())
NHIST = {"water_photon_2MeV": 3000, "slab_spectrum": 3000, "water_electron_20MeV": 300,
         "perturbed_photon_6MeV": 2000, "water_positron_5MeV": 1000, "mixed_media_electron": 1000}


@pytest.mark.parametrize("name,wl", CASES, ids=[c[0] for c in CASES])
def test_history_by_history_fp64(name, wl):
    n = NHIST[name]
    eng, ora = make_pair(wl, precision=64)
    eng.set_history_tally(0, n)
    ora.set_history_tally(0, n)
    eng.run(n, nbatch=2, seed=7)
    ora.run(n, nbatch=2, seed=7)
    hg, ho = eng.history_tally(), ora.history_tally()
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    match = np.mean(rel < 1e-6)
    assert match >= 0.97, "only %.3f of histories agree to 1e-6 (%s)" % (match, name)
    # totals: deposited + escaped conserve the source energy
    t = eng.totals()
    e0 = source_energy(wl["source"])
    if e0 is not None:
        assert abs(t["deposited"] + t["escaped"] - n * e0) < 1e-8 * n * e0


@pytest.mark.parametrize("name", ["water_photon_2MeV", "water_electron_20MeV", "slab_spectrum"])
def test_fp32_against_fp64_common_random_numbers(name):
    wl = dict(CASES)[name]
    nh = {"water_photon_2MeV": 40000, "water_electron_20MeV": 4000, "slab_spectrum": 40000}[name]
    nb = 20
    batches = {}
    for prec in (32, 64):
        eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=prec)
        eng.set_geometry(wl["geometry"])
        eng.set_source(wl["source"])
        prev = np.zeros(wl["geometry"].nvox)
        out = []
        for b in range(nb):
            eng.run(nh, nbatch=1, seed=21, first=b * nh)
            s, _, _ = eng.tallies()
            out.append(s - prev)
            prev = s
        batches[prec] = np.array(out)
    d = batches[32] - batches[64]
    ref = batches[64].mean(axis=0)
    sel = ref > 0.1 * ref.max()
    md, sd = d.mean(axis=0)[sel], d.std(axis=0, ddof=1)[sel]
    z = np.where(sd > 0, md / np.maximum(sd / np.sqrt(nb), 1e-300), 0.0)
    frac3, chi2 = np.mean(np.abs(z) < 3), np.mean(z * z)
    tot_rel = abs(d.sum()) / batches[64].sum()
    assert frac3 >= 0.98 and chi2 < 1.5, (name, frac3, chi2)
    assert tot_rel < 2e-3, (name, tot_rel)


@pytest.mark.parametrize("precision", [32, 64])
def test_energy_conservation(precision):
    wl = W.water128e(32)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    n = 2000
    eng.run(n, nbatch=4, seed=5)
    t = eng.totals()
    e0 = 20.0
    tol = 1e-9 if precision == 64 else 2e-4
    assert abs(t["deposited"] + t["escaped"] - n * e0) < tol * n * e0
    s, _, _ = eng.tallies()
    assert abs(s.sum() - t["deposited"]) < (1e-9 if precision == 64 else 1e-6) * t["deposited"]


def test_autotuned_chunks_cover_every_history():
    # a small queue capacity makes the autotuner start with tiny chunks and
    # grow them many times within one batch; every history must be run once
    wl = W.water30(10)
    n = 60000
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=64, capacity=1 << 15)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    eng.set_history_tally(0, n)
    eng.run(n, nbatch=3, seed=8)
    t = eng.totals()
    assert t["histories"] == n
    assert abs(t["deposited"] + t["escaped"] - 2.0 * n) < 1e-8 * n
    ref = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=64, chunk=n)
    ref.set_geometry(wl["geometry"])
    ref.set_source(wl["source"])
    ref.set_history_tally(0, n)
    ref.run(n, nbatch=3, seed=8)
    assert np.allclose(eng.history_tally(), ref.history_tally(), rtol=1e-12, atol=1e-12)
    assert eng.profile()["chunk"] > 2000


@pytest.mark.parametrize("precision", [32, 64])
def test_chunking_invariance(precision):
    wl = W.water30(20)
    n = 5000
    res = []
    for chunk in (0, 333):
        eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision, chunk=chunk)
        eng.set_geometry(wl["geometry"])
        eng.set_source(wl["source"])
        eng.set_history_tally(0, n)
        eng.run(n, nbatch=1, seed=3)
        res.append(eng.history_tally())
    # same streams, same arithmetic: identical per-history results up to the
    # order of the FP64 atomic additions of one history's deposits
    assert np.allclose(res[0], res[1], rtol=1e-12, atol=1e-12)


@pytest.mark.parametrize("precision", [32, 64])
@pytest.mark.parametrize("workload", ["water128e", "slab64"])
def test_scheduling_invariance(precision, workload):
    # parking sparse warps' particles in the next round and batching the
    # interactions of a warp change the scheduling only
    wl = W.WORKLOADS[workload](32)
    n = 40000
    res = []
    for lanes, inter in ((-1, -1), (16, 8), (-1, 24)):
        eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision, requeue_lanes=lanes,
                            inter_batch=inter)
        eng.set_geometry(wl["geometry"])
        eng.set_source(wl["source"])
        eng.set_history_tally(0, n)
        eng.run(n, nbatch=1, seed=9)
        res.append(eng.history_tally())
    # FP32: a parked particle's pending per-voxel FP32 partial sum is split in
    # two, which regroups float additions (relative 1e-7 per deposit)
    tol = 1e-12 if precision == 64 else 2e-5
    for r in res[1:]:
        assert np.allclose(res[0], r, rtol=tol, atol=tol)


@pytest.mark.parametrize("precision", [64, 32])
def test_graph_replay_matches_direct_launches(precision):
    # direct launches, a graph of four rounds per host check, and one graph
    # launch per chunk whose conditional node loops on the device; a small
    # capacity gives several chunks and many rounds
    wl = W.slab64(32)
    n = 20000
    res = []
    for g in (0, 1, 2):
        eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision, use_graph=g, capacity=1 << 14)
        eng.set_geometry(wl["geometry"])
        eng.set_source(wl["source"])
        eng.set_history_tally(0, n)
        eng.run(n, nbatch=2, seed=4)
        res.append(eng.history_tally())
        t = eng.totals()
        assert t["histories"] == n
        assert eng.profile()["graph"] == g
        eng.close()
    tol = 1e-12 if precision == 64 else 2e-5
    for r in res[1:]:
        assert np.allclose(res[0], r, rtol=tol, atol=tol)


def test_device_loop_with_several_phantoms():
    # the batched path under the device-side loop equals its direct launches
    wl = W.batched64(nprob=6, scale=0.0002, edge=(16, 40))
    out = []
    for g in (0, 2):
        eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=64, use_graph=g)
        eng.set_phantoms(wl["problems"])
        eng.run_phantoms(nbatch=2)
        out.append(eng.tallies()[0])
        assert eng.profile()["graph"] == g
        eng.close()
    assert out[0].sum() > 0 and np.allclose(out[0], out[1], rtol=1e-12, atol=1e-15)


def test_checkpoint_restore_roundtrip():
    wl = W.water30(10)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"])
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    eng.run(2000, nbatch=2, seed=1)
    blob = eng.checkpoint()
    s1, q1, t1 = eng.tallies()
    eng.run(2000, nbatch=2, seed=1, first=2000)
    eng.restore(blob)
    s2, q2, t2 = eng.tallies()
    assert np.array_equal(s1, s2) and np.array_equal(q1, q2)
    assert t1[0] == t2[0]
    # resume: continuing from the checkpoint equals one uninterrupted run
    eng.run(2000, nbatch=2, seed=1, first=2000)
    ref = eg.DoseEngine(wl["media"], ecut=wl["ecut"])
    ref.set_geometry(wl["geometry"])
    ref.set_source(wl["source"])
    ref.run(2000, nbatch=2, seed=1)
    ref.run(2000, nbatch=2, seed=1, first=2000)
    a, _, _ = eng.tallies()
    b, _, _ = ref.tallies()
    assert np.allclose(a, b, rtol=1e-12, atol=0)


def test_capacity_error_is_reported():
    wl = W.water30(10)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], capacity=64, chunk=1000)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    with pytest.raises(eg.EGSError) as ei:
        eng.run(1000, nbatch=1, seed=1)
    assert ei.value.code == 5


@pytest.mark.parametrize("precision", [64, 32])
def test_launch_shape_autotuner(precision):
    # a small queue capacity gives many chunks: the chunk size settles, then
    # successive chunks try every launch shape and the fastest is kept; the
    # per-history results must equal those of a fixed shape
    wl = W.slab64(24)
    n = 400000
    got = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision, capacity=1 << 16)
    ref = eg.DoseEngine(wl["media"], ecut=wl["ecut"], precision=precision, capacity=1 << 16, block_size=128)
    for e in (got, ref):
        e.set_geometry(wl["geometry"])
        e.set_source(wl["source"])
        e.set_history_tally(0, n)
        e.run(n, nbatch=1, seed=12)
    assert 0 <= got.profile()["launch_shape"] < 6
    assert ref.profile()["launch_shape"] == -1
    tol = 1e-12 if precision == 64 else 2e-5
    assert np.allclose(got.history_tally(), ref.history_tally(), rtol=tol, atol=tol)
