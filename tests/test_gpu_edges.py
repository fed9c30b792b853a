"""Edge cases of the CUDA engine, through the C ABI, against the oracle.

  * an empty run, and history indices at the top of their 32-bit range;
  * a beam that misses the phantom (EGS_XYZGeometry howfar from outside
    returns no region: the history deposits and escapes nothing);
  * ragged planes (every voxel a different size) with oblique beams, history
    by history in FP64 and energy conservation in FP32;
  * a phantom of more than 2^24 voxels with dimensions that are not powers
    of two, which exercises the multiply-high voxel decoding far from zero;
  * rejected geometries (planes not increasing, medium out of range,
    non-positive density) and run ranges;
  * tallies read into the caller's buffers.
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle

pytestmark = pytest.mark.gpu

MEDIA = [W.WATER, W.LUNG, W.BONE]


def pair(geom, src, precision=64, media=MEDIA, ecut=0.521, pcut=0.01):
    e = eg.DoseEngine(media, ecut=ecut, pcut=pcut, precision=precision)
    e.set_geometry(geom)
    e.set_source(src)
    o = Oracle(media, ecut=ecut, pcut=pcut)
    o.set_geometry(geom)
    o.set_source(src)
    return e, o


def by_history(e, o, n, first=0, seed=5, threads=1):
    e.set_history_tally(first, n)
    o.set_history_tally(first, n)
    e.run(n, nbatch=2, seed=seed, first=first)
    o.run(n, nbatch=2, seed=seed, first=first, threads=threads)
    hg, ho = e.history_tally(), o.history_tally()
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    return np.mean(rel < 1e-6), hg, ho


def ragged(seed=3, n=(13, 11, 17)):
    rng = np.random.default_rng(seed)
    planes = [np.concatenate([[0.0], np.cumsum(rng.uniform(0.05, 1.5, k))]) for k in n]
    planes = [p - p[-1] / 2 for p in planes[:2]] + [planes[2]]
    nv = int(np.prod(n))
    med = rng.integers(0, len(MEDIA), nv).astype(np.int32)
    rhor = rng.uniform(0.7, 1.3, nv)
    return eg.XYZGeometry(planes[0], planes[1], planes[2], med, rhor)


def test_zero_histories_is_a_no_op():
    e, _ = pair(W.centred_geometry(8, 1.0), eg.ParallelBeam(charge=0, energy=1.0, position=(0, 0, -1)))
    e.run(0, nbatch=1, seed=1)
    s, s2, _ = e.tallies()
    t = e.totals()
    assert not s.any() and not s2.any()
    assert t["histories"] == 0 and t["deposited"] == 0 and t["escaped"] == 0
    e.close()


def test_history_indices_at_the_top_of_the_range():
    g = W.centred_geometry(10, 1.0)
    src = eg.ParallelBeam(charge=0, energy=2.0, position=(0.1, -0.2, -1.0))
    e, o = pair(g, src)
    top = (1 << 32) - 1
    match, hg, _ = by_history(e, o, 200, first=top - 200)
    assert match >= 0.97 and hg.sum() > 0
    with pytest.raises(eg.EGSError) as ex:
        e.run(201, nbatch=1, seed=5, first=top - 200)
    assert ex.value.code == 1
    with pytest.raises(eg.EGSError):
        e.run(10, nbatch=1, seed=5, first=-1)
    e.close()


@pytest.mark.parametrize("precision", [32, 64])
def test_beam_that_misses_the_phantom(precision):
    g = W.centred_geometry(8, 1.0)
    # beside the phantom and parallel to it, then pointing away from it
    for src in (eg.ParallelBeam(charge=-1, energy=5.0, position=(6.0, 0.0, -1.0)),
                eg.ParallelBeam(charge=0, energy=5.0, position=(0.0, 0.0, -1.0), direction=(0, 0, -1))):
        e, o = pair(g, src, precision=precision)
        e.run(1000, nbatch=2, seed=9)
        o.run(1000, nbatch=2, seed=9)
        t = e.totals()
        _, _, to = o.tallies()
        assert t["deposited"] == 0 and t["escaped"] == 0 and to[2] == 0 and to[3] == 0
        assert t["histories"] == 1000
        e.close()
        o.close()


@pytest.mark.parametrize("charge,energy,direction", [(0, 3.0, (0.3, -0.2, 1.0)), (-1, 8.0, (-0.4, 0.25, 1.0)),
                                                     (1, 2.0, (0.0, 0.6, 1.0))])
def test_ragged_planes_history_by_history_fp64(charge, energy, direction):
    g = ragged()
    src = eg.ParallelBeam(charge=charge, energy=energy, position=(0.0, 0.0, -2.0), direction=direction,
                          rectangle=(-1.5, 1.5, -1.0, 1.0))
    e, o = pair(g, src)
    match, hg, ho = by_history(e, o, 1500)
    assert match >= 0.97, match
    assert ho.sum() > 0
    e.close()
    o.close()


def test_ragged_planes_conserve_energy_fp32():
    g = ragged(seed=11)
    src = eg.ParallelBeam(charge=-1, energy=6.0, position=(0.0, 0.0, -2.0), direction=(0.2, 0.1, 1.0),
                          rectangle=(-2, 2, -2, 2))
    e = eg.DoseEngine(MEDIA, ecut=0.521, pcut=0.01, precision=32)
    e.set_geometry(g)
    e.set_source(src)
    n = 200000
    e.run(n, nbatch=10, seed=4)
    t = e.totals()
    # histories that miss the phantom (the field is wider than it) carry nothing
    assert 0 < t["deposited"] + t["escaped"] <= n * 6.0 * (1 + 1e-6)
    s, _, _ = e.tallies()
    assert s.sum() == pytest.approx(t["deposited"], rel=1e-6)
    e.close()


def test_phantom_beyond_2_24_voxels_history_by_history():
    nx, ny, nz = 397, 403, 109          # 17.4 M voxels, no power-of-two dimension
    dx = 0.1
    g = eg.XYZGeometry(-nx * dx / 2 + dx * np.arange(nx + 1), -ny * dx / 2 + dx * np.arange(ny + 1),
                       dx * np.arange(nz + 1), (np.arange(nx * ny * nz) % 3).astype(np.int32))
    assert g.nvox > 1 << 24
    # a beam along the far corner of the phantom, through its whole depth:
    # the largest voxel indices
    src = eg.ParallelBeam(charge=0, energy=4.0, position=(nx * dx / 2 - 0.3, ny * dx / 2 - 0.3, -1.0),
                          direction=(-0.02, -0.02, 1.0))
    e, o = pair(g, src)
    match, hg, ho = by_history(e, o, 2000)
    assert match >= 0.97 and ho.sum() > 0
    e.close()
    o.close()


def test_rejected_geometries_and_ranges():
    e = eg.DoseEngine(MEDIA, ecut=0.521, pcut=0.01)
    b = np.arange(5.0)
    bad = [
        eg.XYZGeometry([0, 1, 1, 2], b, b, 0),               # planes not increasing
        eg.XYZGeometry(b, b, b, 3),                          # medium out of range
        eg.XYZGeometry(b, b, b, 0, rhor=0.0),                # zero density
        eg.XYZGeometry(b, b, b, 0, rhor=np.nan),             # not finite
    ]
    for g in bad:
        with pytest.raises(eg.EGSError) as ex:
            e.set_geometry(g)
        assert ex.value.code == 1
    e.set_geometry(eg.XYZGeometry(b, b, b, 0))
    with pytest.raises(eg.EGSError) as ex:
        e.run(10, nbatch=1, seed=1)       # no source yet
    assert ex.value.code == 7
    e.set_source(eg.ParallelBeam(charge=0, energy=1.0, position=(2, 2, -1)))
    for kw in (dict(n=-1, nbatch=1), dict(n=10, nbatch=0)):
        with pytest.raises(eg.EGSError):
            e.run(kw["n"], nbatch=kw["nbatch"], seed=1)
    e.close()


def test_tallies_into_caller_buffers():
    g = W.centred_geometry(12, 0.5)
    e, _ = pair(g, eg.ParallelBeam(charge=-1, energy=3.0, position=(0, 0, -1)))
    e.run(2000, nbatch=4, seed=3)
    s, s2, t = e.tallies()
    out = (np.full(g.nvox, np.nan), np.full(g.nvox, np.nan))
    s_b, s2_b, t_b = e.tallies(out=out)
    assert s_b is out[0] and s2_b is out[1]
    assert np.array_equal(s, s_b) and np.array_equal(s2, s2_b) and np.array_equal(t, t_b)
    for bad in ((np.empty(g.nvox - 1), np.empty(g.nvox)), (np.empty(g.nvox, np.float32), np.empty(g.nvox)),
                (np.empty(2 * g.nvox)[::2], np.empty(g.nvox))):
        with pytest.raises(ValueError):
            e.tallies(out=bad)
    e.close()
