"""Phase-space source (egs++ EGS_PhspSource, DOSXYZnrc isource 2) on the GPU.

The particles are those of the reference's BEAMnrc example phase-space file
EX16MVp (15 MV photon beam, MODE2; photons, electrons and positrons): the
FP64 GPU build must follow the oracle history by history, and energy must be
conserved with the weights shared among recycled uses of a particle.
"""
import os

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import formats
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def linac_particles():
    p, h = formats.read_egsphsp(os.path.join(GOLDEN, "EX16MVp.egsphsp1.gz"))
    return p


def test_phsp_history_by_history_fp64():
    p = linac_particles()
    g = W.centred_geometry(20, 1.5)
    src = eg.PhaseSpaceSource(p, position=(0.0, 0.0, -0.5), recycle=1)
    n = 3000
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01, precision=64)
    eng.set_geometry(g)
    eng.set_source(src)
    ora = Oracle([W.WATER], ecut=0.7, pcut=0.01)
    ora.set_geometry(g)
    ora.set_source(src)
    eng.set_history_tally(0, n)
    ora.set_history_tally(0, n)
    eng.run(n, nbatch=2, seed=21)
    ora.run(n, nbatch=2, seed=21)
    hg, ho = eng.history_tally(), ora.history_tally()
    assert ho.sum() > 0
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    assert np.mean(rel < 1e-6) >= 0.97
    # recycled uses: histories 2k and 2k+1 start from the same particle
    # (different random numbers), so both are zero only where it misses
    miss = (hg[0::2] == 0) & (hg[1::2] == 0)
    assert miss.mean() < 0.5


def test_phsp_energy_conservation():
    p = linac_particles()
    inside = (np.abs(p[:, 2]) < 9) & (np.abs(p[:, 3]) < 9) & (p[:, 6] > 0)
    p = p[inside]
    src = eg.PhaseSpaceSource(p, position=(0.0, 0.0, 0.0), recycle=2)
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01, precision=64)
    eng.set_geometry(W.centred_geometry(20, 1.0))
    eng.set_source(src)
    n = 3 * len(p)
    eng.run(n, nbatch=3, seed=5)
    t = eng.totals()
    e = sum(abs(float(q[6])) / 3 * (float(q[1]) + (2 * eg.RM if q[0] > 0 else 0.0)) for q in p) * 3
    assert abs(t["deposited"] + t["escaped"] - e) < 1e-9 * e


def test_rotated_phsp_history_by_history_fp64():
    """egs_transformed_source with a rotation: the EX16MVp particles rotated by
    R_x(1.1) R_y(-0.4) R_z(0.3) and moved off the beam axis enter the phantom
    obliquely from its side; the FP64 GPU build follows the oracle history by
    history, in three media."""
    p = linac_particles()
    med = (np.arange(20 ** 3) % 3).astype(np.int32)
    g = W.centred_geometry(20, 1.0, med)
    R = eg.egs_rotation([1.1, -0.4, 0.3])
    src = eg.PhaseSpaceSource(p, position=(-1.0, -12.0, 2.0), recycle=1, rotation=R)
    n = 3000
    media = [W.WATER, W.LUNG, W.BONE]
    eng = eg.DoseEngine(media, ecut=0.7, pcut=0.01, precision=64)
    eng.set_geometry(g)
    eng.set_source(src)
    ora = Oracle(media, ecut=0.7, pcut=0.01)
    ora.set_geometry(g)
    ora.set_source(src)
    eng.set_history_tally(0, n)
    ora.set_history_tally(0, n)
    eng.run(n, nbatch=2, seed=23)
    ora.run(n, nbatch=2, seed=23)
    hg, ho = eng.history_tally(), ora.history_tally()
    assert (ho > 0).mean() > 0.2
    rel = np.abs(hg - ho) / np.maximum(1e-12, np.abs(ho))
    assert np.mean(rel < 1e-6) >= 0.97


def test_source_rotation_refused():
    p = linac_particles()[:10]
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01)
    eng.set_geometry(W.centred_geometry(8, 1.0))
    bad = np.diag([1.0, 1.0, -1.0])                   # a reflection
    with pytest.raises(eg.EGSError) as e:
        eng.set_source(eg.PhaseSpaceSource(p, rotation=bad))
    assert "rotation" in str(e.value)
    beam = eg.ParallelBeam(charge=0, energy=1.0, position=(0, 0, -5))
    beam.s.rot[:] = tuple(np.eye(3).ravel())
    with pytest.raises(eg.EGSError) as e:
        eng.set_source(beam)
    assert "phase-space" in str(e.value)
    eng.close()
