"""The egs++ input driver (egs_gpu_app) against the Python binding of the same C ABI.

The driver reads an egs++ input file (run control, EGS_XYZGeometry with
`set medium`, parallel-beam or phase-space source, transport parameters, rng
seeds) and writes a .3ddose file; the same problem set up through the Python
binding must give the same dose (both are FP32 runs of the same histories;
the file holds single-precision values).
"""
import gzip
import os
import shutil
import subprocess

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import formats
from egsnrc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
APP = os.path.join(os.path.dirname(HERE), "egsnrc_gb300", "egs_gpu_app")

SLAB = """
:start run control:
    ncase = 40000
    nbatch = 4
:stop run control:
:start geometry definition:
    :start geometry:
        name     = plate
        library  = egs_ndgeometry
        type     = EGS_XYZGeometry
        x-planes = -5, 5
        y-planes = -5, 5
        z-slabs = 0, 0.5, 20
        :start media input:
            media = H2O521ICRU ICRPBONE521ICRU
            set medium = 4 6 1
        :stop media input:
    :stop geometry:
    simulation geometry = plate
:stop geometry definition:
:start source definition:
    :start source:
        name      = beam
        library   = egs_parallel_beam
        charge    = -1
        direction = 0 0 1
        :start spectrum:
            type = monoenergetic
            energy = 12
        :stop spectrum:
        :start shape:
            type     = point
            position = 0 0 -8
        :stop shape:
    :stop source:
    simulation source = beam
:stop source definition:
:start MC transport parameter:
    Global ECUT = 0.7
    Global PCUT = 0.01
:stop MC transport parameter:
:start rng definition:
    initial seeds = 7 9
:stop rng definition:
"""

PHSP = """
:start run control:
    ncase = 30000
    nbatch = 3
:stop run control:
:start geometry definition:
    :start geometry:
        name     = box
        library  = egs_ndgeometry
        type     = EGS_XYZGeometry
        x-slabs = -15, 2, 15
        y-slabs = -15, 2, 15
        z-slabs = 0, 2, 15
        :start media input:
            media = H2O521ICRU
        :stop media input:
    :stop geometry:
    simulation geometry = box
:stop geometry definition:
:start source definition:
    :start source:
        name      = linac
        library   = egs_phsp_source
        phase space file = PHSPFILE
        particle type = all
        recycle photons = 1
        recycle electrons = 1
    :stop source:
    :start source:
        name      = moved
        library   = egs_transformed_source
        source name = linac
        :start transformation:
            translation = 0 0 -0.5
        :stop transformation:
    :stop source:
    simulation source = moved
:stop source definition:
:start MC transport parameter:
    Global ECUT = 0.7
    Global PCUT = 0.01
:stop MC transport parameter:
:start rng definition:
    initial seeds = 3
:stop rng definition:
"""


def run_app(tmp_path, text, name):
    f = tmp_path / (name + ".egsinp")
    f.write_text(text)
    r = subprocess.run([APP, "-i", str(f), "-p", "521icru", "-o", str(tmp_path / name)], capture_output=True,
                       text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    (nx, ny, nz), planes, dose, rel = formats.read_3ddose(str(tmp_path / (name + ".3ddose")))
    return dose, rel


def phsp_norm(nparticles, incident, ncase=30000, recycle=1):
    """EGS_DoseScoring's factor ncase / F for a phase-space source, F = incident
    * Nread / Nparticle with Nread the records read for ncase histories."""
    nread = (ncase + recycle) // (recycle + 1)
    return ncase / (incident * nread / nparticles)


def compare(dose_file, dose_py):
    # the file holds %g of the single-precision dose (6 digits); doses are
    # ~1e-11 Gy per history, so the comparison is relative only
    sel = dose_py > 1e-3 * dose_py.max()
    assert sel.sum() > 5
    assert np.allclose(dose_file[sel], dose_py[sel].astype(np.float32), rtol=2e-5, atol=0)


def test_app_slab_matches_binding(tmp_path):
    dose_file, _ = run_app(tmp_path, SLAB, "slab")
    zb = 0.5 * np.arange(21)          # z-slabs = 0, 0.5, 20: 20 slabs from 0 to 10 cm
    med = np.zeros(len(zb) - 1, dtype=np.int32)
    med[4:7] = 1                      # set medium = 4 6 1: regions 4..6 (0-based) are bone
    g = eg.XYZGeometry([-5, 5], [-5, 5], zb, med)
    eng = eg.DoseEngine([W.WATER, W.BONE], ecut=0.7, pcut=0.01)
    eng.set_geometry(g)
    eng.set_source(eg.ParallelBeam(charge=-1, energy=12.0, position=(0, 0, -8)))
    eng.run(40000, nbatch=4, seed=7)
    compare(dose_file, eng.dose()[0])


def test_app_phase_space_source_matches_binding(tmp_path):
    path = tmp_path / "EX16MVp.egsphsp1"
    with gzip.open(os.path.join(HERE, "golden", "EX16MVp.egsphsp1.gz"), "rb") as a, open(path, "wb") as b:
        shutil.copyfileobj(a, b)
    dose_file, _ = run_app(tmp_path, PHSP.replace("PHSPFILE", str(path)), "phsp")
    p, _ = formats.read_egsphsp(str(path))
    b = -15 + 2.0 * np.arange(16)
    g = eg.XYZGeometry(b, b, 2.0 * np.arange(16), 0)
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01)
    eng.set_geometry(g)
    eng.set_source(eg.PhaseSpaceSource(p, position=(0, 0, -0.5), recycle=1))
    eng.run(30000, nbatch=3, seed=3)
    compare(dose_file, eng.dose()[0] * phsp_norm(len(p), 15000))


def ex16_particles(tmp_path):
    path = tmp_path / "EX16MVp.egsphsp1"
    with gzip.open(os.path.join(HERE, "golden", "EX16MVp.egsphsp1.gz"), "rb") as a, open(path, "wb") as b:
        shutil.copyfileobj(a, b)
    p, hdr = formats.read_egsphsp(str(path))
    return path, p, hdr


def binding_dose(p, recycle=1):
    """The binding's dose per history, times the driver's phase-space normalisation."""
    b = -15 + 2.0 * np.arange(16)
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01)
    eng.set_geometry(eg.XYZGeometry(b, b, 2.0 * np.arange(16), 0))
    eng.set_source(eg.PhaseSpaceSource(p, position=(0, 0, -0.5), recycle=recycle))
    eng.run(30000, nbatch=3, seed=3)
    return eng.dose()[0] * phsp_norm(len(p), 15000, recycle=recycle)


def test_app_iaea_phase_space_source_matches_binding(tmp_path):
    """iaea_phsp_source: the EX16MVp particles written as an IAEA file on the
    plane z = 0.25 and moved by -0.75 cm give the dose of the same particles
    placed at z = -0.5 through the binding."""
    _, p, hdr = ex16_particles(tmp_path)
    base = tmp_path / "ex16"
    formats.write_iaea_phsp(str(base), p, hdr["incident"], new_history=hdr["new_history"], z=0.25)
    text = PHSP.replace("egs_phsp_source", "iaea_phsp_source").replace("phase space file = PHSPFILE",
                                                                       "iaea phase space file = " + str(base))
    text = text.replace("recycle photons", "reuse photons").replace("recycle electrons", "reuse electrons")
    text = text.replace("translation = 0 0 -0.5", "translation = 0 0 -0.75")
    dose_file, _ = run_app(tmp_path, text, "iaea")
    compare(dose_file, binding_dose(p))


def test_app_phase_space_selection_matches_binding(tmp_path):
    """'particle type', 'cutout' and 'weight window' of egs_phsp_source: the
    rejected particles carry weight 0, the rest are transported unchanged."""
    path, p, _ = ex16_particles(tmp_path)
    text = PHSP.replace("PHSPFILE", str(path)).replace("particle type = all", "particle type = photons\n"
                                                       "        cutout = -4 4 -3 5\n"
                                                       "        weight window = 0.0001 0.0249")
    dose_file, _ = run_app(tmp_path, text, "phsp_sel")
    q = p.copy()
    wt = q[:, 6].astype(np.float64) / 2.0   # the stored weight over the two uses of each particle
    keep = (q[:, 0] == 0) & (q[:, 2] >= -4) & (q[:, 2] <= 4) & (q[:, 3] >= -3) & (q[:, 3] <= 5)
    keep &= (wt >= 0.0001) & (wt <= 0.0249)
    assert 100 < keep.sum() < len(q) - 100
    q[~keep, 6] = np.where(q[~keep, 6] < 0, -0.0, 0.0)
    compare(dose_file, binding_dose(q))


def test_app_latch_filter_matches_binding(tmp_path):
    """'filter type = 0' with 'latch setting = 0011 000000001': keep particles
    with LATCH bit 2 or 3, reject those with bit 4 + 8 = 12."""
    path, p, _ = ex16_particles(tmp_path)
    text = PHSP.replace("PHSPFILE", str(path)).replace("particle type = all", "particle type = all\n"
                                                       "        filter type = 0\n"
                                                       "        latch setting = 0011 000000001")
    dose_file, _ = run_app(tmp_path, text, "phsp_latch")
    _, info = eg.read_phase_space(str(path))
    latch = info["latch"]
    keep = ((latch & 0b1100) != 0) & ((latch & (1 << 12)) == 0) & ((latch >> 31) == 0)
    assert 100 < keep.sum() < len(p) - 100
    q = p.copy()
    q[~keep, 6] = np.where(q[~keep, 6] < 0, -0.0, 0.0)
    compare(dose_file, binding_dose(q))


def test_app_rotated_phase_space_source_matches_binding(tmp_path):
    """egs_transformed_source with 'rotation = 1.1 -0.4 0.3' and a translation:
    the driver builds R_x R_y R_z as egsnrc_gb300.egs_rotation does, so the run
    equals the binding's with that matrix."""
    path, p, _ = ex16_particles(tmp_path)
    text = PHSP.replace("PHSPFILE", str(path)).replace(
        "translation = 0 0 -0.5", "translation = -1 -20 4\n            rotation = 1.1 -0.4 0.3")
    dose_file, _ = run_app(tmp_path, text, "phsp_rot")
    b = -15 + 2.0 * np.arange(16)
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01)
    eng.set_geometry(eg.XYZGeometry(b, b, 2.0 * np.arange(16), 0))
    eng.set_source(eg.PhaseSpaceSource(p, position=(-1, -20, 4), recycle=1, rotation=eg.egs_rotation([1.1, -0.4, 0.3])))
    eng.run(30000, nbatch=3, seed=3)
    compare(dose_file, eng.dose()[0] * phsp_norm(len(p), 15000))


def test_app_presta1_and_smax_match_binding(tmp_path):
    """The transport keys "Boundary crossing algorithm = PRESTA-I", "Skin
    depth for BCA" and "Global Smax" reach the engine as the binding sets them."""
    text = SLAB.replace("    Global PCUT = 0.01\n", "    Global PCUT = 0.01\n    Boundary crossing algorithm = PRESTA-I\n"
                        "    Skin depth for BCA = 0\n    Global Smax = 0.3\n")
    dose_file, _ = run_app(tmp_path, text, "slab_p1")
    zb = 0.5 * np.arange(21)
    med = np.zeros(len(zb) - 1, dtype=np.int32)
    med[4:7] = 1
    g = eg.XYZGeometry([-5, 5], [-5, 5], zb, med)
    eng = eg.DoseEngine([W.WATER, W.BONE], ecut=0.7, pcut=0.01, bca_algorithm=1, skindepth=0.0, smax=0.3)
    eng.set_geometry(g)
    eng.set_source(eg.ParallelBeam(charge=-1, energy=12.0, position=(0, 0, -8)))
    eng.run(40000, nbatch=4, seed=7)
    compare(dose_file, eng.dose()[0])
    # and they changed the transport: the EXACT run of the same input differs
    exact, _ = run_app(tmp_path, SLAB, "slab_exact")
    sel = dose_file > 1e-3 * dose_file.max()
    assert np.max(np.abs(exact[sel] / dose_file[sel] - 1)) > 1e-3
