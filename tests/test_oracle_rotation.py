"""Rotated phase-space sources (egs++ EGS_TransformedSource with a rotation)
in the oracle, and the egs++ rotation conventions (CPU only).

* A rotation by the identity matrix changes nothing, bit for bit.
* A rotation by pi about the z-axis in a phantom symmetric under
  (x, y) -> (-x, -y) maps every history onto its mirror image: the energy each
  history deposits is the same as without the rotation.  Sign changes are
  exact in floating point, so the histories agree except where the geometry
  breaks a tie the other way (a particle on a voxel face, equal distances to
  two faces), which forks a few of them.
* egs_rotation builds R_z(phi) R_x(theta) and R_x(a) R_y(b) R_z(c) from the
  rotX/rotY/rotZ matrices of egs++/egs_transformations.h:303-326 and returns
  proper rotations for every input form.
"""
import math
import os

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import formats
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def particles():
    p, _ = formats.read_egsphsp(os.path.join(GOLDEN, "EX16MVp.egsphsp1.gz"))
    return p


def oracle(src, g):
    o = Oracle([W.WATER], ecut=0.7, pcut=0.01)
    o.set_geometry(g)
    o.set_source(src)
    return o


def test_identity_rotation_changes_nothing():
    p = particles()
    g = W.centred_geometry(12, 1.0)
    a = oracle(eg.PhaseSpaceSource(p, position=(0, 0, -7.0)), g)
    b = oracle(eg.PhaseSpaceSource(p, position=(0, 0, -7.0), rotation=np.eye(3)), g)
    a.run(2000, nbatch=2, seed=3, threads=4)
    b.run(2000, nbatch=2, seed=3, threads=4)
    sa, sb = a.tallies()[0], b.tallies()[0]
    assert sa.sum() > 0 and np.array_equal(sa, sb)


def test_half_turn_mirrors_every_history():
    p = particles()
    g = W.centred_geometry(12, 1.0)
    n = 2000
    a = oracle(eg.PhaseSpaceSource(p, position=(0, 0, -7.0)), g)
    c = oracle(eg.PhaseSpaceSource(p, position=(0, 0, -7.0), rotation=np.diag([-1.0, -1.0, 1.0])), g)
    a.set_history_tally(0, n)
    c.set_history_tally(0, n)
    a.run(n, nbatch=2, seed=4, threads=4)
    c.run(n, nbatch=2, seed=4, threads=4)
    ha, hc = a.history_tally(), c.history_tally()
    assert (ha > 0).mean() > 0.2
    rel = np.abs(ha - hc) / np.maximum(1e-12, np.abs(ha))
    assert np.mean(rel < 1e-9) >= 0.97


def rx(t):
    return np.array([[1, 0, 0], [0, math.cos(t), math.sin(t)], [0, -math.sin(t), math.cos(t)]])


def ry(t):
    return np.array([[math.cos(t), 0, -math.sin(t)], [0, 1, 0], [math.sin(t), 0, math.cos(t)]])


def rz(t):
    return np.array([[math.cos(t), math.sin(t), 0], [-math.sin(t), math.cos(t), 0], [0, 0, 1]])


@pytest.mark.parametrize("form", [[0.4, 0.9], [1.1, -0.4, 0.3], [1.0, 2.0, 3.0, 0.7], "vector", "matrix"])
def test_egs_rotation_forms(form):
    if form == "vector":
        R = eg.egs_rotation(rotation_vector=[1.0, -2.0, 0.5])
    elif form == "matrix":
        M = rz(0.2) @ rx(-0.5)
        R = eg.egs_rotation(list(M.ravel()))
        assert np.array_equal(R, M)
    else:
        R = eg.egs_rotation(form)
    assert np.allclose(R @ R.T, np.eye(3), atol=1e-12) and abs(np.linalg.det(R) - 1) < 1e-12
    if isinstance(form, list) and len(form) == 2:
        assert np.allclose(R, rz(form[0]) @ rx(form[1]), atol=1e-15)
    if isinstance(form, list) and len(form) == 3:
        assert np.allclose(R, rx(form[0]) @ ry(form[1]) @ rz(form[2]), atol=1e-15)
    assert np.array_equal(eg.egs_rotation(), np.eye(3))
