"""The oracle's HOWFARLESS mode (DOSXYZnrc ihowfarless) on the CPU.

In a homogeneous water phantom, HOWFARLESS transport must give the voxel
doses of voxel-by-voxel transport within statistics, with far fewer
condensed-history steps, and conserve energy to the 1e-3 that DOSXYZnrc's
hinge allows (a hinge segment of negative length is skipped).
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W
from oracle.oracle_binding import Oracle


@pytest.mark.parametrize("charge,energy,n", [(-1, 6.0, 6000), (0, 6.0, 30000)])
def test_oracle_howfarless_matches_voxel_transport(charge, energy, n):
    g = W.centred_geometry(16, 0.5)
    src = eg.ParallelBeam(charge=charge, energy=energy, position=(0, 0, -1.0), rectangle=(-2, 2, -2, 2))
    res = []
    for hfl in (False, True):
        o = Oracle([W.WATER], ecut=0.7, pcut=0.01)
        o.set_geometry(g)
        o.set_source(src)
        if hfl:
            o.set_howfarless(True)
        o.run(n, nbatch=10, seed=5, threads=8)
        s, s2, t = o.tallies()
        assert abs(t[2] + t[3] - n * energy) < 1e-3 * n * energy
        res.append((s, s2, t[4]))
    (a, a2, steps0), (b, b2, steps1) = res
    assert steps1 < 0.5 * steps0
    # voxels above 20% of the maximum, each with its batch sigma
    def sig(s, s2, nb=10):
        m = s / nb
        return np.sqrt(np.maximum(s2 / nb - m * m, 0) / (nb - 1)) * nb
    sel = a > 0.2 * a.max()
    z = (b[sel] - a[sel]) / np.hypot(sig(a, a2)[sel], sig(b, b2)[sel])
    assert np.mean(np.abs(z) < 2) >= 0.85 and np.mean(np.abs(z) < 3) >= 0.95
    assert abs(b[sel].sum() / a[sel].sum() - 1) < 0.02
