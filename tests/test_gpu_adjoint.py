"""Seed-replay adjoint (egsgpu_adjoint) and its torch.autograd binding.

In the kerma limit (ECUT above every electron energy, so each electron's
energy stays where it is set in motion) the adjoint is the exact score of the
photon paths and must agree with central finite differences taken with
common random numbers: the mean over independent seeds of both estimates,
at voxels on the beam axis, off it and far outside the beam, and for a
uniform scaling of all densities, within 3.5 combined standard errors.
Finite differences use a 10% density step: smaller steps leave the estimate
dominated by interactions shifted across voxel faces (heavy-tailed noise).
"""
import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W

pytestmark = pytest.mark.gpu


def kerma_case():
    rng = np.random.default_rng(5)
    n, dx = 10, 0.5
    rhor = 1 + 0.1 * rng.uniform(-1, 1, n ** 3)
    g = W.centred_geometry(n, dx, 0, rhor)
    src = eg.ParallelBeam(charge=0, energy=2.0, position=(0, 0, -1.0), rectangle=(-1.5, 1.5, -1.5, 1.5))
    c = rng.uniform(0, 1, n ** 3)
    vox = [0 + 0 * n + 5 * n * n] + [5 + 5 * n + iz * n * n for iz in (1, 5, 8)] + [7 + 5 * n + 3 * n * n]
    return g, src, c, vox


def dose(eng, g, rhor, n, seed):
    eng.set_geometry(eg.XYZGeometry(g.xb, g.yb, g.zb, g.med, rhor))
    eng.reset()
    eng.run(n, nbatch=1, seed=seed)
    return eng.dose()[0]


def test_adjoint_matches_finite_differences_kerma():
    g, src, c, vox = kerma_case()
    eng = eg.DoseEngine([W.WATER], ecut=3.0, pcut=0.01, precision=64)
    eng.set_source(src)
    n, M, h = 400000, 8, 0.1
    A, F, U, FU = [], [], [], []
    for m in range(M):
        seed = 700 + m
        dose(eng, g, g.rhor, n, seed)
        gr = eng.adjoint(c, n, seed=seed)
        A.append(gr[vox])
        U.append(float(g.rhor @ gr))
        row = []
        for v in vox:
            r = g.rhor.copy(); r[v] *= 1 + h
            lp = c @ dose(eng, g, r, n, seed)
            r = g.rhor.copy(); r[v] *= 1 - h
            lm = c @ dose(eng, g, r, n, seed)
            row.append((lp - lm) / (2 * h * g.rhor[v]))
        F.append(row)
        FU.append((c @ dose(eng, g, g.rhor * 1.02, n, seed) - c @ dose(eng, g, g.rhor * 0.98, n, seed)) / 0.04)
    A, F = np.array(A), np.array(F)
    se = lambda x: x.std(0, ddof=1) / np.sqrt(len(x))
    z = (A.mean(0) - F.mean(0)) / np.hypot(se(A), se(F))
    assert np.all(np.abs(z) < 3.5), z
    U, FU = np.array(U), np.array(FU)
    zu = (U.mean() - FU.mean()) / np.hypot(se(U), se(FU))
    assert abs(zu) < 3.5, zu
    # the on-axis entrance voxel's gradient is resolved by the adjoint
    assert abs(A.mean(0)[1]) > 4 * se(A)[1]
    eng.close()


def test_autograd_backward_is_the_adjoint():
    torch = pytest.importorskip("torch")
    from egsnrc_gb300.autograd import voxel_dose
    g, src, c, vox = kerma_case()
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01, precision=32)
    eng.set_source(src)
    rhor = torch.tensor(g.rhor, dtype=torch.float64, requires_grad=True)
    target = torch.zeros(g.nvox, dtype=torch.float64)
    d = voxel_dose(rhor, eng, g, 20000, seed=3, nbatch=4)
    loss = ((d - target) ** 2).sum()
    loss.backward()
    direct = eng.adjoint(2 * d.detach().numpy(), 20000, seed=3)
    assert np.array_equal(rhor.grad.numpy(), direct) or np.allclose(rhor.grad.numpy(), direct, rtol=1e-6,
                                                                    atol=1e-6 * np.abs(direct).max())
    assert np.isfinite(direct).all() and np.abs(direct).max() > 0
    eng.close()
