"""egsphant and .3ddose formats: the reference's example phantom parses, and
write/read round trips are exact to the stored precision."""
import os

import numpy as np

from egsnrc_gb300 import formats
from egsnrc_gb300 import workloads as W

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_egsphant_roundtrip(tmp_path):
    g = W.slab64(8)["geometry"]
    rho = np.linspace(0.2, 1.9, g.nvox)
    p = str(tmp_path / "p.egsphant")
    formats.write_egsphant(p, [W.WATER, W.LUNG, W.BONE], g, rho)
    names, g2, rho2 = formats.read_egsphant(p, pegs_density={W.WATER: 1.0, W.LUNG: 0.26, W.BONE: 1.85})
    assert names == [W.WATER, W.LUNG, W.BONE]
    assert np.array_equal(g2.med, g.med)
    assert np.allclose(rho2, rho, rtol=1e-7)
    dens = np.array([1.0, 0.26, 1.85])[g.med]
    assert np.allclose(g2.rhor, rho / dens, rtol=1e-7)
    assert np.allclose(g2.zb, g.zb)


def test_reference_example_phantom_parses(tmp_path):
    # egs++/geometry/examples/ndgeom_egsphant.egsphant, shipped gzipped as a fixture
    import gzip
    p = str(tmp_path / "ndgeom_egsphant.egsphant")
    with gzip.open(os.path.join(GOLDEN, "ndgeom_egsphant.egsphant.gz"), "rb") as f, open(p, "wb") as g:
        g.write(f.read())
    names, g, rho = formats.read_egsphant(p)
    assert names == ["MEDIUM_1", "MEDIUM_2"]
    assert (g.nx, g.ny, g.nz) == (53, 53, 53)
    assert g.xb[0] == -15 and g.xb[-1] == 15 and abs(g.xb[1] + 5.1) < 1e-12
    assert set(np.unique(g.med)) <= {0, 1}
    assert rho.shape == (53 ** 3,) and rho.min() > 0


def test_3ddose_roundtrip(tmp_path):
    g = W.water30(6)["geometry"]
    d = np.random.default_rng(1).uniform(0, 1e-12, g.nvox)
    d[3] = 0
    s = 0.01 * d
    p = str(tmp_path / "d.3ddose")
    formats.write_3ddose(p, g, d, s)
    (nx, ny, nz), (xb, yb, zb), d2, r2 = formats.read_3ddose(p)
    assert (nx, ny, nz) == (6, 6, 6)
    # %g keeps 6 significant digits (<= 5e-6 relative); doses ~1e-12 need atol=0
    assert np.allclose(d2, d.astype(np.float32), rtol=5e-6, atol=0)
    assert r2[3] == 1.0 and np.allclose(r2[d > 0], 0.01, rtol=1e-5)


def test_reference_phase_space_files_are_self_consistent():
    # BEAMnrc example phase-space files shipped with the reference (MODE0 and
    # MODE2): the records reproduce the counts and energies of their header
    for name, mode, n, nphot, ninc in (("EXslabs", "MODE0", 1030, 31, 1000.0),
                                       ("EX16MVp", "MODE2", 3882, 2542, 15000.0)):
        p, h = formats.read_egsphsp(os.path.join(GOLDEN, name + ".egsphsp1.gz"))
        assert (h["mode"], h["n"], h["photons"], h["incident"]) == (mode, n, nphot, ninc)
        assert p.shape == (n, 7)
        assert int((p[:, 0] == 0).sum()) == nphot
        assert p[:, 1].max() == np.float32(h["ekmax"])
        assert abs(p[p[:, 0] != 0, 1].min() - h["ekmin_e"]) < 2e-6
        assert np.all(p[:, 1] > 0) and np.all(np.abs(p[:, 6]) > 0)
        assert np.all(p[:, 4] ** 2 + p[:, 5] ** 2 <= 1 + 1e-5)
        assert 0 < h["new_history"].sum() <= ninc


def test_phase_space_roundtrip(tmp_path):
    rng = np.random.default_rng(3)
    k = 500
    u = rng.uniform(-0.5, 0.5, k)
    v = rng.uniform(-0.5, 0.5, k)
    p = np.stack([rng.choice([-1, 0, 1], k), rng.uniform(0.1, 10, k), rng.uniform(-5, 5, k),
                  rng.uniform(-5, 5, k), u, v, rng.choice([-1, 1], k) * rng.uniform(0.5, 2, k)], 1)
    newh = rng.uniform(size=k) < 0.3
    for mode in ("MODE0", "MODE2"):
        f = str(tmp_path / ("t_" + mode + ".egsphsp1"))
        formats.write_egsphsp(f, p, incident=123.0, new_history=newh, mode=mode)
        q, h = formats.read_egsphsp(f)
        assert h["mode"] == mode and h["n"] == k and h["incident"] == 123.0
        assert np.array_equal(h["new_history"], newh)
        assert np.array_equal(q[:, 0], p[:, 0])
        assert np.allclose(q[:, 1], p[:, 1], rtol=1e-6, atol=2e-6)
        assert np.allclose(q[:, 2:], p[:, 2:], rtol=1e-6, atol=1e-6)
