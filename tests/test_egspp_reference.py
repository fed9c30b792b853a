"""The restatement's XYZ geometry and parallel-beam source against the
reference's own egs++ classes.

The reference's EGS_XYZGeometry, EGS_ParallelBeam, EGS_RectangleShape,
tabulated spectrum and RANMAR are compiled from its sources into
oracle/_ref/libegspp_ref.so (oracle/Makefile, target `ref`);
tests/golden/egspp_reference.json holds their outputs on the seeded query sets
of tests/golden/egspp_cases.py (make_egspp_fixtures.py).  Where the library is
present the tests compare with it element by element; everywhere they compare
with the fixture.

* Geometry (egs_nd_geometry.h:769-1379): isWhere, howfar from inside,
  howfarFromOut and hownear must agree bit for bit in FP64 on 100,000 queries
  per kind and per plane set (uniform 1 cm and 0.25 cm planes, ragged planes),
  with points on planes, steps down to 2^-40 cm and directions along the axes.
* Source (egs_parallel_beam.h:150, egs_spectra.cpp:466-800, entry as in
  egs_application.cpp:938-945): kinetic energy and entry x and y histograms
  of 10^6 particles against the reference's (two-sample chi-square,
  p > 1e-3); every particle enters at z = 0.  The generators differ
  (RANMAR there, Philox here), so only distributions can agree.
"""
import json
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import egspp_cases as EC  # noqa: E402
from oracle import egspp_ref as R  # noqa: E402
from oracle.oracle_binding import Oracle  # noqa: E402

from egsnrc_gb300 import XYZGeometry  # noqa: E402
from egsnrc_gb300 import workloads as W  # noqa: E402

FIX = json.load(open(os.path.join(HERE, "golden", "egspp_reference.json")))


def geometry_results(query, name, planes):
    """isWhere, howfar from inside, howfar from outside and hownear of the
    query set through query(op, ireg, x, u, t) -> (inew, t)."""
    q = EC.queries(name, planes)
    where, _ = query(0, None, q["where_x"], None, None)
    in_new, in_t = query(1, q["in_ireg"], q["in_x"], q["in_u"], q["in_t"])
    out_new, out_t = query(1, np.full(len(q["out_t"]), -1, np.int32), q["out_x"], q["out_u"], q["out_t"])
    _, near = query(2, q["near_ireg"], q["near_x"], None, None)
    return q, dict(where=where, in_new=in_new, in_t=in_t, out_new=out_new, out_t=out_t, near=near)


def digests(r):
    return dict(where=EC.digest(r["where"]), howfar_in=EC.digest(r["in_new"], r["in_t"]),
                howfar_out=EC.digest(r["out_new"], r["out_t"]), hownear=EC.digest(r["near"]))


def oracle_for(planes):
    ora = Oracle([W.WATER], ecut=0.7, pcut=0.01)
    ora.set_geometry(XYZGeometry(*planes, 0))
    return ora


@pytest.mark.parametrize("name", sorted(EC.geometries()))
def test_query_inputs_reproduce(name):
    planes = EC.geometries()[name]
    assert EC.input_digest(EC.queries(name, planes)) == FIX["geometry"][name]["inputs"]


@pytest.mark.parametrize("name", sorted(EC.geometries()))
def test_oracle_geometry_bitwise_against_reference(name):
    planes = EC.geometries()[name]
    ora = oracle_for(planes)
    q, got = geometry_results(ora.geometry_query, name, planes)
    if R.available():
        g = R.XYZ(*planes)
        want = dict(where=g.is_where(q["where_x"]))
        want["in_new"], want["in_t"] = g.howfar(q["in_ireg"], q["in_x"], q["in_u"], q["in_t"])
        want["out_new"], want["out_t"] = g.howfar(np.full(len(q["out_t"]), -1, np.int32), q["out_x"], q["out_u"],
                                                  q["out_t"])
        want["near"] = g.hownear(q["near_ireg"], q["near_x"])
        for k in want:
            bad = np.flatnonzero(got[k] != want[k])
            assert bad.size == 0, (k, bad[:5], got[k][bad[:5]], want[k][bad[:5]])
    fx = FIX["geometry"][name]
    assert digests(got) == {k: fx[k] for k in ("where", "howfar_in", "howfar_out", "hownear")}
    # the sets exercise what they should: points outside, crossings, exits, entries
    c = fx["counts"]
    assert int((got["where"] < 0).sum()) == c["where_outside"] > 0
    assert int((got["in_new"] != q["in_ireg"]).sum()) == c["in_crossing"] > 0
    assert int((got["out_new"] >= 0).sum()) == c["out_entering"] > 0


def test_point_on_interior_plane_belongs_to_the_slab_below():
    # findRegion (egs_base_geometry.h:178-190): x on plane k is in slab k-1;
    # the water30 pencil beam enters on the planes x = y = 0
    planes = EC.geometries()["water30"]
    ora = oracle_for(planes)
    x = np.array([[0.0, 0.0, 0.5], [-15.0, -15.0, 0.0], [15.0, 15.0, 30.0]])
    where, _ = ora.geometry_query(0, None, x)
    assert list(where) == [14 + 14 * 30, 0, 29 + 29 * 30 + 29 * 900]


def chi2_two_sample(a, b):
    """Two-sample chi-square over histogram bins with counts in both, for
    samples of equal size: statistic, degrees of freedom and p value."""
    from scipy.stats import chi2
    a = np.asarray(a, float)
    b = np.asarray(b, float)
    m = (a + b) > 0
    stat = float((((a[m] - b[m]) ** 2) / (a[m] + b[m])).sum())
    dof = int(m.sum())
    return stat, dof, float(chi2.sf(stat, dof))


@pytest.mark.parametrize("case", ["slab64_photons", "water128e_electrons"])
def test_oracle_source_distribution_against_reference(case):
    fx = FIX["source"][case]
    wl = W.WORKLOADS[{"slab64_photons": "slab64", "water128e_electrons": "water128e"}[case]]()
    ora = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
    ora.set_geometry(wl["geometry"])
    ora.set_source(wl["source"])
    n = fx["n"]
    parts = ora.sample_source(n, seed=5)
    assert int((parts[:, 8] >= 0).sum()) == fx["entered"] == n
    assert set(parts[:, 4].tolist()) == {0.0} and fx["z_entry"] == [0.0]
    he, _ = np.histogram(parts[:, 1], bins=EC.E_BINS, range=tuple(fx["erange"]))
    hx, _ = np.histogram(parts[:, 2], bins=EC.XY_BINS, range=(-5.0, 5.0))
    hy, _ = np.histogram(parts[:, 3], bins=EC.XY_BINS, range=(-5.0, 5.0))
    for ours, ref in ((he, fx["energy"]), (hx, fx["x"]), (hy, fx["y"])):
        stat, dof, p = chi2_two_sample(ours, ref)
        assert p > 1e-3, (case, stat, dof, p)
    # mean energy within 4 standard errors of the reference's
    sd = parts[:, 1].std()
    assert abs(parts[:, 1].mean() - fx["mean_energy"]) < 4 * sd * np.sqrt(2.0 / n) + 1e-12


@pytest.mark.skipif(not R.available(), reason="reference egs++ library not built (sources absent)")
def test_fixture_is_the_reference():
    # the committed digests are what the reference library gives now
    for name, planes in EC.geometries().items():
        g = R.XYZ(*planes)
        q = EC.queries(name, planes)
        where = g.is_where(q["where_x"])
        assert EC.digest(where) == FIX["geometry"][name]["where"]
        near = g.hownear(q["near_ireg"], q["near_x"])
        assert EC.digest(near) == FIX["geometry"][name]["hownear"]


def test_egspp_application_binding_compiles():
    # the egs++ application binding against the reference's headers
    from egsnrc_gb300 import build
    ref = build.reference_dir()
    if not ref:
        pytest.skip("reference sources absent")
    import subprocess
    here = os.path.join(os.path.dirname(HERE), "oracle")
    target = os.path.join("_ref", "egs_gpu_dose_application.o")
    r = subprocess.run(["make", "-s", target, "REF=" + ref], cwd=here, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    assert os.path.exists(os.path.join(here, target))
