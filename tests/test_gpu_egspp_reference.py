"""The engine's XYZ geometry against the reference's own EGS_XYZGeometry, on
the GPU and through the C ABI (egsgpu_geometry_query).

The FP64 build runs the kernels' geometry functions (isWhere, howfar,
howfarFromOut, hownear) on the seeded query sets of
tests/golden/egspp_cases.py; the SHA-256 digests of its results must equal
those of the reference's egs++ classes in tests/golden/egspp_reference.json
(made by make_egspp_fixtures.py from the reference's sources): bit for bit,
100,000 queries per kind and per plane set.  The FP32 build must place points
in the same region except within FP32 rounding of a plane.
"""
import json
import os
import sys

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))
import egspp_cases as EC  # noqa: E402

pytestmark = pytest.mark.gpu
FIX = json.load(open(os.path.join(HERE, "golden", "egspp_reference.json")))


def engine_for(planes, precision):
    eng = eg.DoseEngine([W.WATER], ecut=0.7, pcut=0.01, precision=precision)
    eng.set_geometry(eg.XYZGeometry(*planes, 0))
    return eng


def results(eng, name, planes):
    q = EC.queries(name, planes)
    assert EC.input_digest(q) == FIX["geometry"][name]["inputs"]
    where, _ = eng.geometry_query(0, None, q["where_x"])
    in_new, in_t = eng.geometry_query(1, q["in_ireg"], q["in_x"], q["in_u"], q["in_t"])
    out_new, out_t = eng.geometry_query(1, np.full(len(q["out_t"]), -1, np.int32), q["out_x"], q["out_u"], q["out_t"])
    _, near = eng.geometry_query(2, q["near_ireg"], q["near_x"])
    return q, dict(where=where, in_new=in_new, in_t=in_t, out_new=out_new, out_t=out_t, near=near)


@pytest.mark.parametrize("name", sorted(EC.geometries()))
def test_fp64_geometry_bitwise_against_reference(name):
    planes = EC.geometries()[name]
    eng = engine_for(planes, 64)
    q, r = results(eng, name, planes)
    fx = FIX["geometry"][name]
    assert EC.digest(r["where"]) == fx["where"]
    assert EC.digest(r["in_new"], r["in_t"]) == fx["howfar_in"]
    assert EC.digest(r["out_new"], r["out_t"]) == fx["howfar_out"]
    assert EC.digest(r["near"]) == fx["hownear"]
    assert int((r["out_new"] >= 0).sum()) == fx["counts"]["out_entering"]
    eng.close()


@pytest.mark.parametrize("name", sorted(EC.geometries()))
def test_fp32_regions_against_fp64(name):
    planes = EC.geometries()[name]
    e64, e32 = engine_for(planes, 64), engine_for(planes, 32)
    q, r64 = results(e64, name, planes)
    _, r32 = results(e32, name, planes)
    # points away from every plane by more than FP32 rounding land alike
    x = q["where_x"]
    gap = np.min([np.min(np.abs(x[:, a:a + 1] - planes[a][None, :]), axis=1) for a in range(3)], axis=0)
    far = gap > 1e-5
    assert np.array_equal(r32["where"][far], r64["where"][far])
    # hownear within FP32 rounding of the coordinates
    assert np.allclose(r32["near"], r64["near"], rtol=0, atol=4e-6)
    # howfar: same region for steps not within FP32 rounding of a face
    clear = np.abs(r64["in_t"] - q["in_t"]) > 1e-4 * np.maximum(1.0, q["in_t"])
    clear |= r64["in_new"] == q["in_ireg"]
    agree = np.mean(r32["in_new"][clear] == r64["in_new"][clear])
    assert agree > 0.995, agree
    e64.close()
    e32.close()


def test_region_query_refuses_out_of_range_regions():
    planes = EC.geometries()["water30"]
    eng = engine_for(planes, 64)
    with pytest.raises(eg.EGSError) as ex:
        eng.geometry_query(2, np.array([27000], np.int32), np.zeros((1, 3)))
    assert ex.value.code == 1
    eng.close()
