"""Writes egspp_reference.json: outputs of the reference's own egs++ classes
(EGS_XYZGeometry, EGS_ParallelBeam with its rectangle shape and tabulated
spectrum, RANMAR), compiled from the reference's sources into
oracle/_ref/libegspp_ref.so by oracle/Makefile (target `ref`).

  geometry.<case>   SHA-256 digests of the reference's isWhere, howfar (from
                    inside and from outside) and hownear results on the query
                    sets of egspp_cases.py, with the digest of the inputs and
                    a few summary counts
  source.<case>     histograms of SOURCE_SAMPLES particles of the reference's
                    parallel beam after entering the phantom: kinetic energy
                    and entry x and y

Usage: python tests/golden/make_egspp_fixtures.py   (after building oracle/_ref)
"""
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, HERE)

import egspp_cases as EC  # noqa: E402
from oracle import egspp_ref as R  # noqa: E402

OUT = os.path.join(HERE, "egspp_reference.json")


def reference_geometry(name, planes):
    q = EC.queries(name, planes)
    g = R.XYZ(*planes)
    where = g.is_where(q["where_x"])
    in_new, in_t = g.howfar(q["in_ireg"], q["in_x"], q["in_u"], q["in_t"])
    out_new, out_t = g.howfar(np.full(len(q["out_t"]), -1, np.int32), q["out_x"], q["out_u"], q["out_t"])
    near = g.hownear(q["near_ireg"], q["near_x"])
    res = dict(inputs=EC.input_digest(q), boundary_tolerance=g.boundary_tolerance(),
               where=EC.digest(where), howfar_in=EC.digest(in_new, in_t), howfar_out=EC.digest(out_new, out_t),
               hownear=EC.digest(near),
               counts=dict(where_outside=int((where < 0).sum()), in_crossing=int((in_new != q["in_ireg"]).sum()),
                           in_leaving=int((in_new < 0).sum()), out_entering=int((out_new >= 0).sum())))
    g.close()
    return res, dict(where=where, in_new=in_new, in_t=in_t, out_new=out_new, out_t=out_t, near=near)


def source_cases():
    from egsnrc_gb300 import workloads as W
    edges, counts = W.bremsstrahlung_spectrum()
    return {
        "slab64_photons": dict(spectrum=R.spectrum_block(edges, counts), charge=0, rect=(-5.0, 5.0, -5.0, 5.0),
                               z0=-1.0, workload="slab64", erange=(0.1, 6.0)),
        "water128e_electrons": dict(spectrum=R.mono_block(20.0), charge=-1, rect=(-5.0, 5.0, -5.0, 5.0),
                                    z0=-1.0, workload="water128e", erange=(19.5, 20.5)),
    }


def histograms(parts, erange):
    he, _ = np.histogram(parts[:, 1], bins=EC.E_BINS, range=erange)
    hx, _ = np.histogram(parts[:, 2], bins=EC.XY_BINS, range=(-5.0, 5.0))
    hy, _ = np.histogram(parts[:, 3], bins=EC.XY_BINS, range=(-5.0, 5.0))
    return he, hx, hy


def reference_source(case):
    from egsnrc_gb300 import workloads as W
    wl = W.WORKLOADS[case["workload"]]()
    gb = wl["geometry"]
    g = R.XYZ(gb.xb, gb.yb, gb.zb)
    parts = R.parallel_beam(case["spectrum"], case["charge"], case["rect"], case["z0"], EC.SOURCE_SAMPLES, 0, g)
    g.close()
    he, hx, hy = histograms(parts, case["erange"])
    return dict(n=EC.SOURCE_SAMPLES, erange=list(case["erange"]), energy=he.tolist(), x=hx.tolist(), y=hy.tolist(),
                entered=int((parts[:, 8] >= 0).sum()), z_entry=sorted(set(parts[:, 4].tolist()))[:4],
                mean_energy=float(parts[:, 1].mean()))


def main():
    if not R.available():
        sys.exit("oracle/_ref/libegspp_ref.so is missing: build oracle/_ref first")
    out = dict(geometry={}, source={})
    for name, planes in EC.geometries().items():
        out["geometry"][name], _ = reference_geometry(name, planes)
    for name, case in source_cases().items():
        out["source"][name] = reference_source(case)
    with open(OUT, "w") as f:
        json.dump(out, f, indent=1)
    print(OUT)


if __name__ == "__main__":
    main()
