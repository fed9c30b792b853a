"""Host data layer (the HATCH restatement) pinned against the raw data files.

Each check rebuilds a quantity independently in numpy from the staged data
files (the PEGS4 material file and the XCOM tables) and compares it with the
table the engine and the oracle read.
"""
import math
import os

import numpy as np
import pytest

from egsnrc_gb300 import DATA_DIR, PEGS_FILE, RM
from oracle.oracle_binding import Oracle, lib

MEDIA = ["H2O521ICRU", "LUNG521ICRU", "ICRPBONE521ICRU", "ICRUTISSUE521ICRU"]


@pytest.fixture(scope="module")
def ora():
    return Oracle(MEDIA, ecut=0.521, pcut=0.01)


def pegs_block(name):
    """Independent parse of one PEGS4 medium block (numbers only)."""
    lines = open(PEGS_FILE).read().splitlines()
    i = next(k for k, l in enumerate(lines) if l.startswith(" MEDIUM=") and l[8:32].strip() == name)
    comp = lines[i + 1]
    ne = int(comp.split("NE=")[1].split(",")[0])
    elems = []
    for k in range(ne):
        l = lines[i + 2 + k]
        elems.append((float(l.split(",Z=")[1].split(",")[0]), float(l.split(",A=")[1].split(",")[0]),
                      float(l.split(",PZ=")[1].split(",")[0])))
    rho = float(comp.split("RHO=")[1].split(",")[0])
    j = i + 2 + ne
    toks = []
    sizes = None
    for l in lines[j:j + 4000]:
        if l.startswith(" MEDIUM="):
            break
        if sizes is None and len(toks) == 5:
            sizes = [int(x) for x in l.split()]
            continue
        toks.extend(float(x) for x in l.replace("D", "E").split())
    rlc, ae, ap, ue, up = toks[:5]
    meke = sizes[3]
    # DL (36), DELCM..DELPOS (7), XR0.. (4), EKE0 EKE1 (2), then 16 * MEKE
    off = 5 + 36 + 7 + 4
    eke0, eke1 = toks[off], toks[off + 1]
    etab = np.array(toks[off + 2:off + 2 + 16 * meke]).reshape(meke, 16)
    return dict(rho=rho, elems=elems, rlc=rlc, ae=ae, ap=ap, up=up, meke=meke, eke0=eke0, eke1=eke1, etab=etab)


@pytest.mark.parametrize("im,name", list(enumerate(MEDIA)))
def test_electron_tables_match_pegs4(ora, im, name):
    b = pegs_block(name)
    for i in (3, 40, 90, 140):
        # energy at the middle of PWLF bin i (1-based i+1)
        elke = (i + 1.5 - b["eke0"]) / b["eke1"]
        eke = math.exp(elke)
        got = ora.electron_xsec(im, eke)
        row = b["etab"][i]
        esig = (row[0] + row[1] * elke) / b["rlc"]
        ededx = (row[4] + row[5] * elke) / b["rlc"]
        pdedx = (row[6] + row[7] * elke) / b["rlc"]
        ebr1 = row[8] + row[9] * elke
        pbr2 = row[12] + row[13] * elke
        assert got[0] == pytest.approx(esig, rel=1e-9)
        assert got[2] == pytest.approx(ededx, rel=1e-9)
        assert got[3] == pytest.approx(pdedx, rel=1e-9)
        assert got[4] == pytest.approx(ebr1, rel=1e-9, abs=1e-12)
        assert got[6] == pytest.approx(pbr2, rel=1e-9, abs=1e-12)


def read_xcom(fname):
    toks = open(os.path.join(DATA_DIR, fname)).read().split()
    out, p = {}, 0
    for z in range(1, 101):
        n = int(toks[p]); p += 1
        v = np.array(toks[p:p + 2 * n], dtype=float).reshape(n, 2); p += 2 * n
        out[z] = v
    return out


def loglog(tab, gle):
    e, f = tab[:, 0], tab[:, 1]
    k = np.searchsorted(e, gle, side="right") - 1
    while e[k + 1] - e[k] <= 0:
        k += 1
    p = (gle - e[k]) / (e[k + 1] - e[k])
    return math.exp(p * f[k + 1] + (1 - p) * f[k])


def kn_total(e):
    """Klein-Nishina total cross section per electron (barn), textbook form."""
    k = e / RM
    r0sq = 0.0794077   # classical electron radius squared, barn
    a = (1 + k) / k ** 2 * (2 * (1 + k) / (1 + 2 * k) - math.log(1 + 2 * k) / k)
    b = math.log(1 + 2 * k) / (2 * k) - (1 + 3 * k) / (1 + 2 * k) ** 2
    return 2 * math.pi * r0sq * (a + b)


@pytest.mark.parametrize("e", [0.03, 0.2, 1.0, 5.0, 40.0])
def test_klein_nishina(e):
    assert lib().oracle_kn_sigma0(e) == pytest.approx(kn_total(e), rel=2e-4)


def test_water_attenuation_from_xcom(ora):
    """gmfp at grid energies rebuilt from the XCOM files for water (H2, O)."""
    photo, pair, trip = read_xcom("xcom_photo.data"), read_xcom("xcom_pair.data"), read_xcom("xcom_triplet.data")
    bc = open(os.path.join(DATA_DIR, "compton_sigma.data")).read().split()
    emin, emax, nbc = float(bc[0]), float(bc[1]), int(bc[2])
    bcz = np.array(bc[3:3 + 100 * nbc], dtype=float).reshape(100, nbc)
    b = pegs_block("H2O521ICRU")
    elems = [(1, 1.008, 2.0), (8, 15.999, 1.0)]
    sumZ = sum(pz * z for z, a, pz in elems)
    sumA = sum(pz * a for z, a, pz in elems)
    bcd = np.log(sum(pz * z * bcz[int(z) - 1] for z, a, pz in elems) / sumZ)
    dle = math.log(emax / emin) / (nbc - 1)
    ge1 = 1999 / math.log(b["up"] / b["ap"])
    ge0 = 1 - ge1 * math.log(b["ap"])
    for i in (100, 700, 1200, 1650):   # grid index, 1-based
        gle = (i - ge0) / ge1
        e = math.exp(gle)
        sph = sum(pz * loglog(photo[z], gle) for z, a, pz in elems)

        def thr(tab, eth):
            et = np.concatenate([[math.log(eth)], tab[:, 0]])
            ft = tab[:, 1] - 3 * np.log(1 - eth / np.exp(tab[:, 0]))
            ft = np.concatenate([[ft[0]], ft])
            if gle < et[0]:
                return 0.0
            return loglog(np.stack([et, ft], 1), gle) * (1 - eth / e) ** 3
        sp = sum(pz * (thr(pair[z], 2 * RM) + thr(trip[z], 4 * RM)) for z, a, pz in elems)
        aj = 1 + math.log(e / emin) / dle
        j = int(aj)
        aj -= j
        bcf = math.exp(bcd[j - 1] * (1 - aj) + bcd[j] * aj) if e < emax else 1.0
        skn = sumZ * kn_total(e) * bcf
        sigma = sph + sp + skn
        gmfp = 1 / (sigma * b["rho"] / (sumA * 1.6605655))
        got = ora.photon_xsec(0, e)
        assert got[0] == pytest.approx(gmfp, rel=5e-4)
        assert got[1] == pytest.approx(sp / sigma, rel=5e-4, abs=1e-9)
        assert got[2] == pytest.approx((sp + skn) / sigma, rel=5e-4)


def test_attenuation_of_media_is_physical(ora):
    # mu/rho of water at 1 MeV (XCOM total without coherent ~ 0.0707 cm^2/g)
    assert 1 / ora.photon_xsec(0, 1.0)[0] == pytest.approx(0.0707, rel=0.01)
    # lung at its PEGS density scales as rho; bone is denser and higher-Z
    mu_w = 1 / ora.photon_xsec(0, 0.05)[0]
    mu_b = 1 / ora.photon_xsec(2, 0.05)[0] / 1.85
    assert mu_b > 1.5 * mu_w
