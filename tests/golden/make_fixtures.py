"""Regenerates the fixtures in this folder from an EGSnrc HEN_HOUSE tree.

  ndgeom_egsphant.egsphant.gz  egs++/geometry/examples/ndgeom_egsphant.egsphant
                               (the reference's example voxel phantom), gzipped
  EXslabs.egsphsp1.gz          omega/beamnrc/BEAMnrc_examples/EXslabs/EXslabs.egsphsp1
  EX16MVp.egsphsp1.gz          omega/beamnrc/BEAMnrc_examples/EX16MVp/EX16MVp.egsphsp1
                               (BEAMnrc example phase-space files, MODE0 and
                               MODE2, shipped with the reference), gzipped
  beamnrc_examples.json        the results that the reference's own listings
                               EXslabs.egslst and EXphantom.egslst (BEAMnrc,
                               EGSnrc, 2004) print for those runs: dose per
                               zone with its uncertainty, the scoring-plane
                               fluence, the step counts, the PRESTA-I skin
                               depth and the phase-space source counts that
                               set the dose normalisation

Usage: python tests/golden/make_fixtures.py <HEN_HOUSE>
"""
import gzip
import json
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
NUM = r"[-+]?\d*\.?\d+(?:[EeDd][-+]?\d+)?"


def _f(s):
    return float(s.replace("D", "E").replace("d", "e"))


def dose_zones(lines):
    """Rows of the 'TOTAL DOSE PER INCIDENT PARTICLE' table: zone, mass (g),
    dose (Gy), its uncertainty (%), energy deposited (J)."""
    i = next(k for k, l in enumerate(lines) if "TOTAL DOSE PER INCIDENT PARTICLE" in l)
    out = []
    rx = re.compile(r"^\s*(\d+)\s+(%s)\s+(%s)\s*\+/-\s*(%s)%%\s+(%s)\s*\+/-" % (NUM, NUM, NUM, NUM))
    for l in lines[i + 1:]:
        m = rx.match(l)
        if m:
            out.append(dict(zone=int(m.group(1)), mass_g=_f(m.group(2)), dose_gy=_f(m.group(3)),
                            sigma_pct=_f(m.group(4)), energy_j=_f(m.group(5))))
        elif out:
            break
    return out


def value_pct(lines, key):
    """A 'key  value +/- pct%' line."""
    for l in lines:
        if key in l:
            m = re.search(r"(%s)\s*\+/-\s*(%s)%%" % (NUM, NUM), l)
            if m:
                return dict(value=_f(m.group(1)), sigma_pct=_f(m.group(2)))
    raise KeyError(key)


def int_after(lines, key):
    for l in lines:
        if key in l:
            return _f(re.findall(NUM, l.split(key, 1)[1])[0])
    raise KeyError(key)


def plane_zone1(lines, kind):
    """Zone 1 of the first-crossing scoring-plane table for ELECTRONS or
    PHOTONS: number, fluence, mean energy, mean angle (value, %)."""
    i = next(k for k, l in enumerate(lines) if "FIRST TIME CROSSINGS" in l)
    j = next(k for k in range(i, len(lines)) if lines[k].strip() == kind)
    rx = re.compile(r"^\s*1\s+" + r"\s+".join([r"(%s)\s*\+-\s*(%s)%%\*?" % (NUM, NUM)] * 4))
    m = rx.match(lines[j + 1])
    v = [_f(x) for x in m.groups()]
    tot = next(l for l in lines[j + 1:] if l.strip().startswith("Tot"))
    t = re.search(r"(%s)\s*\+-\s*(%s)%%" % (NUM, NUM), tot)
    return dict(number=v[0:2], fluence=v[2:4], energy_mev=v[4:6], angle_deg=v[6:8],
                total_number=[_f(t.group(1)), _f(t.group(2))])


def listings(hh):
    ex = os.path.join(hh, "omega", "beamnrc", "BEAMnrc_examples")
    slabs = open(os.path.join(ex, "EXslabs", "EXslabs.egslst")).read().splitlines()
    phan = open(os.path.join(ex, "EXphantom", "EXphantom.egslst")).read().splitlines()
    radii = next(l for l in slabs if re.match(r"^\s*1\s+1\s+100\.00", l))
    return {
        "EXslabs": dict(
            dose=dose_zones(slabs),
            charged_steps_per_history=value_pct(slabs, "# CHARGED PARTICLE STEPS/INITIAL HISTORY"),
            presta2_step_fraction=value_pct(slabs, "# PRESTA-II STEPS/TOTAL # CHARGED PARTICLE STEPS"),
            skindepth_mfp=int_after(slabs, "Skin-depth for boundary crossing (MFP)"),
            brems_events=int_after(slabs, "NO. OF BREMSSTRAHLUNG EVENTS IN THIS RUN:"),
            histories=int_after(slabs, "Max # of histories: to run"),
            plane_radii_cm=[_f(x) for x in radii.split()[4:]],
            plane_electrons=plane_zone1(slabs, "ELECTRONS"),
            plane_photons=plane_zone1(slabs, "PHOTONS")),
        "EXphantom": dict(
            dose=dose_zones(phan),
            histories=int_after(phan, "Max # of histories: to run"),
            phsp_particles=int_after(phan, "total # of particles"),
            phsp_photons=int_after(phan, "# of photons"),
            phsp_incident=int_after(phan, "original source"),
            recycle=int_after(phan, "# of times to recycle particles"),
            particles_used=int_after(phan, "Used total of")),
    }


def gz(src, name):
    """Gzips src to name here (no time stamp, so reruns give the same bytes)."""
    with open(src, "rb") as f, open(os.path.join(HERE, name), "wb") as raw, \
            gzip.GzipFile(filename="", mode="wb", compresslevel=9, fileobj=raw, mtime=0) as g:
        shutil.copyfileobj(f, g)


if __name__ == "__main__":
    hh = sys.argv[1]
    gz(os.path.join(hh, "egs++", "geometry", "examples", "ndgeom_egsphant.egsphant"), "ndgeom_egsphant.egsphant.gz")
    for name in ("EXslabs", "EX16MVp"):
        gz(os.path.join(hh, "omega", "beamnrc", "BEAMnrc_examples", name, name + ".egsphsp1"), name + ".egsphsp1.gz")
    with open(os.path.join(HERE, "beamnrc_examples.json"), "w") as f:
        json.dump(listings(hh), f, indent=1)
        f.write("\n")
