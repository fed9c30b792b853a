"""Stage the EGSnrc cross-section data files this engine reads into this folder.

The transport engine reads the same data files as EGSnrc's HATCH step: the
PEGS4 material files (``pegs4/data/521icru.pegs4dat``; ``700icru.pegs4dat``,
the AE = 0.700 MeV media of the BEAMnrc examples), the screened-Rutherford
multiple-scattering surface (``data/msnew.data``), the XCOM photon cross
sections (``data/xcom_{photo,pair,triplet,rayleigh}.data``), the bound-Compton
correction (``data/compton_sigma.data``), the Compton-profile shell list
(``data/incoh.data``), the photo-absorption edge fits and shell probabilities
(``data/photo_cs.data``, ``data/photo_relax.data``) and the IAM atomic form
factors (``pegs4/pgs4form.dat``).  They are physical data distributed with
EGSnrc under the AGPL (see ``LICENCE_DATA.md``); the files are copied verbatim
so that a run needs no EGSnrc installation.

Usage::

    python egsnrc_gb300/data/stage_data.py <HEN_HOUSE>
"""
import os
import shutil
import sys

FILES = [
    ("pegs4/data/521icru.pegs4dat", "521icru.pegs4dat"),
    ("pegs4/data/700icru.pegs4dat", "700icru.pegs4dat"),
    ("pegs4/pgs4form.dat", "pgs4form.dat"),
    ("data/msnew.data", "msnew.data"),
    ("data/xcom_photo.data", "xcom_photo.data"),
    ("data/xcom_pair.data", "xcom_pair.data"),
    ("data/xcom_triplet.data", "xcom_triplet.data"),
    ("data/xcom_rayleigh.data", "xcom_rayleigh.data"),
    ("data/compton_sigma.data", "compton_sigma.data"),
    ("data/incoh.data", "incoh.data"),
    ("data/photo_cs.data", "photo_cs.data"),
    ("data/photo_relax.data", "photo_relax.data"),
]


def stage(hen_house: str, dest: str) -> None:
    for src, name in FILES:
        shutil.copyfile(os.path.join(hen_house, src), os.path.join(dest, name))
    shutil.copyfile(os.path.join(hen_house, "data", "LICENCE.md"),
                    os.path.join(dest, "LICENCE_DATA.md"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: stage_data.py <HEN_HOUSE>")
    stage(sys.argv[1], os.path.dirname(os.path.abspath(__file__)))
