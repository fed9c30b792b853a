"""Regenerates the fixtures in this folder from an EGSnrc HEN_HOUSE tree.

  ndgeom_egsphant.egsphant.gz  egs++/geometry/examples/ndgeom_egsphant.egsphant
                               (the reference's example voxel phantom), gzipped
  EXslabs.egsphsp1.gz          omega/beamnrc/BEAMnrc_examples/EXslabs/EXslabs.egsphsp1
  EX16MVp.egsphsp1.gz          omega/beamnrc/BEAMnrc_examples/EX16MVp/EX16MVp.egsphsp1
                               (BEAMnrc example phase-space files, MODE0 and
                               MODE2, shipped with the reference), gzipped

Usage: python tests/golden/make_fixtures.py <HEN_HOUSE>
"""
import gzip
import os
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))

if __name__ == "__main__":
    hh = sys.argv[1]
    src = os.path.join(hh, "egs++", "geometry", "examples", "ndgeom_egsphant.egsphant")
    with open(src, "rb") as f, gzip.open(os.path.join(HERE, "ndgeom_egsphant.egsphant.gz"), "wb", 9) as g:
        shutil.copyfileobj(f, g)
    for name in ("EXslabs", "EX16MVp"):
        src = os.path.join(hh, "omega", "beamnrc", "BEAMnrc_examples", name, name + ".egsphsp1")
        with open(src, "rb") as f, gzip.open(os.path.join(HERE, name + ".egsphsp1.gz"), "wb", 9) as g:
            shutil.copyfileobj(f, g)
