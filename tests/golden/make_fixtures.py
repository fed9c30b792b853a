"""Regenerates the fixtures in this folder from an EGSnrc HEN_HOUSE tree.

  ndgeom_egsphant.egsphant.gz  egs++/geometry/examples/ndgeom_egsphant.egsphant
                               (the reference's example voxel phantom), gzipped

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
