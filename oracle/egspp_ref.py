"""ORACLE -- test infrastructure only: ctypes binding of oracle/_ref/libegspp_ref.so,
the reference's own egs++ XYZ geometry, parallel beam, rectangle shape,
spectra and RANMAR compiled from the reference's sources with the harness
oracle/egspp_ref.cpp (oracle/Makefile, target `ref`).  The library exists only
where the reference's sources were present at build time; `available()` says
whether it does.  Used by tests/ and the fixture script in tests/golden/ as
the checker; never by the product path.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_ref", "libegspp_ref.so")

_L = None


def available():
    return os.path.exists(LIB_PATH)


def lib():
    global _L
    if _L is None:
        # egs++'s geometry registry reads HEN_HOUSE while the library loads
        # (egs_base_geometry.cpp:90-110: it only forms a plug-in path from it;
        # nothing is loaded from there)
        os.environ.setdefault("HEN_HOUSE", "/nonexistent/")
        L = C.CDLL(LIB_PATH)
        vp = C.c_void_p
        L.egsref_xyz_new.restype = vp
        L.egsref_xyz_new.argtypes = [C.c_int, C.c_int, C.c_int, vp, vp, vp]
        L.egsref_xyz_free.argtypes = [vp]
        L.egsref_boundary_tolerance.restype = C.c_double
        L.egsref_boundary_tolerance.argtypes = [vp]
        L.egsref_xyz_iswhere.argtypes = [vp, C.c_longlong, vp, vp]
        L.egsref_xyz_howfar.argtypes = [vp, C.c_longlong, vp, vp, vp, vp, vp]
        L.egsref_xyz_hownear.argtypes = [vp, C.c_longlong, vp, vp, vp]
        L.egsref_parallel_beam.restype = C.c_longlong
        L.egsref_parallel_beam.argtypes = [C.c_char_p, C.c_int, vp, C.c_double, vp, vp, C.c_longlong, C.c_int, vp]
        _L = L
    return _L


def _p(a):
    return a.ctypes.data


class XYZ:
    """The reference's EGS_XYZGeometry over the given plane positions."""

    def __init__(self, xb, yb, zb):
        self.b = [np.ascontiguousarray(v, dtype=np.float64) for v in (xb, yb, zb)]
        n = [len(v) - 1 for v in self.b]
        self.h = lib().egsref_xyz_new(n[0], n[1], n[2], _p(self.b[0]), _p(self.b[1]), _p(self.b[2]))

    def close(self):
        if self.h:
            lib().egsref_xyz_free(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def boundary_tolerance(self):
        return lib().egsref_boundary_tolerance(self.h)

    def is_where(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(len(x), dtype=np.int32)
        lib().egsref_xyz_iswhere(self.h, len(x), _p(x), _p(out))
        return out

    def howfar(self, ireg, x, u, t):
        ireg = np.ascontiguousarray(ireg, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64)
        u = np.ascontiguousarray(u, dtype=np.float64)
        t = np.array(t, dtype=np.float64)
        out = np.empty(len(ireg), dtype=np.int32)
        lib().egsref_xyz_howfar(self.h, len(ireg), _p(ireg), _p(x), _p(u), _p(t), _p(out))
        return out, t

    def hownear(self, ireg, x):
        ireg = np.ascontiguousarray(ireg, dtype=np.int32)
        x = np.ascontiguousarray(x, dtype=np.float64)
        out = np.empty(len(ireg), dtype=np.float64)
        lib().egsref_xyz_hownear(self.h, len(ireg), _p(ireg), _p(x), _p(out))
        return out


def spectrum_block(edges, counts_per_mev):
    """An egs++ ':start spectrum:' block for a histogram in counts per MeV
    (EGS_BaseSpectrum::createSpectrum, egs_spectra.cpp:706-790, mode 1)."""
    e = " ".join("%.17g" % v for v in edges)
    p = " ".join("%.17g" % v for v in counts_per_mev)
    return (":start spectrum:\n type = tabulated spectrum\n energies = %s\n probabilities = %s\n"
            " spectrum mode = 1\n:stop spectrum:\n" % (e, p))


def mono_block(energy):
    return ":start spectrum:\n type = monoenergetic\n energy = %.17g\n:stop spectrum:\n" % energy


def parallel_beam(spectrum, charge, rect, z0, n, seed=0, geometry=None):
    """n particles of the reference's EGS_ParallelBeam along +z from the
    rectangle rect = (xmin, xmax, ymin, ymax) in the plane z = z0, entered into
    `geometry` (an XYZ) as simulateSingleShower does.  Rows: charge, kinetic
    energy, x, y, z, u, v, w, region."""
    out = np.empty(9 * n, dtype=np.float64)
    r = np.array(rect, dtype=np.float64)
    d = np.array([0.0, 0.0, 1.0])
    got = lib().egsref_parallel_beam(spectrum.encode(), int(charge), _p(r), float(z0), _p(d),
                                     geometry.h if geometry is not None else None, int(n), int(seed), _p(out))
    if got != n:
        raise RuntimeError("reference parallel beam: input error")
    return out.reshape(n, 9)
