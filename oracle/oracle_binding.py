"""ORACLE -- test infrastructure only: ctypes binding of the FP64 CPU oracle
(oracle/egs_oracle.cpp).  Used by tests/, __graft_entry__.smoke() and the
CPU-baseline leg of bench.py as the checker; never by the product path."""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
LIB_PATH = os.path.join(HERE, "liboracle.so")
# the same restatement built for speed (-O3 -ffast-math, the reference's own
# Fortran flags); the CPU-baseline timings of bench.py use it, the parity
# checks use LIB_PATH (no contraction, rounding like the GPU's FP64 build)
FAST_LIB_PATH = os.path.join(HERE, "liboracle_fast.so")
DATA_DIR = os.path.join(ROOT, "egsnrc_gb300", "data")
PEGS_FILE = os.path.join(DATA_DIR, "521icru.pegs4dat")

_L = None
_LF = None


def lib(fast=False):
    global _L, _LF
    if fast:
        if _LF is None:
            if not os.path.exists(FAST_LIB_PATH):
                import subprocess
                subprocess.run(["make", "-s", "liboracle_fast.so"], cwd=HERE, check=True)
            _LF = _declare(C.CDLL(FAST_LIB_PATH))
        return _LF
    if _L is None:
        if not os.path.exists(LIB_PATH):
            import subprocess
            subprocess.run(["make", "-s"], cwd=HERE, check=True)
        _L = _declare(C.CDLL(LIB_PATH))
    return _L


def _declare(L):
    if True:   # argument types of every exported function
        vp, dp, i64 = C.c_void_p, C.POINTER(C.c_double), C.c_longlong
        L.oracle_create.restype = vp
        L.oracle_create.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int, C.c_double, C.c_double]
        L.oracle_create_bca.restype = vp
        L.oracle_create_bca.argtypes = [C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int, C.c_double,
                                        C.c_double, C.c_int, C.c_double]
        L.oracle_skindepth.restype = C.c_double
        L.oracle_skindepth.argtypes = [vp]
        L.oracle_charged_steps.restype = C.c_double
        L.oracle_charged_steps.argtypes = [vp]
        L.oracle_msdist_steps.restype = C.c_double
        L.oracle_msdist_steps.argtypes = [vp]
        L.oracle_destroy.argtypes = [vp]
        L.oracle_set_geometry.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, dp, dp, C.POINTER(C.c_int32), dp]
        L.oracle_set_source.argtypes = [vp, C.c_void_p]
        L.oracle_set_howfarless.argtypes = [vp, C.c_int]
        L.oracle_set_smax.argtypes = [vp, C.c_double]
        L.oracle_set_escape_log.argtypes = [vp, C.c_int]
        L.oracle_get_escapes.restype = i64
        L.oracle_get_escapes.argtypes = [vp, dp, i64]
        L.oracle_run.argtypes = [vp, i64, i64, C.c_int, C.c_uint32, C.c_int, C.c_int]
        L.oracle_set_history_tally.argtypes = [vp, i64, i64]
        L.oracle_get_history_tally.argtypes = [vp, dp]
        L.oracle_get_tallies.argtypes = [vp, dp, dp, dp]
        L.oracle_philox.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.oracle_ranmar.argtypes = [C.c_int, C.c_int, i64, dp]
        L.oracle_child_sid.restype = C.c_uint64
        L.oracle_child_sid.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32]
        L.oracle_kn_sigma0.restype = C.c_double
        L.oracle_kn_sigma0.argtypes = [C.c_double]
        L.oracle_photon_xsec.argtypes = [vp, C.c_int, C.c_double, dp]
        L.oracle_electron_xsec.argtypes = [vp, C.c_int, C.c_double, dp]
        L.oracle_geometry_query.argtypes = [vp, C.c_int, i64, vp, vp, vp, vp, vp]
        L.oracle_sample_source.argtypes = [vp, i64, i64, C.c_uint32, dp]
        L.oracle_sample_interaction.argtypes = [vp, C.c_int, C.c_int, C.c_double, i64, C.c_uint32, dp]
        L.oracle_medium_pair.argtypes = [vp, C.c_int, dp]
        L.oracle_medium_thresholds.argtypes = [vp, C.c_int, dp]
        L.oracle_medium_elements.argtypes = [vp, C.c_int, C.c_int, dp]
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class Oracle:
    def __init__(self, media, ecut=0.521, pcut=0.010, pegs_file=PEGS_FILE, bca_algorithm=0, skindepth=3.0,
                 fast=False):
        """bca_algorithm 0: EXACT boundary crossing, 1: PRESTA-I (with
        skindepth <= 1e-4 the old PRESTA default skin depth).  fast: the
        build for timing (FAST_LIB_PATH)."""
        L = lib(fast)
        names = (C.c_char_p * len(media))(*[m.encode() for m in media])
        h = L.oracle_create_bca(DATA_DIR.encode(), pegs_file.encode(), names, len(media), ecut, pcut,
                                int(bca_algorithm), float(skindepth))
        if not h:
            raise RuntimeError("oracle: media load failed")
        self.h = C.c_void_p(h)
        self.L = L
        self.geom = None

    def set_geometry(self, g):
        self.geom = g
        rc = self.L.oracle_set_geometry(self.h, g.nx, g.ny, g.nz, _dp(g.xb), _dp(g.yb), _dp(g.zb),
                                        g.med.ctypes.data_as(C.POINTER(C.c_int32)), _dp(g.rhor))
        if rc:
            raise RuntimeError("oracle: bad geometry")

    def set_howfarless(self, on=True):
        """DOSXYZnrc HOWFARLESS transport in the current (homogeneous) phantom."""
        assert self.L.oracle_set_howfarless(self.h, int(bool(on))) == 0

    def skindepth(self):
        """The skin depth for boundary crossing in use (elastic MFPs)."""
        return self.L.oracle_skindepth(self.h)

    def charged_steps(self):
        """Charged-particle steps of non-zero length so far."""
        return self.L.oracle_charged_steps(self.h)

    def msdist_steps(self):
        """PRESTA-II (msdist) steps so far."""
        return self.L.oracle_msdist_steps(self.h)

    def set_smax(self, smax):
        """Maximum charged-particle step in cm (<= 0: no limit)."""
        assert self.L.oracle_set_smax(self.h, float(smax)) == 0

    def set_escape_log(self, on=True):
        """Record (or stop recording) every particle that leaves the phantom."""
        assert self.L.oracle_set_escape_log(self.h, int(bool(on))) == 0

    def escapes(self):
        """The recorded escapes as an (n, 10) array: charge, kinetic energy,
        x, y, z, u, v, w, weight, history."""
        n = self.L.oracle_get_escapes(self.h, None, 0)
        out = np.zeros((n, 10))
        if n:
            self.L.oracle_get_escapes(self.h, _dp(out), n)
        return out

    def set_source(self, src):
        self.src = src
        self.L.oracle_set_source(self.h, C.byref(src.s))

    def run(self, n, nbatch=10, seed=1, first=0, ranmar=False, threads=1):
        rc = self.L.oracle_run(self.h, int(first), int(n), int(nbatch), int(seed), int(bool(ranmar)), int(threads))
        if rc:
            raise RuntimeError("oracle run error %d" % rc)

    def tallies(self):
        nv = self.geom.nvox
        s, s2, t = np.zeros(nv), np.zeros(nv), np.zeros(8)
        self.L.oracle_get_tallies(self.h, _dp(s), _dp(s2), _dp(t))
        return s, s2, t

    def set_history_tally(self, first, n):
        self._hist_n = n
        self.L.oracle_set_history_tally(self.h, int(first), int(n))

    def history_tally(self):
        out = np.zeros(self._hist_n)
        self.L.oracle_get_history_tally(self.h, _dp(out))
        return out

    def geometry_query(self, op, ireg=None, x=None, u=None, t=None):
        """isWhere (op 0), howfar (op 1; howfarFromOut where ireg < 0) and
        hownear (op 2) on the current phantom, as egsgpu_geometry_query."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = len(x)
        ireg = np.ascontiguousarray(ireg if ireg is not None else np.zeros(n), dtype=np.int32)
        u = np.ascontiguousarray(u if u is not None else np.zeros((n, 3)), dtype=np.float64)
        t = np.array(t if t is not None else np.zeros(n), dtype=np.float64)
        inew = np.zeros(n, dtype=np.int32)
        rc = self.L.oracle_geometry_query(self.h, int(op), n, ireg.ctypes.data, x.ctypes.data, u.ctypes.data,
                                          t.ctypes.data, inew.ctypes.data)
        if rc:
            raise RuntimeError("oracle geometry query: bad arguments")
        return inew, t

    def sample_source(self, n, seed=1, first=0):
        """Source particles of histories [first, first+n) as they enter the
        phantom: rows of charge, kinetic energy, x, y, z, u, v, w, region."""
        out = np.zeros((n, 9))
        if self.L.oracle_sample_source(self.h, int(first), int(n), int(seed), _dp(out)):
            raise RuntimeError("oracle source sampling error")
        return out

    def sample_interaction(self, kind, med, energy, n, seed=1):
        """n samples of one interaction sampler alone (kind 0 Klein-Nishina on
        free electrons, 1 bound Compton, 2 photo-electron direction, 3 pair,
        4 Moller, 5 Bhabha, 6 bremsstrahlung, 7 Rayleigh, 8 annihilation in
        flight); rows of 3 values as
        oracle_sample_interaction describes."""
        out = np.zeros((n, 3))
        rc = self.L.oracle_sample_interaction(self.h, int(kind), int(med), float(energy), int(n), int(seed), _dp(out))
        if rc:
            raise RuntimeError("oracle sampler error %d" % rc)
        return out

    def thresholds(self, med):
        """te (kinetic delta-ray threshold), thmoll (Moller threshold, total
        energy) and ap (bremsstrahlung photon threshold) of medium med, MeV."""
        out = np.zeros(3)
        assert self.L.oracle_medium_thresholds(self.h, int(med), _dp(out)) == 0
        return float(out[0]), float(out[1]), float(out[2])

    def elements(self, med):
        """Atomic numbers and atoms per molecule of medium med (PEGS4)."""
        nmax = 32
        out = np.zeros(1 + 2 * nmax)
        assert self.L.oracle_medium_elements(self.h, int(med), nmax, _dp(out)) == 0
        n = int(out[0])
        return out[1:1 + n].astype(int), out[1 + n:1 + 2 * n].copy()

    def pair_constants(self, med):
        """dl[6][8], delcm and bpar[2] of medium med."""
        out = np.zeros(51)
        assert self.L.oracle_medium_pair(self.h, int(med), _dp(out)) == 0
        return out[:48].reshape(6, 8), out[48], out[49:51]

    def photon_xsec(self, med, e):
        out = np.zeros(4)
        self.L.oracle_photon_xsec(self.h, med, e, _dp(out))
        return out

    def electron_xsec(self, med, eke):
        out = np.zeros(8)
        self.L.oracle_electron_xsec(self.h, med, eke, _dp(out))
        return out

    def close(self):
        if self.h:
            self.L.oracle_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def philox(ctr, key):
    c = (C.c_uint32 * 4)(*ctr)
    k = (C.c_uint32 * 2)(*key)
    o = (C.c_uint32 * 4)()
    lib().oracle_philox(c, k, o)
    return list(o)


def ranmar(n, ixx=0, jxx=0):
    out = np.zeros(n)
    lib().oracle_ranmar(ixx, jxx, n, _dp(out))
    return out
