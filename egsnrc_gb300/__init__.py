"""egsnrc_gb300: GB300-native coupled photon/electron voxel-dose transport.

Python mirror of the egs++ voxel-dose application path (EGS_XYZGeometry +
EGS_ParallelBeam + EGS_DoseScoring), driving the CUDA engine through the C
ABI declared in include/egsgpu.h.  The engine library must be built
(``python -m egsnrc_gb300.build``); importing the transport classes without
it raises instead of falling back to anything else.
"""
import ctypes as C
import math
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
DATA_DIR = os.path.join(HERE, "data")
PEGS_FILE = os.path.join(DATA_DIR, "521icru.pegs4dat")
RM = 0.5109989461

ERRORS = {1: "bad argument", 2: "data file", 3: "medium", 4: "CUDA", 5: "queue capacity",
          6: "iteration cap", 7: "call order"}


class EGSError(RuntimeError):
    """An engine call returned a non-zero status (the C ABI's error class)."""

    def __init__(self, code, msg):
        super().__init__("egsgpu error %d (%s): %s" % (code, ERRORS.get(code, "?"), msg))
        self.code = code


class Config(C.Structure):
    _fields_ = [("ecut", C.c_double), ("pcut", C.c_double), ("estepe", C.c_double), ("ximax", C.c_double),
                ("skindepth", C.c_double), ("precision", C.c_int), ("block_size", C.c_int),
                ("ctas_per_sm", C.c_int), ("chunk", C.c_longlong), ("capacity", C.c_longlong),
                ("requeue_lanes", C.c_int), ("use_graph", C.c_int), ("inter_batch", C.c_int),
                ("howfarless", C.c_int), ("smax", C.c_double), ("bca_algorithm", C.c_int),
                ("loop_cap", C.c_int), ("step_cap", C.c_int), ("fp64_near_faces", C.c_int)]


class SourceStruct(C.Structure):
    _fields_ = [("charge", C.c_int), ("shape", C.c_int), ("pos", C.c_double * 3), ("xmin", C.c_double),
                ("xmax", C.c_double), ("ymin", C.c_double), ("ymax", C.c_double), ("dir", C.c_double * 3),
                ("spectrum", C.c_int), ("energy", C.c_double), ("nbins", C.c_int),
                ("edges", C.POINTER(C.c_double)), ("weights", C.POINTER(C.c_double)),
                ("nphsp", C.c_longlong), ("phsp", C.POINTER(C.c_float)), ("recycle", C.c_int),
                ("rot", C.c_double * 9)]


class PhspInfo(C.Structure):
    _fields_ = [("format", C.c_int), ("has_latch", C.c_int), ("n", C.c_longlong), ("photons", C.c_longlong),
                ("incident", C.c_double), ("ekmax", C.c_double), ("zmin", C.c_double), ("zmax", C.c_double)]


_LIB = None
NOALLOC_MAX_HISTORIES = 2048   # EGSGPU_NOALLOC_MAX_HISTORIES in include/egsgpu.h


def library_path():
    return os.path.join(HERE, "libegsgpu.so")


def load_library():
    """Loads libegsgpu.so (the CUDA engine). Raises if it has not been built."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        raise RuntimeError("libegsgpu.so not built: run `python -m egsnrc_gb300.build`")
    L = C.CDLL(path)
    vp, i64, dp = C.c_void_p, C.c_longlong, C.POINTER(C.c_double)
    L.egsgpu_default_config.argtypes = [C.POINTER(Config)]
    L.egsgpu_create.argtypes = [C.POINTER(Config), C.POINTER(vp)]
    L.egsgpu_load_media.argtypes = [vp, C.c_char_p, C.c_char_p, C.POINTER(C.c_char_p), C.c_int]
    L.egsgpu_set_xyz_geometry.argtypes = [vp, C.c_int, C.c_int, C.c_int, dp, dp, dp, C.POINTER(C.c_int32), dp]
    L.egsgpu_set_source.argtypes = [vp, C.POINTER(SourceStruct)]
    L.egsgpu_run.argtypes = [vp, i64, i64, C.c_int, C.c_uint32, vp]
    L.egsgpu_run_noalloc.argtypes = [vp, i64, i64, C.c_uint32, vp, vp]
    L.egsgpu_reset.argtypes = [vp]
    L.egsgpu_adjoint.argtypes = [vp, i64, i64, C.c_uint32, dp, dp]
    L.egsgpu_set_phantoms.argtypes = [vp, C.c_int, C.POINTER(PhantomStruct)]
    L.egsgpu_run_phantoms.argtypes = [vp, C.c_int, vp]
    L.egsgpu_get_phantom_dose.argtypes = [vp, C.c_int, dp, dp]
    L.egsgpu_get_phantom_info.argtypes = [vp, C.c_int, C.POINTER(C.c_longlong)]
    L.egsgpu_get_tallies.argtypes = [vp, dp, dp, dp]
    L.egsgpu_get_dose.argtypes = [vp, dp, dp]
    L.egsgpu_get_profile.argtypes = [vp, dp]
    L.egsgpu_get_medium.argtypes = [vp, C.c_int, dp]
    L.egsgpu_set_history_tally.argtypes = [vp, i64, i64]
    L.egsgpu_get_history_tally.argtypes = [vp, dp]
    L.egsgpu_geometry_query.argtypes = [vp, C.c_int, i64, vp, vp, vp, vp, vp]
    L.egsgpu_combine_checkpoints.argtypes = [vp, C.c_size_t, vp, C.c_size_t, vp, C.POINTER(C.c_size_t)]
    L.egsgpu_checkpoint.argtypes = [vp, vp, C.POINTER(C.c_size_t)]
    L.egsgpu_restore.argtypes = [vp, vp, C.c_size_t]
    L.egsgpu_read_phsp.argtypes = [C.c_char_p, i64, i64, C.POINTER(PhspInfo), C.POINTER(C.c_float),
                                   C.POINTER(C.c_uint32), C.POINTER(C.c_ubyte)]
    L.egsgpu_last_error.argtypes = [vp]
    L.egsgpu_last_error.restype = C.c_char_p
    L.egsgpu_destroy.argtypes = [vp]
    _LIB = L
    return L


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


class XYZGeometry:
    """EGS_XYZGeometry: plane positions (cm), medium index and relative density per voxel
    (voxel index ix + iy*nx + iz*nx*ny)."""

    def __init__(self, xb, yb, zb, med, rhor=None):
        self.xb = np.ascontiguousarray(xb, dtype=np.float64)
        self.yb = np.ascontiguousarray(yb, dtype=np.float64)
        self.zb = np.ascontiguousarray(zb, dtype=np.float64)
        self.nx, self.ny, self.nz = len(self.xb) - 1, len(self.yb) - 1, len(self.zb) - 1
        nv = self.nx * self.ny * self.nz
        self.med = np.ascontiguousarray(np.broadcast_to(np.asarray(med, dtype=np.int32).ravel(), (nv,)),
                                        dtype=np.int32)
        r = np.ones(nv) if rhor is None else np.asarray(rhor, dtype=np.float64).ravel()
        self.rhor = np.ascontiguousarray(np.broadcast_to(r, (nv,)), dtype=np.float64)

    @staticmethod
    def uniform(n, size, origin=(0.0, 0.0, 0.0), med=0, rhor=None):
        nx, ny, nz = (n, n, n) if np.isscalar(n) else n
        dx, dy, dz = (size, size, size) if np.isscalar(size) else size
        return XYZGeometry(origin[0] + dx * np.arange(nx + 1), origin[1] + dy * np.arange(ny + 1),
                           origin[2] + dz * np.arange(nz + 1), med, rhor)

    @property
    def nvox(self):
        return self.nx * self.ny * self.nz

    def volumes(self):
        dx, dy, dz = np.diff(self.xb), np.diff(self.yb), np.diff(self.zb)
        return (dz[:, None, None] * dy[None, :, None] * dx[None, None, :]).ravel()


class ParallelBeam:
    """EGS_ParallelBeam with a point or rectangle shape and a monoenergetic or
    histogram spectrum (energies are kinetic, MeV)."""

    def __init__(self, charge=0, energy=None, spectrum=None, position=(0.0, 0.0, 0.0), direction=(0.0, 0.0, 1.0),
                 rectangle=None):
        self.s = SourceStruct()
        self.s.charge = int(charge)
        self.s.pos[:] = tuple(float(v) for v in position)
        self.s.dir[:] = tuple(float(v) for v in direction)
        if rectangle is not None:
            self.s.shape = 1
            self.s.xmin, self.s.xmax, self.s.ymin, self.s.ymax = (float(v) for v in rectangle)
        if spectrum is None:
            self.s.spectrum = 0
            self.s.energy = float(energy)
            self._edges = self._w = None
        else:
            edges, weights = spectrum
            self._edges = np.ascontiguousarray(edges, dtype=np.float64)
            self._w = np.ascontiguousarray(weights, dtype=np.float64)
            self.s.spectrum = 1
            self.s.nbins = len(self._w)
            self.s.edges = _dp(self._edges)
            self.s.weights = _dp(self._w)
            self.s.energy = float(self._edges[-1])


class PhantomStruct(C.Structure):
    _fields_ = [("nx", C.c_int), ("ny", C.c_int), ("nz", C.c_int),
                ("xb", C.POINTER(C.c_double)), ("yb", C.POINTER(C.c_double)), ("zb", C.POINTER(C.c_double)),
                ("med", C.POINTER(C.c_int32)), ("rhor", C.POINTER(C.c_double)),
                ("source", SourceStruct), ("seed", C.c_uint32), ("histories", C.c_longlong)]


class PhaseSpaceSource:
    """EGS_PhspSource / DOSXYZnrc isource 2: particles read from a phase-space
    file (formats.read_egsphsp) or given as an (n, 7) float32 array of
    {charge, kinetic energy (MeV), x, y, u, v, weight} (a negative weight
    means w < 0), placed in the plane z = position[2] and shifted by
    position[0], position[1].  Each particle is used recycle + 1 times with
    its weight shared."""

    def __init__(self, particles, position=(0.0, 0.0, 0.0), recycle=0, rotation=None):
        self._p = np.ascontiguousarray(particles, dtype=np.float32).reshape(-1, 7)
        self.s = SourceStruct()
        self.s.shape = 2
        self.s.pos[:] = tuple(float(v) for v in position)
        self.s.dir[:] = (0.0, 0.0, 1.0)
        self.s.nphsp = len(self._p)
        self.s.phsp = self._p.ctypes.data_as(C.POINTER(C.c_float))
        self.s.recycle = int(recycle)
        self.s.energy = float(self._p[:, 1].max())
        self.s.charge = -1 if np.any(self._p[:, 0] != 0) else 0
        if rotation is not None:
            self.s.rot[:] = tuple(float(v) for v in np.asarray(rotation, dtype=np.float64).reshape(9))

    @classmethod
    def from_file(cls, path, shift=(0.0, 0.0, 0.0), recycle=0, rotation=None):
        """The particles of an egsphsp or IAEA file (read_phase_space), on the
        file's plane (z = 0 for egsphsp, the IAEA constant Z), rotated by
        `rotation` and moved by shift, as egs_transformed_source moves them."""
        p, info = read_phase_space(path)
        if not info["zmin"] == info["zmax"]:
            raise ValueError("%s: the particles are not on one plane z = const" % path)
        R = np.eye(3) if rotation is None else np.asarray(rotation, dtype=np.float64).reshape(3, 3)
        # the file's plane z0: R (x, y, z0) + shift = R (x, y, 0) + (shift + z0 R e_z)
        t = np.asarray(shift, dtype=np.float64) + info["zmin"] * R[:, 2]
        src = cls(p, position=tuple(t), recycle=recycle, rotation=rotation)
        src.info = info
        return src


def _mul(A, B):
    # row-by-column sums in the order egs++ forms them (egs_transformations.h:251-259)
    return [[A[i][0] * B[0][j] + A[i][1] * B[1][j] + A[i][2] * B[2][j] for j in range(3)] for i in range(3)]


def _rot(axis, c, s):
    # egs++ EGS_RotationMatrix::rotX/rotY/rotZ (egs++/egs_transformations.h:303-326)
    if axis == 0:
        return [[1.0, 0.0, 0.0], [0.0, c, s], [0.0, -s, c]]
    if axis == 1:
        return [[c, 0.0, -s], [0.0, 1.0, 0.0], [s, 0.0, c]]
    return [[c, s, 0.0], [-s, c, 0.0], [0.0, 0.0, 1.0]]


def _angle(axis, phi):
    return _rot(axis, math.cos(phi), math.sin(phi))


def _rot_from_vector(v):
    # the matrix EGS_RotationMatrix(const EGS_Vector &) builds (egs_transformations.h:153-182):
    # rotY(cos t, -sin t) rotZ(cos p, sin p) with t, p the polar and azimuthal angles of v
    x, y, z = (float(t) for t in v)
    sinz = x * x + y * y
    norm = sinz + z * z
    if norm < 1e-10:
        raise ValueError("no rotation from a zero vector")
    norm = math.sqrt(norm)
    if sinz > 1e-10:
        sinz = math.sqrt(sinz)
        return _mul(_rot(1, z / norm, -sinz / norm), _rot(2, x / sinz, y / sinz))
    if z < 0:
        return _angle(0, math.pi)
    return _rot(2, 1.0, 0.0)


def egs_rotation(rotation=None, rotation_vector=None):
    """The rotation matrix of an egs++ transformation block
    (EGS_AffineTransform::getTransformation, egs++/egs_transformations.cpp:44-108):
    'rotation vector' = v (3 numbers) is the matrix EGS_RotationMatrix(v) builds,
    rotY(cos t, -sin t) rotZ(cos p, sin p) for the polar and azimuthal angles t,
    p of v; 'rotation' = phi theta (2 numbers) is R_z(phi) R_x(theta), alpha
    beta gamma (3 numbers) R_x(alpha) R_y(beta) R_z(gamma), vx vy vz phi (4
    numbers) R1^T R_z(phi) R1 with R1 the matrix of v, or the 9 matrix elements
    row by row.  rotX/Y/Z(c, s) are the matrices of egs_transformations.h:303-326;
    angles in radians.  Formed in the order of operations egs_gpu_app uses, so
    both give the same bits."""
    if rotation_vector is not None and len(rotation_vector) == 3:
        return np.array(_rot_from_vector(rotation_vector))
    r = [] if rotation is None else [float(t) for t in rotation]
    if len(r) == 2:
        m = _mul(_angle(2, r[0]), _angle(0, r[1]))
    elif len(r) == 3:
        m = _mul(_mul(_angle(0, r[0]), _angle(1, r[1])), _angle(2, r[2]))
    elif len(r) == 4:
        r1 = _rot_from_vector(r[:3])
        r1t = [[r1[j][i] for j in range(3)] for i in range(3)]
        m = _mul(_mul(r1t, _angle(2, r[3])), r1)
    elif len(r) == 9:
        m = [r[0:3], r[3:6], r[6:9]]
    else:
        m = _rot(2, 1.0, 0.0)
    return np.array(m, dtype=np.float64)


PHSP_FORMATS = {0: "MODE0", 1: "MODE2", 2: "IAEA"}


def read_phase_space(path, first=0, count=None):
    """Reads a phase-space file through the library's reader (egsgpu_read_phsp;
    host only, no GPU): a BEAMnrc .egsphsp file or an IAEA pair
    <name>.IAEAheader + <name>.IAEAphsp (path = <name>, with or without either
    extension).  Returns (particles, info): particles an (count, 7) float32
    array of {charge, kinetic energy, x, y, u, v, weight} as PhaseSpaceSource
    takes them; info a dict with format, n, photons, incident, ekmax, zmin,
    zmax, has_latch, latch and new_history (arrays over the records read)."""
    L = load_library()
    info = PhspInfo()
    p = str(path).encode()
    rc = L.egsgpu_read_phsp(p, 0, 0, C.byref(info), None, None, None)
    if rc:
        raise EGSError(rc, L.egsgpu_last_error(None).decode())
    n = info.n - first if count is None else count
    parts = np.zeros((max(n, 0), 7), dtype=np.float32)
    latch = np.zeros(max(n, 0), dtype=np.uint32)
    newh = np.zeros(max(n, 0), dtype=np.uint8)
    rc = L.egsgpu_read_phsp(p, first, n, C.byref(info), parts.ctypes.data_as(C.POINTER(C.c_float)),
                            latch.ctypes.data_as(C.POINTER(C.c_uint32)), newh.ctypes.data_as(C.POINTER(C.c_ubyte)))
    if rc:
        raise EGSError(rc, L.egsgpu_last_error(None).decode())
    out = dict(format=PHSP_FORMATS[info.format], n=info.n, photons=info.photons, incident=info.incident,
               ekmax=info.ekmax, zmin=info.zmin, zmax=info.zmax, has_latch=bool(info.has_latch), latch=latch,
               new_history=newh.astype(bool))
    return parts, out


def combine_checkpoints(a, b):
    """The checkpoint of the union of two shards' runs (egsgpu_combine_checkpoints);
    host only."""
    L = load_library()
    n = C.c_size_t(0)
    rc = L.egsgpu_combine_checkpoints(a, len(a), b, len(b), None, C.byref(n))
    if rc:
        raise EGSError(rc, "checkpoints of different phantoms or malformed")
    out = C.create_string_buffer(n.value)
    rc = L.egsgpu_combine_checkpoints(a, len(a), b, len(b), out, C.byref(n))
    if rc:
        raise EGSError(rc, "shards with different histories per batch")
    return out.raw


def checkpoint_arrays(blob):
    """Header, energy totals, counters and per-voxel sums of a checkpoint:
    dict(histories, batches, deposited, escaped, counters[8], sum, sum2)."""
    hdr = np.frombuffer(blob, dtype=np.int64, count=4)
    nv = int(hdr[1])
    en = np.frombuffer(blob, dtype=np.float64, count=2, offset=32)
    cnt = np.frombuffer(blob, dtype=np.uint64, count=8, offset=48)
    sums = np.frombuffer(blob, dtype=np.float64, count=2 * nv, offset=112)
    return dict(histories=int(hdr[2]), batches=int(hdr[3]), deposited=float(en[0]), escaped=float(en[1]),
                counters=cnt.copy(), sum=sums[:nv].copy(), sum2=sums[nv:].copy())


def default_config(**kw):
    """egsgpu_default_config with the named fields of egsgpu_config replaced;
    an unknown name raises TypeError (a ctypes structure would otherwise take
    it as a plain attribute and the engine would never see it)."""
    cfg = Config()
    load_library().egsgpu_default_config(C.byref(cfg))
    fields = {f[0] for f in Config._fields_}
    for k, v in kw.items():
        if k not in fields:
            raise TypeError("egsgpu_config has no field %r" % k)
        setattr(cfg, k, v)
    return cfg


class DoseEngine:
    """One engine handle (egsgpu_create) with its media, phantom, source and tallies."""

    def __init__(self, media, config=None, data_dir=DATA_DIR, pegs_file=PEGS_FILE, **kw):
        self.L = load_library()
        self.cfg = config if config is not None else default_config(**kw)
        h = C.c_void_p()
        self._check(self.L.egsgpu_create(C.byref(self.cfg), C.byref(h)), None)
        self.h = h
        names = (C.c_char_p * len(media))(*[m.encode() for m in media])
        self.media = list(media)
        self._check(self.L.egsgpu_load_media(self.h, data_dir.encode(), pegs_file.encode(), names, len(media)))
        self.geom = None

    def _check(self, rc, h=True):
        if rc:
            msg = self.L.egsgpu_last_error(self.h if h else None).decode() if h else "create failed"
            raise EGSError(rc, msg)

    def medium(self, index):
        o = np.zeros(4)
        self._check(self.L.egsgpu_get_medium(self.h, int(index), _dp(o)))
        return dict(rho=o[0], ae=o[1], ap=o[2], nelements=int(o[3]))

    def set_geometry(self, g):
        self.geom = g
        self._check(self.L.egsgpu_set_xyz_geometry(self.h, g.nx, g.ny, g.nz, _dp(g.xb), _dp(g.yb), _dp(g.zb),
                                                   g.med.ctypes.data_as(C.POINTER(C.c_int32)), _dp(g.rhor)))

    def set_source(self, src):
        self.src = src
        self._check(self.L.egsgpu_set_source(self.h, C.byref(src.s)))

    def run(self, n, nbatch=10, seed=1, first=0, stream=None):
        st = C.c_void_p(stream) if stream else None
        self._check(self.L.egsgpu_run(self.h, int(first), int(n), int(nbatch), int(seed), st))

    def run_noalloc(self, dose_ptr, n, seed=1, first=0, stream=None):
        """Transports histories [first, first+n) into the caller's device
        array of nvox doubles at address `dose_ptr` (overwritten with this
        call's energy per voxel, MeV) without allocating device memory; the
        handle's own tallies are untouched.  At most NOALLOC_MAX_HISTORIES
        histories per call; calls overlapping on the GPU race."""
        st = C.c_void_p(stream) if stream else None
        self._check(self.L.egsgpu_run_noalloc(self.h, int(first), int(n), int(seed), C.c_void_p(dose_ptr), st))

    def reset(self):
        self._check(self.L.egsgpu_reset(self.h))

    def adjoint(self, dL_dD, n, seed=1, first=0):
        """dL/d(rhor) per voxel for a loss of the dose of the run held in the
        tallies (histories [first, first+n) with `seed` since the last reset),
        given dL/dD per voxel (egsgpu_adjoint)."""
        g = np.ascontiguousarray(dL_dD, dtype=np.float64).ravel()
        out = np.zeros_like(g)
        self._check(self.L.egsgpu_adjoint(self.h, int(first), int(n), int(seed), _dp(g), _dp(out)))
        return out

    def set_phantoms(self, phantoms):
        """Several independent problems run together (egsgpu_set_phantoms):
        `phantoms` is a list of dicts with geometry (XYZGeometry), source
        (ParallelBeam), seed and histories (per egsgpu_run_phantoms call)."""
        arr = (PhantomStruct * len(phantoms))()
        for a, ph in zip(arr, phantoms):
            g = ph["geometry"]
            a.nx, a.ny, a.nz = g.nx, g.ny, g.nz
            a.xb, a.yb, a.zb = _dp(g.xb), _dp(g.yb), _dp(g.zb)
            a.med = g.med.ctypes.data_as(C.POINTER(C.c_int32))
            a.rhor = _dp(g.rhor)
            a.source = ph["source"].s
            a.seed = int(ph["seed"])
            a.histories = int(ph["histories"])
        self._check(self.L.egsgpu_set_phantoms(self.h, len(phantoms), arr))
        self.phantoms = [ph["geometry"] for ph in phantoms]
        self.geom = None
        self._nvox_all = sum(g.nvox for g in self.phantoms)

    def run_phantoms(self, nbatch=10, stream=None):
        st = C.c_void_p(stream) if stream else None
        self._check(self.L.egsgpu_run_phantoms(self.h, int(nbatch), st))

    def phantom_info(self, k):
        """(first global voxel index, voxels, histories run) of phantom k."""
        o = (C.c_longlong * 3)()
        self._check(self.L.egsgpu_get_phantom_info(self.h, int(k), o))
        return int(o[0]), int(o[1]), int(o[2])

    def phantom_dose(self, k):
        nv = self.phantoms[k].nvox
        d, s = np.zeros(nv), np.zeros(nv)
        self._check(self.L.egsgpu_get_phantom_dose(self.h, int(k), _dp(d), _dp(s)))
        return d, s

    def phantom_tallies(self, k):
        """Energy-deposit sum and sum of squares (MeV) of phantom k's voxels."""
        s, s2, _ = self.tallies()
        off, nv, _ = self.phantom_info(k)
        return s[off:off + nv], s2[off:off + nv]

    def tallies(self, out=None):
        """(sum, sum2, totals) of the energy per voxel over batches (MeV).
        `out`: an optional (sum, sum2) pair of contiguous float64 arrays of
        nvox elements to fill, so that a caller reading the tallies every step
        reuses its host memory, as a C caller of egsgpu_get_tallies does."""
        nv = self.geom.nvox if self.geom is not None else self._nvox_all
        if out is None:
            s, s2 = np.empty(nv), np.empty(nv)   # every element is written
        else:
            s, s2 = out
            for a in (s, s2):
                if a.dtype != np.float64 or a.size != nv or not a.flags.c_contiguous or not a.flags.writeable:
                    raise ValueError("tallies(out=...) wants two writable contiguous float64 arrays of %d elements" % nv)
        t = np.zeros(8)
        self._check(self.L.egsgpu_get_tallies(self.h, _dp(s), _dp(s2), _dp(t)))
        return s, s2, t

    def totals(self):
        t = np.zeros(8)
        self._check(self.L.egsgpu_get_tallies(self.h, None, None, _dp(t)))
        return dict(histories=t[0], batches=t[1], deposited=t[2], escaped=t[3], steps=t[4], photon_steps=t[5],
                    electron_steps=t[6], pushes=t[7])

    def dose(self):
        nv = self.geom.nvox
        d, s = np.zeros(nv), np.zeros(nv)
        self._check(self.L.egsgpu_get_dose(self.h, _dp(d), _dp(s)))
        return d, s

    def profile(self):
        o = np.zeros(20)
        self._check(self.L.egsgpu_get_profile(self.h, _dp(o)))
        keys = ("source", "photon", "electron", "batch")
        d = {"ms_" + k: o[i] for i, k in enumerate(keys)}
        d.update({"launches_" + k: int(o[4 + i]) for i, k in enumerate(keys)})
        d.update(photon_steps=o[8], electron_steps=o[9], photon_pushes=o[10], electron_pushes=o[11],
                 photon_interactions=o[12], electron_interactions=o[13], chunk=int(o[14]),
                 graph=int(o[15]), photon_busy_lanes=o[16], electron_busy_lanes=o[17], electron_wide_steps=o[18],
                 launch_shape=int(o[19]))
        return d

    def set_history_tally(self, first, n):
        self._hist_n = n
        self._check(self.L.egsgpu_set_history_tally(self.h, int(first), int(n)))

    def history_tally(self):
        out = np.zeros(self._hist_n)
        self._check(self.L.egsgpu_get_history_tally(self.h, _dp(out)))
        return out

    def geometry_query(self, op, ireg=None, x=None, u=None, t=None):
        """The kernels' geometry functions on the current phantom
        (egsgpu_geometry_query): op 0 isWhere of x, op 1 howfar from region
        ireg (howfarFromOut where ireg < 0) along u within t, op 2 hownear.
        Returns (new regions, distances)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        n = len(x)
        ireg = np.ascontiguousarray(ireg if ireg is not None else np.zeros(n), dtype=np.int32)
        u = np.ascontiguousarray(u if u is not None else np.zeros((n, 3)), dtype=np.float64)
        t = np.array(t if t is not None else np.zeros(n), dtype=np.float64)
        inew = np.zeros(n, dtype=np.int32)
        self._check(self.L.egsgpu_geometry_query(self.h, int(op), n, ireg.ctypes.data, x.ctypes.data, u.ctypes.data,
                                                 t.ctypes.data, inew.ctypes.data))
        return inew, t

    def checkpoint(self):
        size = C.c_size_t(0)
        self._check(self.L.egsgpu_checkpoint(self.h, None, C.byref(size)))
        buf = C.create_string_buffer(size.value)
        self._check(self.L.egsgpu_checkpoint(self.h, buf, C.byref(size)))
        return buf.raw

    def restore(self, blob):
        self._check(self.L.egsgpu_restore(self.h, blob, len(blob)))

    def close(self):
        if getattr(self, "h", None):
            self.L.egsgpu_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
