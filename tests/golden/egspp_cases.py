"""Seeded geometry query sets for the bitwise check of the XYZ geometry against
the reference's own EGS_XYZGeometry (egs++/geometry/egs_nd_geometry/
egs_nd_geometry.h:769-1379), and the source cases for its EGS_ParallelBeam.

The inputs are built from the generator's uniform doubles with +, *, / and
sqrt only (correctly rounded on every IEEE machine) and exact powers of two,
so that the x86 machine that ran the reference and the Arm machine with the
GPU build the same bytes; `digest` of the inputs is stored beside the
outputs' to show it.

Used by make_egspp_fixtures.py (which runs the reference and writes
egspp_reference.json) and by the tests.
"""
import hashlib

import numpy as np

N_QUERIES = 100000


def geometries():
    """Plane sets: the water30 and slab64 phantoms' planes and a ragged one."""
    g = {}
    b = -15.0 + np.arange(31, dtype=np.float64)
    g["water30"] = (b, b.copy(), np.arange(31, dtype=np.float64))
    b = -8.0 + 0.25 * np.arange(65, dtype=np.float64)
    g["slab64"] = (b, b.copy(), 0.25 * np.arange(65, dtype=np.float64))
    rng = np.random.default_rng(4242)
    planes = []
    for n, x0 in ((17, -3.1), (13, -1.7), (11, 0.4)):
        w = 0.05 + 1.95 * rng.random(n)
        planes.append(x0 + np.concatenate([[0.0], np.cumsum(w)]))
    g["ragged"] = tuple(planes)
    return g


def _directions(rng, n):
    """Unit vectors, isotropic by rejection from the cube; a fifth have one
    component exactly zero and a twentieth lie along an axis."""
    out = np.empty((n, 3))
    k = 0
    while k < n:
        v = rng.random((2 * (n - k) + 16, 3)) * 2.0 - 1.0
        r2 = v[:, 0] * v[:, 0] + v[:, 1] * v[:, 1] + v[:, 2] * v[:, 2]
        v = v[(r2 > 0.01) & (r2 <= 1.0)][: n - k]
        out[k:k + len(v)] = v
        k += len(v)
    kind = rng.integers(0, 20, n)
    zero = rng.integers(0, 3, n)
    m = kind < 4
    out[m, zero[m]] = 0.0
    m = kind == 19
    out[m] = 0.0
    out[m, zero[m]] = np.where(rng.random(m.sum()) < 0.5, -1.0, 1.0)
    norm = np.sqrt(out[:, 0] * out[:, 0] + out[:, 1] * out[:, 1] + out[:, 2] * out[:, 2])
    return out / norm[:, None]


def _steps(rng, n):
    """Step lengths: m * 2^e with m in [1, 2) and e in [-40, 6], or veryFar."""
    t = np.ldexp(1.0 + rng.random(n), rng.integers(-40, 7, n))
    t[rng.random(n) < 0.1] = 1e30
    return t


def _inside(rng, planes, n):
    """Voxels and points inside them; each coordinate lies on one of its
    voxel's faces with probability 0.15."""
    nx, ny, nz = (len(p) - 1 for p in planes)
    idx = [rng.integers(0, m, n) for m in (nx, ny, nz)]
    x = np.empty((n, 3))
    for a in range(3):
        lo, hi = planes[a][idx[a]], planes[a][idx[a] + 1]
        x[:, a] = lo + (hi - lo) * rng.random(n)
        snap = rng.random(n)
        x[snap < 0.075, a] = lo[snap < 0.075]
        m = (snap >= 0.075) & (snap < 0.15)
        x[m, a] = hi[m]
    ireg = (idx[0] + idx[1] * nx + idx[2] * nx * ny).astype(np.int32)
    return ireg, x


def _anywhere(rng, planes, n):
    """Points around the phantom, half of their coordinates on a plane."""
    x = np.empty((n, 3))
    for a in range(3):
        p = planes[a]
        L = p[-1] - p[0]
        x[:, a] = p[0] - 0.1 * L + 1.2 * L * rng.random(n)
        on = rng.random(n) < 0.5
        x[on, a] = p[rng.integers(0, len(p), on.sum())]
    return x


def _outside(rng, planes, n):
    """Points outside the phantom beyond one face (or on it), with
    directions of which most point inwards."""
    x = _anywhere(rng, planes, n)
    u = _directions(rng, n)
    a = rng.integers(0, 3, n)
    side = rng.random(n) < 0.5
    gap = np.ldexp(1.0 + rng.random(n), rng.integers(-40, 4, n))
    gap[rng.random(n) < 0.05] = 0.0
    for k in range(3):
        m = a == k
        lo, hi = planes[k][0], planes[k][-1]
        x[m & side, k] = lo - gap[m & side]
        x[m & ~side, k] = hi + gap[m & ~side]
        inward = rng.random(n) < 0.8
        mm = m & side & inward
        u[mm, k] = np.abs(u[mm, k])
        mm = m & ~side & inward
        u[mm, k] = -np.abs(u[mm, k])
    return x, u


def queries(name, planes, n=N_QUERIES):
    """The query set of one geometry: where[x], howfar inside (ireg, x, u, t),
    howfar from outside (x, u, t) and hownear (ireg, x)."""
    seed = {"water30": 1, "slab64": 2, "ragged": 3}[name]
    rng = np.random.default_rng(9000 + seed)
    q = {}
    q["where_x"] = _anywhere(rng, planes, n)
    q["in_ireg"], q["in_x"] = _inside(rng, planes, n)
    q["in_u"] = _directions(rng, n)
    q["in_t"] = _steps(rng, n)
    q["out_x"], q["out_u"] = _outside(rng, planes, n)
    q["out_t"] = _steps(rng, n)
    q["near_ireg"], q["near_x"] = _inside(rng, planes, n)
    return q


def digest(*arrays):
    """SHA-256 of the arrays' little-endian bytes, in order."""
    h = hashlib.sha256()
    for a in arrays:
        a = np.ascontiguousarray(a)
        h.update(a.astype(a.dtype.newbyteorder("<"), copy=False).tobytes())
    return h.hexdigest()


def input_digest(q):
    return digest(*(q[k] for k in sorted(q)))


# Source cases for EGS_ParallelBeam: the slab64 photon field and the
# water128e electron field (both from z = -1 cm into the phantom).
SOURCE_SAMPLES = 1000000
E_BINS = 120
XY_BINS = 40
