"""On-disk formats either side of the transport path.

* ``.egsphant`` voxel phantoms (DOSXYZnrc / egs++ ``egsphant file`` input,
  egs++/geometry/egs_nd_geometry/egs_nd_geometry.cpp:600-700): medium names,
  voxel boundaries, one medium character per voxel and the mass density per
  voxel.  Relative densities follow the egs++ rule rho_rel = rho / rho_PEGS4.
* ``.3ddose`` dose files (egs++/ausgab_objects/egs_dose_scoring/egs_dose_scoring.cpp:416-480,
  user_codes/dosxyznrc/dosxyznrc.mortran write_dose): voxel counts, boundaries,
  dose per voxel (x fastest) and relative uncertainties.
* ``.egsphsp`` phase-space files (BEAMnrc output, the input of egs++
  EGS_PhspSource and DOSXYZnrc isource 2; egs++/sources/egs_phsp_source/
  egs_phsp_source.cpp:64-130 header, :360-423 records): a header record
  "MODE0"/"MODE2", particle and photon counts, maximum kinetic energy,
  minimum electron kinetic energy and incident-history count, then one
  record per particle: LATCH (bit 30 electron, bit 29 positron), E (total
  energy for charged particles; negative for the first particle of a new
  incident history), X, Y, U, V, WT (negative when W < 0) and, in MODE2, ZLAST.
"""
import numpy as np

from . import XYZGeometry

MEDIUM_CHARS = "123456789ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz"


def read_egsphant(path, pegs_density=None):
    """Returns (media names, XYZGeometry with medium indices and relative
    densities, mass densities).  `pegs_density` maps medium name -> PEGS4
    density; without it relative densities are returned as the mass densities."""
    with open(path) as f:
        lines = [l.rstrip("\n") for l in f]
    pos = 0

    def nxt():
        nonlocal pos
        while not lines[pos].strip():
            pos += 1
        pos += 1
        return lines[pos - 1]

    nmed = int(nxt().split()[0])
    names = [nxt().strip() for _ in range(nmed)]
    nxt()   # ESTEPE values (unused)
    nx, ny, nz = (int(v) for v in nxt().split()[:3])

    def floats(n):
        out = []
        while len(out) < n:
            out.extend(float(v) for v in nxt().split())
        return np.array(out[:n])

    xb, yb, zb = floats(nx + 1), floats(ny + 1), floats(nz + 1)
    med = np.empty((nz, ny, nx), dtype=np.int32)
    for k in range(nz):
        for j in range(ny):
            row = nxt().strip()
            if len(row) < nx:
                raise ValueError("short medium row in %s" % path)
            med[k, j] = [MEDIUM_CHARS.index(c) for c in row[:nx]]
    rho = np.empty((nz, ny, nx))
    for k in range(nz):
        for j in range(ny):
            rho[k, j] = floats(nx)
    if np.any(med >= nmed) or np.any(med < 0):
        raise ValueError("medium index outside the medium list in %s" % path)
    rel = rho.copy()
    if pegs_density is not None:
        dens = np.array([pegs_density[n] for n in names])
        rel = rho / dens[med]
    return names, XYZGeometry(xb, yb, zb, med.ravel(), rel.ravel()), rho.ravel()


def write_egsphant(path, names, geom, rho, estepe=0.25):
    nx, ny, nz = geom.nx, geom.ny, geom.nz
    med = geom.med.reshape(nz, ny, nx)
    rho = np.asarray(rho).reshape(nz, ny, nx)
    with open(path, "w") as f:
        f.write("%d\n" % len(names))
        for n in names:
            f.write(n + "\n")
        f.write("\t".join("%g" % estepe for _ in names) + "\n")
        f.write("%d\t%d\t%d\n" % (nx, ny, nz))
        for b in (geom.xb, geom.yb, geom.zb):
            f.write("\t".join("%.10g" % v for v in b) + "\n")
        for k in range(nz):
            for j in range(ny):
                f.write("".join(MEDIUM_CHARS[m] for m in med[k, j]) + "\n")
            f.write("\n")
        for k in range(nz):
            for j in range(ny):
                f.write("\t".join("%.8g" % v for v in rho[k, j]) + "\n")
            f.write("\n")


def write_3ddose(path, geom, dose, sigma):
    """Dose (Gy per particle) and absolute 1-sigma; the file stores relative
    uncertainties (1 where the dose is zero), single-precision values."""
    dose = np.asarray(dose, dtype=np.float64)
    rel = np.where(dose > 0, np.asarray(sigma) / np.where(dose > 0, dose, 1.0), 1.0)
    with open(path, "w") as f:
        f.write("%d %d %d\n" % (geom.nx, geom.ny, geom.nz))
        for b in (geom.xb, geom.yb, geom.zb):
            f.write(" ".join("%g" % np.float32(v) for v in b) + " \n")
        f.write(" ".join("%g" % np.float32(v) for v in dose) + " \n")
        f.write(" ".join("%g" % np.float32(v) for v in rel) + " \n")


def read_3ddose(path):
    """Returns (nx, ny, nz), (xb, yb, zb), dose, relative uncertainty."""
    toks = open(path).read().split()
    nx, ny, nz = (int(v) for v in toks[:3])
    p = 3
    v = np.array(toks[p:], dtype=np.float64)
    xb = v[:nx + 1]; yb = v[nx + 1:nx + ny + 2]; zb = v[nx + ny + 2:nx + ny + nz + 3]
    p = nx + ny + nz + 3
    n = nx * ny * nz
    return (nx, ny, nz), (xb, yb, zb), v[p:p + n], v[p + n:p + 2 * n]


PHSP_E_BIT = 1 << 30    # LATCH bit: electron
PHSP_P_BIT = 1 << 29    # LATCH bit: positron


def read_egsphsp(path, rm=0.5109989461):
    """Returns (particles, header): particles an (n, 7) float32 array of
    {charge, kinetic energy, x, y, u, v, weight} as PhaseSpaceSource takes
    them, header a dict with mode, n, photons, ekmax, ekmin_e, incident and
    new_history (bool array: the particle starts a new incident history)."""
    if str(path).endswith(".gz"):
        import gzip
        with gzip.open(path, "rb") as f:
            raw = f.read()
    else:
        with open(path, "rb") as f:
            raw = f.read()
    mode = raw[:5].decode("ascii")
    if mode not in ("MODE0", "MODE2"):
        raise ValueError("%s: not an egsphsp file" % path)
    rec = 28 if mode == "MODE0" else 32
    n, nphot = np.frombuffer(raw[5:13], dtype="<i4")
    ekmax, ekmin, ninc = np.frombuffer(raw[13:25], dtype="<f4")
    fields = [("latch", "<u4"), ("e", "<f4"), ("x", "<f4"), ("y", "<f4"), ("u", "<f4"), ("v", "<f4"), ("wt", "<f4")]
    if rec == 32:
        fields.append(("zlast", "<f4"))
    r = np.frombuffer(raw[rec:rec + int(n) * rec], dtype=np.dtype(fields))
    if len(r) != n:
        raise ValueError("%s: %d records, header says %d" % (path, len(r), n))
    q = np.where(r["latch"] & PHSP_E_BIT, -1, np.where(r["latch"] & PHSP_P_BIT, 1, 0)).astype(np.float32)
    e = np.abs(r["e"]).astype(np.float64)
    ek = np.where(q != 0, e - rm, e)
    out = np.stack([q, ek.astype(np.float32), r["x"], r["y"], r["u"], r["v"], r["wt"]], axis=1).astype(np.float32)
    hdr = dict(mode=mode, n=int(n), photons=int(nphot), ekmax=float(ekmax), ekmin_e=float(ekmin),
               incident=float(ninc), new_history=r["e"] < 0)
    return out, hdr


def write_egsphsp(path, particles, incident, new_history=None, mode="MODE0", rm=0.5109989461):
    """Writes particles ({charge, kinetic energy, x, y, u, v, weight} rows)
    as an egsphsp file of the given mode (ZLAST = 0 in MODE2)."""
    p = np.asarray(particles, dtype=np.float64).reshape(-1, 7)
    n = len(p)
    rec = 28 if mode == "MODE0" else 32
    latch = np.where(p[:, 0] < 0, PHSP_E_BIT, np.where(p[:, 0] > 0, PHSP_P_BIT, 0)).astype("<u4")
    e = np.where(p[:, 0] != 0, p[:, 1] + rm, p[:, 1])
    if new_history is not None:
        e = np.where(new_history, -e, e)
    fields = [("latch", "<u4"), ("e", "<f4"), ("x", "<f4"), ("y", "<f4"), ("u", "<f4"), ("v", "<f4"), ("wt", "<f4")]
    if rec == 32:
        fields.append(("zlast", "<f4"))
    r = np.zeros(n, dtype=np.dtype(fields))
    r["latch"], r["e"], r["x"], r["y"], r["u"], r["v"], r["wt"] = latch, e, p[:, 2], p[:, 3], p[:, 4], p[:, 5], p[:, 6]
    charged = p[:, 0] != 0
    hdr = bytearray(rec)
    hdr[:5] = mode.encode()
    hdr[5:13] = np.array([n, int((~charged).sum())], dtype="<i4").tobytes()
    ekmin = float(p[charged, 1].min()) if charged.any() else 0.0
    hdr[13:25] = np.array([p[:, 1].max(), ekmin, incident], dtype="<f4").tobytes()
    with open(path, "wb") as f:
        f.write(bytes(hdr))
        f.write(r.tobytes())
