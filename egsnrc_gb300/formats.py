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
* IAEA phase-space files (the input of egs++ IAEA_PhspSource,
  egs++/sources/iaea_phsp_source/iaea_phsp_source.cpp:77-224, :310-417; format
  HEN_HOUSE/iaea_phsp/iaea_header.cpp:60-330 and :700-800, iaea_record.cpp:85-230):
  a text header <name>.IAEAheader of "$KEYWORD:" blocks and binary records in
  <name>.IAEAphsp.  A record holds the particle type as a signed byte (1
  photon, 2 e-, 3 e+; negative when W < 0), the kinetic energy (negative for a
  new history), the stored ones of X Y Z U V WEIGHT (RECORD_CONTENTS; the rest
  are RECORD_CONSTANT values), extra floats and extra int32s (type 1 the
  incremental history number, type 2 the EGS LATCH).
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


IAEA_KEYS = ("X", "Y", "Z", "U", "V", "W", "Weight")


def _iaea_blocks(text):
    """The "$KEY:" blocks of an IAEA header, comments removed, blank lines skipped."""
    import re
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    text = re.sub(r"//[^\n]*", "", text)
    blocks, cur = {}, None
    for line in text.splitlines():
        line = line.strip()
        if not line:
            continue
        if line.startswith("$") and ":" in line:
            cur = blocks.setdefault(line[1:line.index(":")], [])
            continue
        if cur is not None:
            cur.append(line)
    return blocks


def _iaea_base(path):
    p = str(path)
    for ext in (".IAEAheader", ".IAEAphsp"):
        if p.endswith(ext):
            return p[:-len(ext)]
    return p


def read_iaea_phsp(path):
    """Returns (particles, header) like read_egsphsp for an IAEA phase-space
    pair (path = <name>, with or without either extension); header has mode
    "IAEA", n, photons, incident, z (the constant Z, or the array of stored
    Z), latch (zeros if none is stored) and new_history."""
    base = _iaea_base(path)
    with open(base + ".IAEAheader") as f:
        B = _iaea_blocks(f.read())
    contents = [int(float(v.split()[0])) for v in B["RECORD_CONTENTS"]]
    nxf, nxl = contents[7], contents[8]
    ftypes = contents[9:9 + nxf]
    ltypes = contents[9 + nxf:9 + nxf + nxl]
    const = {}
    vals = iter(B.get("RECORD_CONSTANT", []))
    for i, k in enumerate(IAEA_KEYS):
        if contents[i] <= 0:
            const[k] = float(next(vals).split()[0])
    order = int(B["BYTE_ORDER"][0].split()[0])
    end = "<" if order == 1234 else ">"
    fields = [("type", "i1"), ("e", end + "f4")]
    fields += [(k, end + "f4") for i, k in enumerate(IAEA_KEYS) if i != 5 and contents[i] > 0]
    fields += [("xf%d" % j, end + "f4") for j in range(nxf)]
    fields += [("xl%d" % j, end + "i4") for j in range(nxl)]
    dt = np.dtype(fields)
    n = int(float(B["PARTICLES"][0].split()[0]))
    raw = np.fromfile(base + ".IAEAphsp", dtype=np.uint8)
    if raw.size != n * dt.itemsize or int(float(B["CHECKSUM"][0].split()[0])) != raw.size:
        raise ValueError("%s: file size does not match the header" % base)
    r = np.frombuffer(raw.tobytes(), dtype=dt)
    t = r["type"].astype(np.int32)
    wneg = t < 0
    t = np.abs(t)
    if np.any((t < 1) | (t > 3)):
        raise ValueError("%s: records other than photons, electrons and positrons" % base)
    col = {k: (r[k].astype(np.float32) if k in r.dtype.names else np.full(n, const[k], dtype=np.float32))
           for i, k in enumerate(IAEA_KEYS) if i != 5}
    u, v = col["U"].copy(), col["V"].copy()
    if contents[5] > 0:
        aux = u * u + v * v                       # float32, as the record reader forms it
        big = aux.astype(np.float64) > 1.0
        s = np.sqrt(aux[big])
        u[big] /= s
        v[big] /= s
        w = np.where(big, np.float32(0), np.sqrt((1.0 - aux.astype(np.float64)).clip(0).astype(np.float32)))
        w = np.where(wneg, -w, w)
    else:
        w = np.full(n, const["W"], dtype=np.float32)
    q = np.where(t == 1, 0, np.where(t == 2, -1, 1)).astype(np.float32)
    wt = np.abs(col["Weight"])
    wt = np.where((w < 0) | ((w == 0) & wneg), -wt, wt)
    parts = np.stack([q, np.abs(r["e"]).astype(np.float32), col["X"], col["Y"], u, v, wt], axis=1).astype(np.float32)
    newh = r["e"] < 0
    latch = np.zeros(n, dtype=np.uint32)
    for j, lt in enumerate(ltypes):
        if lt == 1:
            newh = r["xl%d" % j] > 0
        if lt == 2:
            latch = r["xl%d" % j].astype(np.uint32)
    hdr = dict(mode="IAEA", n=n, photons=int(float(B["PHOTONS"][0].split()[0])) if "PHOTONS" in B else 0,
               incident=float(B["ORIG_HISTORIES"][0].split()[0]) if "ORIG_HISTORIES" in B else 0.0,
               z=col["Z"] if contents[2] > 0 else const["Z"], latch=latch, new_history=newh,
               extra_float_types=ftypes, extra_long_types=ltypes)
    return parts, hdr


def write_iaea_phsp(path, particles, incident, new_history=None, z=0.0, latch=None, constant=(),
                    byte_order="little", pcut=0.0, ecut=0.0, code="egsnrc_gb300"):
    """Writes particles ({charge, kinetic energy, x, y, u, v, weight} rows, a
    negative weight meaning w < 0) as an IAEA phase-space pair <path>.IAEAheader
    and <path>.IAEAphsp.  z is the plane (a constant) or an array stored per
    particle; quantities named in `constant` (of X, Y, U, V, Weight) are
    written once in RECORD_CONSTANT from the first particle; latch, when given,
    is stored as an EGS LATCH extra int32.  pcut and ecut (kinetic, MeV) are
    the header's global photon and particle energy cutoffs."""
    base = _iaea_base(path)
    p = np.asarray(particles, dtype=np.float32).reshape(-1, 7)
    n = len(p)
    wneg = p[:, 6] < 0
    z_arr = np.ndim(z) > 0
    cols = {"X": p[:, 2], "Y": p[:, 3], "Z": np.asarray(z, dtype=np.float32) if z_arr else None,
            "U": p[:, 4], "V": p[:, 5], "Weight": np.abs(p[:, 6])}
    stored = {k: (k == "Z" and z_arr) or (k != "Z" and k not in constant) for k in cols}
    contents = [int(stored["X"]), int(stored["Y"]), int(stored["Z"]), int(stored["U"]), int(stored["V"]), 1,
                int(stored["Weight"]), 0, 1 if latch is not None else 0]
    end = "<" if byte_order == "little" else ">"
    fields = [("type", "i1"), ("e", end + "f4")] + [(k, end + "f4") for k in ("X", "Y", "Z", "U", "V", "Weight")
                                                     if stored[k]]
    if latch is not None:
        fields.append(("xl0", end + "i4"))
    r = np.zeros(n, dtype=np.dtype(fields))
    t = np.where(p[:, 0] == 0, 1, np.where(p[:, 0] < 0, 2, 3)).astype(np.int8)
    r["type"] = np.where(wneg, -t, t)
    e = p[:, 1]
    r["e"] = np.where(new_history, -e, e) if new_history is not None else e
    for k in ("X", "Y", "Z", "U", "V", "Weight"):
        if stored[k]:
            r[k] = cols[k]
    if latch is not None:
        r["xl0"] = np.asarray(latch).astype(np.uint32).view(np.int32)
    with open(base + ".IAEAphsp", "wb") as f:
        f.write(r.tobytes())
    kinds = [(1, "PHOTONS"), (2, "ELECTRONS"), (3, "POSITRONS")]
    L = ["$IAEA_INDEX:", "0", "", "$TITLE:", "phase space", "", "$FILE_TYPE:", "0", "",
         "$CHECKSUM:", "%d" % (n * r.dtype.itemsize), "", "$RECORD_CONTENTS:"]
    L += ["   %d     // %s is stored ?" % (c, k) for c, k in zip(contents[:7], IAEA_KEYS)]
    L += ["   %d     // Extra floats stored ?" % contents[7], "   %d     // Extra longs stored ?" % contents[8]]
    if latch is not None:
        L.append("   2     // LATCH EGS variable stored in the extralong array [ 0]")
    L += ["", "$RECORD_CONSTANT:"]
    for k in IAEA_KEYS:
        if k == "Z" and not z_arr:
            L.append("   %.9g     // Constant Z" % float(z))
        elif k in constant:
            L.append("   %.9g     // Constant %s" % (float(cols[k][0]), k))
    L += ["", "$RECORD_LENGTH:", "%d" % r.dtype.itemsize, "", "$BYTE_ORDER:",
          "1234" if byte_order == "little" else "4321", "",
          "$ORIG_HISTORIES:", "%d" % int(incident), "", "$PARTICLES:", "%d" % n, ""]
    for kind, name in kinds:
        m = int((t == kind).sum())
        if m:
            L += ["$%s:" % name, "%d" % m, ""]
    # every mandatory block carries a line: the reference reader refuses an empty one
    L += ["$TRANSPORT_PARAMETERS:", "-", "", "$MACHINE_TYPE:", "-", "", "$MONTE_CARLO_CODE_VERSION:", code, "",
          "$GLOBAL_PHOTON_ENERGY_CUTOFF:", " %.5f" % pcut, "", "$GLOBAL_PARTICLE_ENERGY_CUTOFF:", " %.5f" % ecut, "",
          "$COORDINATE_SYSTEM_DESCRIPTION:", "-", "", "$STATISTICAL_INFORMATION_PARTICLES:",
          "//        Weight        Wmin       Wmax       <E>         Emin         Emax    Particle"]
    for kind, name in kinds:
        m = t == kind
        if m.any():
            w_, e_ = np.abs(p[m, 6]).astype(np.float64), p[m, 1].astype(np.float64)
            L.append("  %.6g  %.6g  %.6g  %.6g  %.6g  %.6g  %s" % (w_.sum(), w_.min(), w_.max(),
                                                                  (w_ * e_).sum() / w_.sum(), e_.min(), e_.max(),
                                                                  name))
    L += ["", "$STATISTICAL_INFORMATION_GEOMETRY:"]
    for k in ("X", "Y", "Z"):
        if stored[k]:
            L.append(" %.6g  %.6g" % (float(np.min(cols[k])), float(np.max(cols[k]))))
    with open(base + ".IAEAheader", "w") as f:
        f.write("\n".join(L) + "\n")
