"""Phase-space readers and writers (CPU only).

Three readers must agree record for record: the library's egsgpu_read_phsp
(C ABI, used by egs_gpu_app), and formats.read_egsphsp / read_iaea_phsp
(numpy).  The IAEA format is checked against the reference's own IAEA library
(HEN_HOUSE/iaea_phsp, built from its sources into oracle/_ref by the oracle
Makefile): it reads the files formats.write_iaea_phsp writes, and the files it
writes are read back exactly.  Those two tests are skipped where the reference
sources are absent.
"""
import ctypes as C
import gzip
import os
import shutil

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import formats as F

HERE = os.path.dirname(os.path.abspath(__file__))
REF_IAEA = os.path.join(os.path.dirname(HERE), "oracle", "_ref", "libiaea_phsp.so")


def unpack(tmp_path, name):
    out = tmp_path / name
    with gzip.open(os.path.join(HERE, "golden", name + ".gz"), "rb") as a, open(out, "wb") as b:
        shutil.copyfileobj(a, b)
    return str(out)


@pytest.fixture(scope="module")
def ex16(tmp_path_factory):
    path = unpack(tmp_path_factory.mktemp("phsp"), "EX16MVp.egsphsp1")
    p, hdr = F.read_egsphsp(path)
    _, info = eg.read_phase_space(path)
    return path, p, hdr, info


@pytest.mark.parametrize("name", ["EX16MVp.egsphsp1", "EXslabs.egsphsp1"])
def test_egsphsp_library_reader_matches_numpy(tmp_path, name):
    path = unpack(tmp_path, name)
    p, hdr = F.read_egsphsp(path)
    q, info = eg.read_phase_space(path)
    assert np.array_equal(p, q)
    assert info["format"] == hdr["mode"] and info["n"] == hdr["n"] and info["photons"] == hdr["photons"]
    assert info["incident"] == hdr["incident"] and info["ekmax"] == pytest.approx(hdr["ekmax"])
    assert np.array_equal(info["new_history"], hdr["new_history"])
    # a chunk of records
    r, _ = eg.read_phase_space(path, first=100, count=37)
    assert np.array_equal(r, p[100:137])


def test_egsphsp_other_byte_order(tmp_path, ex16):
    """A file written on a machine of the other byte order reads the same."""
    path, p, hdr, info = ex16
    raw = open(path, "rb").read()
    rec = 32 if hdr["mode"] == "MODE2" else 28
    h = bytearray(raw[:rec])
    for off in (5, 9, 13, 17, 21):
        h[off:off + 4] = h[off:off + 4][::-1]
    body = np.frombuffer(raw[rec:], dtype="<u4").byteswap().tobytes()
    sw = tmp_path / "swapped.egsphsp1"
    sw.write_bytes(bytes(h) + body)
    q, qi = eg.read_phase_space(str(sw))
    assert np.array_equal(q, p) and np.array_equal(qi["latch"], info["latch"]) and qi["n"] == hdr["n"]


@pytest.mark.parametrize("order", ["little", "big"])
def test_iaea_round_trip(tmp_path, ex16, order):
    _, p, hdr, info = ex16
    base = str(tmp_path / "ex16")
    F.write_iaea_phsp(base, p, hdr["incident"], new_history=hdr["new_history"], z=50.0, latch=info["latch"],
                      byte_order=order)
    a, ha = F.read_iaea_phsp(base)
    b, hb = eg.read_phase_space(base + ".IAEAphsp")
    assert np.array_equal(a, p) and np.array_equal(b, p)
    assert hb["format"] == "IAEA" and hb["zmin"] == hb["zmax"] == 50.0 and ha["z"] == 50.0
    assert hb["incident"] == hdr["incident"] and hb["photons"] == hdr["photons"] and hb["has_latch"]
    assert np.array_equal(hb["latch"], info["latch"]) and np.array_equal(ha["latch"], info["latch"])
    assert np.array_equal(hb["new_history"], hdr["new_history"])
    assert np.array_equal(ha["new_history"], hdr["new_history"])
    assert hb["ekmax"] == pytest.approx(float(p[:, 1].max()), rel=1e-5)


def test_iaea_constants_stored_z_and_direction_edge(tmp_path):
    """Weight and Y constant, Z stored per particle, u^2 + v^2 > 1 (the reader
    rescales (u, v) to unit length), negative w."""
    p = np.array([[0, 1.0, 0.5, 2.0, 0.6, 0.0, 0.7],
                  [-1, 2.0, -0.5, 2.0, 0.8, 0.61, 0.7],
                  [1, 3.0, 1.5, 2.0, 0.1, 0.2, -0.7]], dtype=np.float32)
    z = np.array([1.0, 1.5, 2.0], dtype=np.float32)
    base = str(tmp_path / "edge")
    F.write_iaea_phsp(base, p, 10, z=z, constant=("Y", "Weight"))
    a, ha = F.read_iaea_phsp(base)
    b, hb = eg.read_phase_space(base)
    assert np.array_equal(a, b)
    assert np.array_equal(ha["z"], z) and hb["zmin"] == 1.0 and hb["zmax"] == 2.0
    s = np.sqrt(np.float32(0.8) ** 2 + np.float32(0.61) ** 2)
    assert b[1, 4] == np.float32(0.8) / s and b[1, 5] == np.float32(0.61) / s
    assert b[2, 6] == np.float32(-0.7) and b[0, 6] == np.float32(0.7)
    assert np.array_equal(b[[0, 2]][:, [0, 1, 2, 3, 4, 5]], p[[0, 2]][:, :6])
    _, h0 = eg.read_phase_space(base, count=0)
    assert np.isnan(h0["zmin"])


def test_phase_space_source_from_file(tmp_path, ex16):
    """PhaseSpaceSource.from_file: the same particles from either format, on the
    file's plane moved by the shift; particles on several planes refused."""
    path, p, hdr, _ = ex16
    base = str(tmp_path / "plane")
    F.write_iaea_phsp(base, p, hdr["incident"], z=0.25)
    a = eg.PhaseSpaceSource.from_file(path, shift=(1.0, 0.0, -0.5), recycle=2)
    b = eg.PhaseSpaceSource.from_file(base, shift=(1.0, 0.0, -0.75), recycle=2)
    assert np.array_equal(a._p, p) and np.array_equal(b._p, p)
    assert tuple(a.s.pos) == tuple(b.s.pos) == (1.0, 0.0, -0.5) and a.s.recycle == b.s.recycle == 2
    assert a.s.nphsp == b.s.nphsp == len(p) and a.info["format"] == "MODE2" and b.info["format"] == "IAEA"
    F.write_iaea_phsp(base, p[:3], 1, z=np.array([0.0, 1.0, 2.0], dtype=np.float32))
    with pytest.raises(ValueError):
        eg.PhaseSpaceSource.from_file(base)


def test_iaea_refusals(tmp_path, ex16):
    _, p, hdr, _ = ex16
    base = str(tmp_path / "bad")
    F.write_iaea_phsp(base, p[:10], 5)
    raw = bytearray(open(base + ".IAEAphsp", "rb").read())
    open(base + ".IAEAphsp", "wb").write(bytes(raw[:-1]))         # truncated
    with pytest.raises(eg.EGSError) as e:
        eg.read_phase_space(base)
    assert e.value.code == 2 and "size" in str(e.value)
    raw[0] = 4                                                     # a neutron
    open(base + ".IAEAphsp", "wb").write(bytes(raw))
    with pytest.raises(eg.EGSError) as e:
        eg.read_phase_space(base)
    assert e.value.code == 2 and "type 4" in str(e.value)
    with pytest.raises(eg.EGSError) as e:
        eg.read_phase_space(str(tmp_path / "missing"))
    assert e.value.code == 2
    with pytest.raises(ValueError):
        F.read_iaea_phsp(base)


# ---- against the reference's own IAEA library ----------------------------------

@pytest.fixture
def ref_lib():
    if not os.path.exists(REF_IAEA):
        pytest.skip("reference IAEA library not built (reference sources absent)")
    yield C.CDLL(REF_IAEA)
    C.CDLL(None).fflush(None)     # the library reports on stdout: flush it while pytest captures it


i32, f32, i64 = C.c_int32, C.c_float, C.c_longlong


def test_reference_library_reads_our_files(tmp_path, ex16, ref_lib):
    L = ref_lib
    _, p, hdr, info = ex16
    base = str(tmp_path / "ours")
    F.write_iaea_phsp(base, p, hdr["incident"], new_history=hdr["new_history"], z=50.0, latch=info["latch"])
    sid, res = i32(0), i32(0)
    b = base.encode()
    L.iaea_new_source(C.byref(sid), C.c_char_p(b), C.byref(i32(1)), C.byref(res), len(b))
    assert res.value >= 0
    n = i64(0)
    L.iaea_get_max_particles(C.byref(sid), C.byref(i32(-1)), C.byref(n))
    assert n.value == len(p)
    pinc = i64(0)
    L.iaea_get_total_original_particles(C.byref(sid), C.byref(pinc))
    assert pinc.value == hdr["incident"]
    ef, ei = (f32 * 10)(), (i32 * 10)()
    rows = []
    for _ in range(len(p)):
        st, ty = i32(), i32()
        v = [f32() for _ in range(8)]
        L.iaea_get_particle(C.byref(sid), C.byref(st), C.byref(ty), *[C.byref(x) for x in v], ef, ei)
        rows.append([st.value, ty.value] + [x.value for x in v] + [ei[0] & 0xffffffff])
    L.iaea_destroy_source(C.byref(sid), C.byref(res))
    r = np.array(rows, dtype=np.float64)
    q = np.where(r[:, 1] == 1, 0, np.where(r[:, 1] == 2, -1, 1))
    assert np.array_equal(q, p[:, 0])
    for col, k in ((2, 1), (4, 2), (5, 3), (7, 4), (8, 5)):    # E, x, y, u, v
        assert np.array_equal(r[:, col].astype(np.float32), p[:, k])
    assert np.array_equal(r[:, 3].astype(np.float32), np.abs(p[:, 6]))
    assert np.array_equal(r[:, 9] < 0, p[:, 6] < 0) and np.all(r[:, 6] == 50.0)
    assert np.array_equal(r[:, 0] > 0, hdr["new_history"])
    assert np.array_equal(r[:, 10].astype(np.uint32), info["latch"])


def test_our_readers_read_reference_files(tmp_path, ref_lib):
    """The reference library writes 400 particles with a constant Z, a ZLAST
    extra float, the incremental history number and the LATCH as extra longs."""
    L = ref_lib
    rng = np.random.default_rng(3)
    n, zc = 400, 12.5
    ty = rng.integers(1, 4, n)
    e = rng.uniform(0.01, 20, n).astype(np.float32)
    wt = rng.uniform(0.1, 2, n).astype(np.float32)
    x, y = rng.uniform(-5, 5, (2, n)).astype(np.float32)
    u, v = rng.uniform(-0.6, 0.6, (2, n)).astype(np.float32)
    w = (np.sqrt(1 - u.astype(np.float64) ** 2 - v.astype(np.float64) ** 2) *
         np.where(rng.random(n) < 0.8, 1, -1)).astype(np.float32)
    nstat = rng.integers(0, 3, n)
    latch = rng.integers(0, 2 ** 31, n)
    base = str(tmp_path / "refmade")
    sid, res = i32(0), i32(0)
    b = base.encode()
    R = C.byref
    L.iaea_new_source(R(sid), C.c_char_p(b), R(i32(2)), R(res), len(b))
    assert res.value >= 0
    L.iaea_set_constant_variable(R(sid), R(i32(2)), R(f32(zc)))
    L.iaea_set_extra_numbers(R(sid), R(i32(1)), R(i32(2)))
    L.iaea_set_type_extrafloat_variable(R(sid), R(i32(0)), R(i32(3)))
    L.iaea_set_type_extralong_variable(R(sid), R(i32(0)), R(i32(1)))
    L.iaea_set_type_extralong_variable(R(sid), R(i32(1)), R(i32(2)))
    L.iaea_set_total_original_particles(R(sid), R(i64(777)))
    for k in range(n):
        ef, ei = (f32 * 1)(7.0), (i32 * 2)(int(nstat[k]), int(latch[k]))
        vals = [f32(float(t)) for t in (e[k], wt[k], x[k], y[k], zc, u[k], v[k], w[k])]
        L.iaea_write_particle(R(sid), R(i32(int(nstat[k]))), R(i32(int(ty[k]))), *[R(t) for t in vals], ef, ei)
    L.iaea_destroy_source(R(sid), R(res))
    want = np.stack([np.where(ty == 1, 0, np.where(ty == 2, -1, 1)), e, x, y, u, v, np.where(w < 0, -wt, wt)],
                    axis=1).astype(np.float32)
    a, ha = F.read_iaea_phsp(base)
    got, hb = eg.read_phase_space(base)
    assert np.array_equal(a, want) and np.array_equal(got, want)
    assert hb["zmin"] == hb["zmax"] == zc and ha["z"] == zc and hb["incident"] == 777 and hb["n"] == n
    assert np.array_equal(hb["new_history"], nstat > 0) and np.array_equal(ha["new_history"], nstat > 0)
    assert np.array_equal(hb["latch"], latch.astype(np.uint32)) and np.array_equal(ha["latch"], hb["latch"])
