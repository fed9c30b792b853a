"""Known-answer tests of the oracle's random-number generators.

RANMAR: the partial sums that EGSnrc's own RANMAR test prints next to the
computed ones (HEN_HOUSE/user_codes/ranmar_test/ranmar_test.mortran, default
seeds ixx = jxx = 0 -> 1802, 9373).  This is the only golden vector the
reference ships for this path.

Philox-4x32-10: the published known-answer vectors of Salmon et al. (SC'11,
Random123 kat_vectors), which the GPU engine's generator is checked against
history by history through the oracle.
"""
import numpy as np
import pytest

from oracle.oracle_binding import lib, philox, ranmar


def test_ranmar_reference_partial_sums():
    r = ranmar(1_000_000)
    assert r.min() >= 0.0 and r.max() < 1.0
    assert abs(r[:10].sum() - 5.88279718) < 5e-9
    assert abs(r[:10_000].sum() - 5034.47920114) < 5e-9
    assert abs(r[:100_000].sum() - 50053.28831381) < 5e-9
    assert abs(r.sum() - 500163.88955361) < 5e-9


@pytest.mark.parametrize("ctr,key,out", [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
])
def test_philox_known_answers(ctr, key, out):
    assert philox(ctr, key) == out


def test_child_streams_are_distinct():
    L = lib()
    seen = set()
    for sid in (0, 1, 12345678901234):
        for n in range(64):
            for k in range(3):
                seen.add(L.oracle_child_sid(sid, n, k))
    assert len(seen) == 3 * 64 * 3


def test_oracle_phase_space_source_conserves_energy():
    # every phase-space particle enters the phantom (field inside its face):
    # deposited + escaped = sum of weight x (kinetic energy, + 2 m c^2 for e+)
    import egsnrc_gb300 as eg
    from egsnrc_gb300 import workloads as W
    from oracle.oracle_binding import Oracle
    rng = np.random.default_rng(8)
    k = 64
    p = np.stack([rng.choice([-1, 0, 1], k, p=[0.3, 0.6, 0.1]), rng.uniform(0.2, 4.0, k), rng.uniform(-2, 2, k),
                  rng.uniform(-2, 2, k), rng.uniform(-0.2, 0.2, k), rng.uniform(-0.2, 0.2, k),
                  rng.uniform(0.5, 1.5, k)], 1).astype(np.float32)
    src = eg.PhaseSpaceSource(p, position=(0.0, 0.0, 0.0), recycle=1)
    ora = Oracle([W.WATER], ecut=0.7, pcut=0.01)
    ora.set_geometry(W.centred_geometry(12, 1.0))
    ora.set_source(src)
    n = 2 * k * 3
    ora.run(n, nbatch=2, seed=4)
    _, _, t = ora.tallies()    # totals: histories, batches, deposited, escaped, ...
    e = 0.0
    for h in range(n):
        q = p[(h // 2) % k]
        e += abs(float(q[6])) / 2 * (float(q[1]) + (2 * eg.RM if q[0] > 0 else 0.0))
    assert abs(t[2] + t[3] - e) < 1e-9 * e
