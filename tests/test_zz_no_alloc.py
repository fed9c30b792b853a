"""The no-allocation entry point (egsgpu_run_noalloc) against egsgpu_run.

egsgpu_run_noalloc transports a small chunk of histories with its particle
queues in a fixed static device array, for callers that may not allocate
device memory while they run.  Every history owns its random-number streams,
so it must deposit the same energy per voxel as egsgpu_run does for the same
histories, up to the order of the FP64 atomic additions.  Two calls in a row
check that the shared array's leftovers from one call do not leak into the
next.  The file is named to be collected last; it also passes alone.
"""
import ctypes as C

import numpy as np
import pytest

import egsnrc_gb300 as eg
from egsnrc_gb300 import workloads as W

pytestmark = pytest.mark.gpu

TOL = 1e-12   # the chunking-invariance tolerance of the parity tests


def engine(wl, precision):
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=precision)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    return eng


def reference_sum(wl, precision, first, n, seed):
    eng = engine(wl, precision)
    eng.run(n, nbatch=1, seed=seed, first=first)
    s, _, _ = eng.tallies()
    eng.close()
    return s


@pytest.mark.parametrize("precision", [64, 32])
@pytest.mark.parametrize("workload,n", [("water30", 2000), ("slab64", 2000), ("water128e", 200)])
def test_noalloc_matches_run_on_two_calls(workload, n, precision):
    import torch
    wl = W.WORKLOADS[workload](20)
    eng = engine(wl, precision)
    dose = torch.full((wl["geometry"].nvox,), 123.0, dtype=torch.float64, device="cuda")
    seed = 11
    for call, first in enumerate((0, 5000)):
        eng.run_noalloc(dose.data_ptr(), n, seed=seed, first=first)
        got = dose.cpu().numpy()
        want = reference_sum(wl, precision, first, n, seed)
        assert want.sum() > 0
        assert np.allclose(got, want, rtol=TOL, atol=TOL), (call, np.abs(got - want).max())
    # the handle's own tallies are not touched
    s, _, t = eng.tallies()
    assert not s.any() and t[0] == 0
    eng.close()


def test_noalloc_rejects_oversized_calls():
    import torch
    wl = W.water30(20)
    eng = engine(wl, 64)
    dose = torch.zeros(wl["geometry"].nvox, dtype=torch.float64, device="cuda")
    with pytest.raises(eg.EGSError) as ex:
        eng.run_noalloc(dose.data_ptr(), eg.NOALLOC_MAX_HISTORIES + 1)
    assert ex.value.code == 1 and "at most" in str(ex.value)
    L = eg.load_library()
    assert L.egsgpu_run_noalloc(eng.h, 0, 10, 1, None, None) == 1
    eng.close()


@pytest.mark.parametrize("option", [{"howfarless": 1}, {"bca_algorithm": 1}])
def test_noalloc_refuses_other_transport_modes(option):
    # HOWFARLESS and PRESTA-I have kernels of their own that the fixed-scratch
    # path does not launch: the call must refuse rather than transport with
    # the default physics
    import torch
    wl = W.water30(20)
    eng = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=64, **option)
    eng.set_geometry(wl["geometry"])
    eng.set_source(wl["source"])
    dose = torch.zeros(wl["geometry"].nvox, dtype=torch.float64, device="cuda")
    with pytest.raises(eg.EGSError) as ex:
        eng.run_noalloc(dose.data_ptr(), 10)
    assert ex.value.code == 1
    eng.close()


def test_noalloc_refuses_a_capturing_stream():
    # the call synchronises its stream every round, so it cannot be recorded
    # into a graph: on a capturing stream it must refuse at once and leave the
    # caller's capture valid
    import torch
    wl = W.water30(20)
    eng = engine(wl, 32)
    dose = torch.zeros(wl["geometry"].nvox, dtype=torch.float64, device="cuda")
    eng.run_noalloc(dose.data_ptr(), 16, seed=3)
    torch.cuda.synchronize()
    side = torch.cuda.Stream()
    g = torch.cuda.CUDAGraph()
    refused = None
    with torch.cuda.graph(g, stream=side):
        dose.mul_(2.0)   # the captured work: the graph must stay usable
        try:
            eng.run_noalloc(dose.data_ptr(), 16, seed=3, stream=side.cuda_stream)
        except eg.EGSError as ex:
            refused = ex
    assert refused is not None and refused.code == 7 and "capturing" in str(refused)
    before = dose.clone()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(dose, 2.0 * before)
    eng.close()
