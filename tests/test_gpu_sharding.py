"""History sharding through the engine: two ranks (gloo, world size 2) share
the one GPU, each transports a disjoint history range through libegsgpu
(FP64), writes a checkpoint, and rank 0 combines the gathered checkpoints with
egsgpu_combine_checkpoints (the .egsdat combine of egs_application.cpp:624-660)
and restores the result into a fresh engine.  Its tallies and doses must equal
those of one engine running every history with the same batches (1e-12).  The
ranks' kernels never wait on one another."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

pytestmark = pytest.mark.gpu

N = 6000
BATCHES_PER_RANK = 3


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def engine():
    import egsnrc_gb300 as eg
    from egsnrc_gb300 import workloads as W
    wl = W.slab64(24)
    e = eg.DoseEngine(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"], precision=64)
    e.set_geometry(wl["geometry"])
    e.set_source(wl["source"])
    return e


def _rank(rank, world, port, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    import egsnrc_gb300 as eg
    e = engine()
    per = N // world
    e.run(per, nbatch=BATCHES_PER_RANK, seed=9, first=rank * per)
    blobs = [None] * world
    dist.all_gather_object(blobs, e.checkpoint())
    e.close()
    if rank == 0:
        comb = blobs[0]
        for b in blobs[1:]:
            comb = eg.combine_checkpoints(comb, b)
        with open(out_path, "wb") as f:
            f.write(comb)
    dist.barrier()
    dist.destroy_process_group()


def test_two_ranks_on_one_gpu_combine_to_one_run(tmp_path):
    out = str(tmp_path / "combined.bin")
    mp.start_processes(_rank, args=(2, free_port(), out), nprocs=2, join=True, start_method="spawn")
    comb = open(out, "rb").read()
    got = engine()
    got.restore(comb)
    ref = engine()
    ref.run(N, nbatch=2 * BATCHES_PER_RANK, seed=9)
    s1, s21, t1 = got.tallies()
    s2, s22, t2 = ref.tallies()
    assert t1[0] == t2[0] == N and t1[1] == t2[1] == 2 * BATCHES_PER_RANK
    assert np.allclose(s1, s2, rtol=1e-12, atol=1e-15)
    assert np.allclose(s21, s22, rtol=1e-12, atol=1e-20)
    assert np.allclose(t1[2:4], t2[2:4], rtol=1e-12)
    d1, e1 = got.dose()
    d2, e2 = ref.dose()
    assert np.allclose(d1, d2, rtol=1e-12, atol=0) and np.allclose(e1, e2, rtol=1e-9, atol=0)
