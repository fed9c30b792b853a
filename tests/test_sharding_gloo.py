"""History sharding across ranks (world_size 2, gloo on CPU).

Histories are independent and own their random-number streams, so ranks
transport disjoint history ranges and only the final per-voxel tallies are
summed (the .egsdat combine of the reference, egs_application.cpp:624-660).
Each rank runs the CPU oracle here (no GPU on this machine) and writes its
tallies in the engine's checkpoint layout; the blobs are gathered over gloo
and combined by the library's host-only egsgpu_combine_checkpoints.  The
combination must equal a single run over all histories.  The same combine of
engine checkpoints on the GPU is tests/test_gpu_sharding.py."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp


def free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, n, out_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from egsnrc_gb300 import workloads as W
    from oracle.oracle_binding import Oracle
    wl = W.water30(12)
    o = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
    o.set_geometry(wl["geometry"])
    o.set_source(wl["source"])
    per = n // world
    o.run(per, nbatch=2, seed=5, first=rank * per)
    s, s2, t = o.tallies()
    mine = checkpoint_blob(s, s2, per, 2, t[2], t[3])
    blobs = [None] * world
    dist.all_gather_object(blobs, mine)
    if rank == 0:
        import egsnrc_gb300 as eg
        comb = blobs[0]
        for b in blobs[1:]:
            comb = eg.combine_checkpoints(comb, b)
        c = eg.checkpoint_arrays(comb)
        np.save(out_path, np.concatenate([c["sum"], c["sum2"], [c["deposited"], c["escaped"], c["histories"],
                                                               c["batches"]]]))
    dist.barrier()
    dist.destroy_process_group()


def checkpoint_blob(s, s2, hist, batches, dep, esc):
    """Tallies in the layout of egsgpu_checkpoint."""
    hdr = np.array([0x45475347505531, len(s), hist, batches], dtype=np.int64).tobytes()
    return (hdr + np.array([dep, esc]).tobytes() + np.zeros(8, np.uint64).tobytes()
            + np.asarray(s, np.float64).tobytes() + np.asarray(s2, np.float64).tobytes())


def test_two_rank_history_sharding(tmp_path):
    n = 4000
    out = str(tmp_path / "sharded.npy")
    mp.spawn(_worker, args=(2, free_port(), n, out), nprocs=2, join=True)
    got = np.load(out)
    from egsnrc_gb300 import workloads as W
    from oracle.oracle_binding import Oracle
    wl = W.water30(12)
    o = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
    o.set_geometry(wl["geometry"])
    o.set_source(wl["source"])
    nv = wl["geometry"].nvox
    # the single run: the same four batches of n/4 histories
    s = np.zeros(nv)
    for b in range(4):
        ob = Oracle(wl["media"], ecut=wl["ecut"], pcut=wl["pcut"])
        ob.set_geometry(wl["geometry"])
        ob.set_source(wl["source"])
        ob.run(n // 4, nbatch=1, seed=5, first=b * n // 4)
        sb, _, _ = ob.tallies()
        s += sb
    o.run(n, nbatch=4, seed=5, first=0)
    s1, s21, t = o.tallies()
    assert np.allclose(got[:nv], s1, rtol=1e-12, atol=1e-15)
    assert np.allclose(got[:nv], s, rtol=1e-12, atol=1e-15)
    assert np.allclose(got[nv:2 * nv], s21, rtol=1e-12, atol=1e-20)
    assert np.allclose(got[2 * nv:2 * nv + 2], t[2:4], rtol=1e-12)
    assert list(got[-2:]) == [n, 4]
