"""History sharding across ranks (world_size 2, gloo on CPU).

Histories are independent and own their random-number streams, so ranks
transport disjoint history ranges and only the final per-voxel tallies are
summed (the .egsdat combine of the reference, egs_application.cpp:624-660).
Each rank runs the CPU oracle here; the sum over ranks must equal a single
run over all histories."""
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
    o.run(per, nbatch=1, seed=5, first=rank * per)
    s, _, t = o.tallies()
    ts = torch.from_numpy(s.copy())
    tt = torch.from_numpy(t[2:4].copy())
    dist.all_reduce(ts)
    dist.all_reduce(tt)
    if rank == 0:
        np.save(out_path, np.concatenate([ts.numpy(), tt.numpy()]))
    dist.barrier()
    dist.destroy_process_group()


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
    o.run(n, nbatch=1, seed=5, first=0)
    s, _, t = o.tallies()
    assert np.allclose(got[:-2], s, rtol=1e-12, atol=1e-15)
    assert np.allclose(got[-2:], t[2:4], rtol=1e-12)
