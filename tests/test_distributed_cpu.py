"""Multi-rank path on CPU (gloo, world_size 2): radial levels are sharded in
contiguous blocks (src/parallel.f90:75-92), each rank transforms only its
own levels with no exchange inside the transform, and the gathered results
equal the single-process transform of all levels."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    from magic_gb300.radial import radial_blocks
    from magic_gb300.workload import spectra
    from oracle.oracle import OracleSHT, set_threads
    set_threads(1)
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    n = 7
    S = spectra(15, 1, n, seed=21)
    lo, hi = radial_blocks(n, world)[rank]
    o = OracleSHT(15, 1, 24, 48)
    mine = np.zeros((n, 48, 24))
    for r in range(lo, hi):
        mine[r] = o.scal_to_spat(S[r])
    t = torch.from_numpy(mine)
    dist.all_reduce(t)  # disjoint level blocks: the sum is a gather
    if rank == 0:
        ref = np.array([o.scal_to_spat(S[r]) for r in range(n)])
        q.put(float(np.abs(t.numpy() - ref).max()))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_radial_sharding():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    err = q.get(timeout=120)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert err == 0.0
