"""LM <-> R transposes (magic_gb300/transpose.py, mpi_transpose.f90:120-620)
on CPU: the lo_map order and lm blocks of blocking.f90 (snake and l-major
forms), and the all-to-all exchange over gloo ranks (world size 2 and 3)
against the global arrays; the transposes move data only, so every
comparison is exact."""
import os
import socket

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from magic_gb300.transpose import _snake_l_lists, lo_map, st_lm2


def test_snake_order_by_hand():
    # l = 4 .. 0 dealt to ranks 0, 1, 1, 0, 0; l = 0 swapped to the front of rank 0's list
    assert _snake_l_lists(4, 2) == [[0, 1, 4], [3, 2]]
    # l = 9 .. 0 dealt to ranks 0,1,2,2,1,0,0,1,2,2: l = 0 on rank 2, so the lists
    # rotate by the reference's cycle (rank 2's list to rank 0, 1's to 2, 0's to 1)
    # and l = 0 swaps with the first l of rank 0
    assert _snake_l_lists(9, 3) == [[0, 6, 1, 7], [9, 4, 3], [8, 5, 2]]
    lm2l, lm2m, blocks = lo_map(4, 1, 2)
    assert blocks == [(0, 8), (8, 15)]
    assert list(lm2l) == [0, 1, 1, 4, 4, 4, 4, 4, 3, 3, 3, 3, 2, 2, 2]
    assert list(lm2m) == [0, 0, 1, 0, 1, 2, 3, 4, 0, 1, 2, 3, 0, 1, 2]


@pytest.mark.parametrize("l_max,minc,n_procs", [(4, 1, 2), (9, 1, 3), (10, 1, 4), (12, 3, 5), (20, 1, 3),
                                                (31, 1, 7), (4, 1, 3), (5, 1, 4), (63, 4, 16)])
def test_lo_map_is_a_blocked_permutation(l_max, minc, n_procs):
    lm2l, lm2m, blocks = lo_map(l_max, minc, n_procs)
    st = st_lm2(l_max, minc)
    idx = st[lm2l, lm2m]
    lm_max = int((st >= 0).sum())
    assert sorted(idx) == list(range(lm_max))            # every mode exactly once
    assert blocks[0][0] == 0 and blocks[-1][1] == lm_max
    assert all(blocks[p][1] == blocks[p + 1][0] for p in range(n_procs - 1))
    assert lm2l[0] == 0 and lm2m[0] == 0                  # l = 0 leads rank 0's block
    if n_procs <= l_max // 2:
        # snake: every l lives on one rank, with all its m in order
        for p, (a, b) in enumerate(blocks):
            ls = lm2l[a:b]
            for l in set(ls):
                ms = lm2m[a:b][ls == l]
                assert list(ms) == list(range(0, min(l, (l_max // minc) * minc) + 1, minc))
                assert (lm2l == l).sum() == len(ms)
        # the numbers of l values per rank differ by at most one
        counts = [len(set(lm2l[a:b])) for a, b in blocks]
        assert max(counts) - min(counts) <= 1
    else:
        # l-major order cut into getBlocks blocks
        assert all(np.diff(lm2l) >= 0)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, q, l_max, minc, n_r_max):
    import sys
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
    import torch
    from magic_gb300.transpose import RadialTransposer
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        t = RadialTransposer(l_max, minc, n_r_max)
        nf = 3
        rng = np.random.default_rng(5)
        G = torch.from_numpy(rng.standard_normal((nf, n_r_max, t.lm_max))
                             + 1j * rng.standard_normal((nf, n_r_max, t.lm_max)))
        Rloc = G[:, t.r_lo:t.r_hi, :].contiguous()
        LM = t.r2lm(Rloc)
        ok = torch.equal(LM, G[:, :, t.st_of_block[rank]])
        back = t.lm2r(LM)
        ok = ok and torch.equal(back, Rloc)
        # the LM block of another distribution of levels comes back in R order
        LM2 = G[:, :, t.st_of_block[rank]].contiguous() * 2
        ok = ok and torch.equal(t.lm2r(LM2), 2 * Rloc)
        q.put((rank, bool(ok)))
    finally:
        dist.barrier()
        dist.destroy_process_group()


@pytest.mark.parametrize("world,l_max,minc,n_r_max", [(2, 15, 1, 9), (3, 10, 2, 8), (3, 4, 1, 7)])
def test_transposes_over_gloo(world, l_max, minc, n_r_max):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, q, l_max, minc, n_r_max)) for r in range(world)]
    for p in procs:
        p.start()
    res = dict(q.get(timeout=120) for _ in range(world))
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert all(res.values()), res
