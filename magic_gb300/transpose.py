"""LM <-> R transposes around the radial loop (mpi_transpose.f90:120-620),
over torch.distributed: NCCL for CUDA tensors, gloo for CPU tensors.

MagIC keeps two distributions of its spectral fields:
  * R-distributed (radial loop): f_Rloc(lm_max, nRstart:nRstop), every lm in
    the standard m-major order (st_map) for this rank's radial levels;
  * LM-distributed (implicit solves): f_LMloc(llm:ulm, n_r_max), this rank's
    block of lm in the load-balancing order lo_map, for every radial level.
The transposes exchange the two with one all-to-all (the alltoallv form of
mpi_transpose.f90:281-530): to each rank p go the lm of p's block (lo_map
order) at this rank's levels.  Arrays here are row-major with the field
first: R-distributed [n_fields][n_r_loc][lm_max], LM-distributed
[n_fields][n_r_max][n_lm_loc] -- the memory order of the reference's
(lm, nR, field) arrays.

The lo_map order and the lm blocks follow initialize_blocking
(blocking.f90:79-95): the snake distribution of the l values
(get_snake_lm_blocking, blocking.f90:387-544) when n_procs <= l_max/2, else
the l-major order (get_lorder_lm_blocking, :339-385) cut into getBlocks
blocks (parallel.f90:75-92); radial levels in getBlocks blocks
(radial_data.f90:22-38).
"""
from __future__ import annotations

from typing import List, Optional, Tuple

import numpy as np

from .radial import radial_blocks


def st_lm2(l_max: int, minc: int, m_max: Optional[int] = None) -> np.ndarray:
    """st_map%lm2 (0-based): index of (l, m) in the m-major order; -1 where
    (l, m) is not a mode (blocking.f90:293-337)."""
    m_max = (l_max // minc) * minc if m_max is None else m_max
    lm2 = -np.ones((l_max + 1, l_max + 1), dtype=np.int64)
    lm = 0
    for m in range(0, m_max + 1, minc):
        for l in range(m, l_max + 1):
            lm2[l, m] = lm
            lm += 1
    return lm2


def lo_map(l_max: int, minc: int, n_procs: int, m_max: Optional[int] = None
           ) -> Tuple[np.ndarray, np.ndarray, List[Tuple[int, int]]]:
    """(lm2l, lm2m, blocks): the lo_map order (0-based lm) and every rank's
    [start, stop) range of it."""
    m_max = (l_max // minc) * minc if m_max is None else m_max
    lm_max = sum(l_max - m + 1 for m in range(0, m_max + 1, minc))
    if n_procs <= l_max // 2:
        l_lists = _snake_l_lists(l_max, n_procs)
        lm2l, lm2m, blocks = [], [], []
        for p in range(n_procs):
            start = len(lm2l)
            for l in l_lists[p]:
                for m in range(0, min(m_max, l) + 1, minc):
                    lm2l.append(l)
                    lm2m.append(m)
            blocks.append((start, len(lm2l)))
    else:
        lm2l, lm2m = [], []
        for l in range(0, l_max + 1):
            for m in range(0, min(m_max, l) + 1, minc):
                lm2l.append(l)
                lm2m.append(m)
        blocks = radial_blocks(lm_max, n_procs)
    assert len(lm2l) == lm_max
    return np.array(lm2l), np.array(lm2m), blocks


def _snake_l_lists(l_max: int, n_procs: int) -> List[List[int]]:
    """The l values of every rank (get_snake_lm_blocking, blocking.f90:405-480):
    l = l_max .. 0 dealt to the ranks back and forth (0, 1, .., n-1, n-1, ..,
    0, 0, 1, ..); the lists then rotated so that the rank holding l = 0 comes
    first, and l = 0 swapped to the front of its list."""
    lists: List[List[int]] = [[] for _ in range(n_procs)]
    proc, ascending, l0proc = 0, True, 0
    for l in range(l_max, -1, -1):
        lists[proc].append(l)
        if l == 0:
            l0proc = proc
        if ascending:
            if proc < n_procs - 1:
                proc += 1
            else:
                ascending = False
        else:
            if proc > 0:
                proc -= 1
            else:
                ascending = True
    if l0proc != 0:
        # the reference's cycle moves list (l0proc + pc) mod n to pc along one cycle
        tmp = lists[0]
        pc = 0
        while True:
            src = (l0proc + pc) % n_procs
            if src != 0:
                lists[pc] = lists[src]
            else:
                lists[pc] = tmp
                break
            pc = src
    first = lists[0]
    if 0 in first:
        i = first.index(0)
        first[0], first[i] = first[i], first[0]
    return lists


class RadialTransposer:
    """LM <-> R transposes of n_fields spectral fields for this rank of the
    default process group (or `group`): r2lm is transp_r2lm, lm2r is
    transp_lm2r.  Tensors are complex128 on the device of the backend (CUDA
    for NCCL, CPU for gloo)."""

    def __init__(self, l_max: int, minc: int, n_r_max: int, group=None, m_max: Optional[int] = None):
        import torch
        import torch.distributed as dist
        self.dist, self.group = dist, group
        self.rank = dist.get_rank(group)
        self.n_procs = dist.get_world_size(group)
        self.l_max, self.minc, self.n_r_max = l_max, minc, n_r_max
        lm2l, lm2m, self.lm_blocks = lo_map(l_max, minc, self.n_procs, m_max)
        st = st_lm2(l_max, minc, m_max)
        self.lm_max = len(lm2l)
        self.r_blocks = radial_blocks(n_r_max, self.n_procs)
        # st_map index of every lo_map entry, per rank block
        self.st_of_block = [torch.as_tensor(st[lm2l[a:b], lm2m[a:b]]) for a, b in self.lm_blocks]
        self.lm_lo, self.lm_hi = self.lm_blocks[self.rank]
        self.r_lo, self.r_hi = self.r_blocks[self.rank]
        self._dev = {}

    @property
    def n_lm_loc(self) -> int:
        return self.lm_hi - self.lm_lo

    @property
    def n_r_loc(self) -> int:
        return self.r_hi - self.r_lo

    def _idx(self, device):
        if device not in self._dev:
            self._dev[device] = [t.to(device) for t in self.st_of_block]
        return self._dev[device]

    def _exchange(self, send, send_counts, recv_counts):
        """all_to_all of complex128 data as float64 pairs (both backends)."""
        import torch
        recv = torch.empty(2 * sum(recv_counts), dtype=torch.float64, device=send.device)
        self.dist.all_to_all_single(recv, torch.view_as_real(send).reshape(-1),
                                    [2 * c for c in recv_counts], [2 * c for c in send_counts], group=self.group)
        return torch.view_as_complex(recv.view(-1, 2))

    def r2lm(self, arr_Rloc, out=None):
        """[n_fields][n_r_loc][lm_max] (st order) -> [n_fields][n_r_max][n_lm_loc] (lo order)."""
        import torch
        nf = arr_Rloc.shape[0]
        assert tuple(arr_Rloc.shape) == (nf, self.n_r_loc, self.lm_max), arr_Rloc.shape
        idx = self._idx(arr_Rloc.device)
        # to rank p: this rank's levels at the lm of p's block, in lo order
        send = torch.cat([arr_Rloc.index_select(2, idx[p]).reshape(-1) for p in range(self.n_procs)])
        scount = [nf * self.n_r_loc * (b - a) for a, b in self.lm_blocks]
        rcount = [nf * (b - a) * self.n_lm_loc for a, b in self.r_blocks]
        recv = self._exchange(send, scount, rcount)
        if out is None:
            out = torch.empty((nf, self.n_r_max, self.n_lm_loc), dtype=arr_Rloc.dtype, device=arr_Rloc.device)
        off = 0
        for p, (a, b) in enumerate(self.r_blocks):
            out[:, a:b, :] = recv[off:off + rcount[p]].view(nf, b - a, self.n_lm_loc)
            off += rcount[p]
        return out

    def lm2r(self, arr_LMloc, out=None):
        """[n_fields][n_r_max][n_lm_loc] (lo order) -> [n_fields][n_r_loc][lm_max] (st order)."""
        import torch
        nf = arr_LMloc.shape[0]
        assert tuple(arr_LMloc.shape) == (nf, self.n_r_max, self.n_lm_loc), arr_LMloc.shape
        idx = self._idx(arr_LMloc.device)
        # to rank p: this rank's lm block at p's levels
        send = torch.cat([arr_LMloc[:, a:b, :].reshape(-1) for a, b in self.r_blocks])
        scount = [nf * (b - a) * self.n_lm_loc for a, b in self.r_blocks]
        rcount = [nf * self.n_r_loc * (b - a) for a, b in self.lm_blocks]
        recv = self._exchange(send, scount, rcount)
        if out is None:
            out = torch.empty((nf, self.n_r_loc, self.lm_max), dtype=arr_LMloc.dtype, device=arr_LMloc.device)
        off = 0
        for p, (a, b) in enumerate(self.lm_blocks):
            out.index_copy_(2, idx[p], recv[off:off + rcount[p]].view(nf, self.n_r_loc, b - a))
            off += rcount[p]
        return out
