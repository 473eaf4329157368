"""Radial-level sharding across ranks, the reference's R-distribution.

getBlocks (src/parallel.f90:75-92) as used by initialize_radial_data
(src/radial_data.f90:22-38): contiguous blocks of radial levels, the
remainder going to the last ranks.  Each rank transforms only its own levels
(no exchange inside the transforms), so a multi-GPU run is N independent
batches over disjoint level ranges.
"""
from __future__ import annotations

from typing import List, Tuple


def radial_blocks(n_points: int, n_procs: int) -> List[Tuple[int, int]]:
    """0-based [start, stop) level range of every rank."""
    loc = n_points // n_procs
    rem = n_points - loc * n_procs
    out = []
    prev_stop = 0
    for p in range(n_procs):
        start = loc * p + max(p + rem - n_procs, 0) + 1
        stop = loc * (p + 1) + max(p + rem + 1 - n_procs, 0)
        if p != 0:
            start = prev_stop + 1
        out.append((start - 1, stop))
        prev_stop = stop
    return out
