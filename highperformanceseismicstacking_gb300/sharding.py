"""Midpoint sharding across processes (one GPU per process, no collective).

The units of work are independent midpoints (the reference splits them across
GPU threads, SingleHostRunner.cpp:141-148, and across SPITS tasks,
SpitzJobManager.cpp:17-42).  A rank gets a contiguous range of CDP midpoints;
for apertures (ZO-CRS / OCT) it also needs the traces within the aperture of
its range edges (the halo), which it reads but does not own.  Results are
concatenated on the host in midpoint order.
"""
from __future__ import annotations

from typing import List, Tuple

import numpy as np


def shard_midpoints(m0s: np.ndarray, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of the sorted midpoint list for `rank`.
    Sizes differ by at most one; every midpoint belongs to exactly one rank."""
    n = len(m0s)
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def halo_trace_range(midpoints: np.ndarray, m_lo: float, m_hi: float,
                     radius: float) -> Tuple[int, int]:
    """Trace index range [a, b) of a (midpoint-sorted) line that a shard
    covering midpoints [m_lo, m_hi] reads: every trace within `radius` of the
    range (radius = apm for ZO-CRS; apm + sqrt(hmax^2 + h0^2) for OCT)."""
    a = int(np.searchsorted(midpoints, np.float32(m_lo - radius), side="left"))
    b = int(np.searchsorted(midpoints, np.float32(m_hi + radius), side="right"))
    return a, b


def gather_results(parts: List[np.ndarray]) -> np.ndarray:
    """Concatenate per-rank result blocks [n_i][2+np][S] in rank order."""
    return np.concatenate(parts, axis=0) if parts else np.zeros((0,))
