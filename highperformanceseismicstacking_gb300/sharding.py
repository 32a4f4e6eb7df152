"""Midpoint sharding across processes (one GPU per process, no collective on
the data path).

The units of work are independent midpoints (the reference splits them
across GPU threads, SingleHostRunner.cpp:141-148, and across SPITS tasks,
SpitzJobManager.cpp:17-42).  A rank gets a contiguous range of CDP
midpoints; for apertures (ZO-CRS / OCT) it also reads the traces within the
selection radius of its range edges (the halo), which it does not own.
Results are concatenated on the host in midpoint order.

Selection radius per model (the largest |m - m0| at which a trace can be
selected for midpoint m0):

* CMP: 0 -- a trace belongs to the gather of its own midpoint
  (selectTracesForCommonMidPoint, m == m0).
* ZO-CRS: apm -- |m0 - m| <= apm (selectTracesForZeroOffsetCommonReflection
  Surface).
* OCT: apm + sqrt(hmax^2 + h0^2).  A trace is selected when |m - mh| <= apm
  for the displaced midpoint mh of some candidate (oct/common.cuh:7-35):
  mh - m0 = 2 theta (h^2 - h0^2) / sqrt(q) with
  q = theta^2 gamma^2 + 2 tq + 2 sqrt(tq^2 + tq theta^2 gamma^2 +
  16 h^2 h0^2 theta^4), gamma = 2 sqrt(h^2 + h0^2), tq = (t0^2 - c h0^2)^2.
  Every term of q is >= 0, so sqrt(q) >= |theta| gamma and
  |mh - m0| <= |h^2 - h0^2| / sqrt(h^2 + h0^2) <= sqrt(h^2 + h0^2); hence
  |m - m0| <= apm + sqrt(h^2 + h0^2) <= apm + sqrt(hmax^2 + h0^2).  The
  radius is widened by 0.1 % + 1 m for FP32 rounding, as the engine's own
  prefilter (hpss_capi.cu, oct_candidate_slots).
"""
from __future__ import annotations

import math
from typing import List, Sequence, Tuple

import numpy as np


def shard_midpoints(m0s: np.ndarray, world: int, rank: int) -> Tuple[int, int]:
    """Contiguous [start, stop) of the sorted midpoint list for `rank`.
    Sizes differ by at most one; every midpoint belongs to exactly one rank."""
    n = len(m0s)
    base, extra = divmod(n, world)
    start = rank * base + min(rank, extra)
    stop = start + base + (1 if rank < extra else 0)
    return start, stop


def selection_radius(model: str, apm: float = 0.0, hmax: float = 0.0,
                     h0s: Sequence[float] = (0.0,)) -> float:
    """Largest |m - m0| at which a trace can be selected (module docstring)."""
    if model == "cmp":
        return 0.0
    if model == "zocrs":
        return float(apm)
    h0 = max(abs(float(v)) for v in h0s) if len(h0s) else 0.0
    return (float(apm) + math.sqrt(float(hmax) ** 2 + h0 * h0)) * 1.001 + 1.0


def halo_trace_range(midpoints: np.ndarray, m_lo: float, m_hi: float,
                     radius: float) -> Tuple[int, int]:
    """Trace index range [a, b) of a (midpoint-sorted) line that a shard
    covering midpoints [m_lo, m_hi] reads: every trace within `radius` of the
    range (selection_radius)."""
    a = int(np.searchsorted(midpoints, np.float32(m_lo - radius), side="left"))
    b = int(np.searchsorted(midpoints, np.float32(m_hi + radius), side="right"))
    return a, b


def shard_plan(cdp_midpoints: np.ndarray, trace_midpoints: np.ndarray, world: int, rank: int,
               radius: float) -> Tuple[Tuple[int, int], Tuple[int, int]]:
    """The midpoints [m_a, m_b) a rank owns and the traces [t_a, t_b) it
    reads (its own and the halo).  An empty shard reads no traces."""
    ma, mb = shard_midpoints(cdp_midpoints, world, rank)
    if mb <= ma:
        return (ma, mb), (0, 0)
    ta, tb = halo_trace_range(trace_midpoints, float(cdp_midpoints[ma]),
                              float(cdp_midpoints[mb - 1]), radius)
    return (ma, mb), (ta, tb)


def gather_results(parts: List[np.ndarray]) -> np.ndarray:
    """Concatenate per-rank result blocks [n_i][2+np][S] in rank order."""
    parts = [p for p in parts if p is not None and len(p)]
    return np.concatenate(parts, axis=0) if parts else np.zeros((0,))
