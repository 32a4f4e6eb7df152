"""Comparison of engine results with the oracle, with the tolerances written
out.

Two FP32 evaluations of the same (t0, candidate) differ by a few ulps of the
traveltime; t/dt ~ 1e3 has an ulp of ~6e-5 samples, which moves the
interpolation fraction and changes the semblance by ~1e-5 .. 1e-4 relative,
and, when a window lies exactly at a trace edge, includes or drops one trace
(a discrete jump).  So results are judged by distributions:

* chosen semblance: samples off by more than 1e-3 absolute (window-edge
  jumps) <= JUMP_FRAC; over the other samples the relative error (floor
  1e-3) at the 99.9th percentile <= SEMBL_P999 x index_scale(S): the
  traveltime's rounding moves t/dt by an ulp of t/dt, so the tolerance grows
  with the largest sample index (1 up to 512 samples, 4 at 2000);
* chosen candidate: identical except where the two best candidates of the
  oracle's own table are within NEAR_TIE relative (near-ties), counted;
  other disagreements <= FAR_FRAC of the samples (window-edge jumps);
* stack at the same chosen candidate: abs error p99.9 <= STACK_P999 * RMS
  amplitude of the selected traces.
"""
from __future__ import annotations

import dataclasses

import numpy as np

from oracle import oracle

SEMBL_P999 = 2e-4
JUMP_FRAC = 5e-3
NEAR_TIE = 1e-4
FAR_FRAC = 2e-3
STACK_P999 = 1e-3


def index_scale(S: int, model: str = "cmp") -> float:
    """ulp of the largest window index of an S-sample trace over that of a
    512-sample trace (at least 1); twice that for OCT, whose time is some 40
    FP32 operations with square roots and divisions (two FP32 evaluations of
    it differ by more ulps than the CMP / ZO-CRS forms)."""
    s = max(1.0, float(2 ** int(np.ceil(np.log2(max(S, 1))))) / 512.0)
    return 2.0 * s if model == "oct" else s


@dataclasses.dataclass
class Report:
    sembl_p999: float = SEMBL_P999
    samples: int = 0
    mismatches: int = 0
    near_ties: int = 0
    far: int = 0
    sembl_rel: list = dataclasses.field(default_factory=list)
    jumps: int = 0
    stack_err: list = dataclasses.field(default_factory=list)

    def check(self):
        rel = np.concatenate(self.sembl_rel) if self.sembl_rel else np.zeros(1)
        se = np.concatenate(self.stack_err) if self.stack_err else np.zeros(1)
        n = max(self.samples, 1)
        assert np.quantile(rel, 0.999) <= self.sembl_p999, np.quantile(rel, 0.999)
        assert self.jumps <= JUMP_FRAC * n, (self.jumps, n)
        assert self.far <= FAR_FRAC * n, (self.far, n)
        assert np.quantile(se, 0.999) <= STACK_P999, np.quantile(se, 0.999)
        return self

    def summary(self):
        rel = np.concatenate(self.sembl_rel) if self.sembl_rel else np.zeros(1)
        return dict(samples=self.samples, mismatches=self.mismatches, near_ties=self.near_ties,
                    far=self.far, jumps=self.jumps, sembl_rel_p999=float(np.quantile(rel, 0.999)),
                    sembl_rel_max=float(rel.max()))


def chosen_index(params: np.ndarray, block: np.ndarray) -> np.ndarray:
    """Candidate index of a result block [(2+np)][S] (velocity via 2/sqrt(c))."""
    v = 2.0 / np.sqrt(params[:, 0].astype(np.float64))
    out = np.full(block.shape[1], -1, np.int64)
    for s in range(block.shape[1]):
        c = np.nonzero(np.isclose(v, block[2, s], rtol=2e-6, atol=0))[0]
        for j in range(1, params.shape[1]):
            c = c[params[c, j] == block[2 + j, s]]
        if c.size:
            out[s] = c[0]
    return out


def compare_block(rep: Report, got: np.ndarray, sem: np.ndarray, stk: np.ndarray,
                  params: np.ndarray, rms: float, raw_params: bool = False):
    """got: engine block [(2+np)][S]; sem/stk: oracle tables [S][P]."""
    ref, idx = oracle.ls_result("x", sem, stk, params)
    S = got.shape[1]
    rep.samples += S
    g0 = got[0].astype(np.float64)
    r0 = ref[0].astype(np.float64)
    rel = np.abs(g0 - r0) / np.maximum(np.abs(r0), 1e-3)
    jump = np.abs(g0 - r0) > 1e-3
    rep.sembl_rel.append(rel[~jump])
    rep.jumps += int(np.sum(jump))
    gi = chosen_index(params, got)
    same = gi == idx
    rows = np.arange(S)
    for s in np.nonzero(~same)[0]:
        rep.mismatches += 1
        best = float(sem[s, idx[s]])
        alt = float(sem[s, gi[s]]) if gi[s] >= 0 else -np.inf
        if abs(best - alt) <= NEAR_TIE * max(abs(best), 1e-3):
            rep.near_ties += 1
        else:
            rep.far += 1
    if same.any():
        rep.stack_err.append(np.abs(got[1][same] - stk[rows[same], idx[same]]) / max(rms, 1e-12))
    return rep


# Stack of the tuned kernel against the plain kernel (or the reference's
# kernels): the tuned kernel sums the same window values in another order
# (the per-tap sums first), so the stack agrees to a few ulp of the summands:
# |a - b| <= STACK_REL * (|b| + max |b| over the midpoint).
STACK_REL = 1e-5


def assert_same_but_stack(a: np.ndarray, b: np.ndarray, n_params: int):
    """a, b: result tables [nM0][2+np][S] (or [S][2+np] rows).  Semblance and
    parameter rows identical; stack within STACK_REL."""
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    assert a.shape == b.shape
    if a.ndim == 3:
        assert np.array_equal(a[:, 0], b[:, 0]), "semblance differs"
        assert np.array_equal(a[:, 2:], b[:, 2:]), "chosen parameters differ"
        sa, sb = a[:, 1], b[:, 1]
        scale = np.max(np.abs(sb), axis=1, keepdims=True)
    else:
        keep = [0] + list(range(2, 2 + n_params))
        assert np.array_equal(a[..., keep], b[..., keep]), "semblance or parameters differ"
        sa, sb = a[..., 1], b[..., 1]
        scale = np.max(np.abs(sb))
    err = np.abs(sa - sb)
    tol = STACK_REL * (np.abs(sb) + scale)
    assert np.all(err <= tol), float(np.max(err / np.maximum(tol, 1e-30)))
    return float(np.max(err / np.maximum(np.abs(sb) + scale, 1e-30)))


def count_near_ties(sem: np.ndarray, rel: float = 1e-4) -> int:
    """Samples of an oracle semblance table [S][P] counted as near-ties by the
    engine (hpss_stats.near_ties): best > 0 and the runner-up within
    rel * max(best, 1e-3) of it."""
    sem = np.where(np.isnan(sem), -np.inf, sem.astype(np.float32))
    if sem.shape[1] < 2:
        return 0
    top = np.sort(sem, axis=1)[:, -2:]
    best, second = top[:, 1], top[:, 0]
    tie = (best > 0) & (second >= 0) & \
        (best - second <= np.float32(rel) * np.maximum(best, np.float32(1e-3)))
    return int(np.sum(tie))
