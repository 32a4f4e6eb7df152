"""The oracle against analytic known-answer cases (CPU only).

The reference ships no tests or fixtures, so these known answers, the FP32 vs
FP64 agreement and the reference-kernel golden fixtures (test_golden.py) are
what pins the oracle.
"""
import numpy as np
import pytest

from oracle import oracle
from highperformanceseismicstacking_gb300 import synthetic


def _line(n_tr=6, S=200, fill=None, h_step=100.0, m=1000.0):
    hoff = (np.arange(n_tr) * h_step + 25).astype(np.float32)
    mid = np.full(n_tr, m, np.float32)
    if fill is None:
        smp = np.zeros((n_tr, S), np.float32)
    else:
        smp = np.full((n_tr, S), fill, np.float32)
    return smp, mid, hoff


def test_constant_traces_semblance_one_and_lowest_index_tie():
    # identical constant traces: every in-trace window gives u = A exactly, so
    # semblance = w*used^2*A^2 / (used*used*w*A^2) = 1 and stack = A for every
    # candidate -> all tie, the lowest index wins (strict '>' from -1)
    smp, mid, hoff = _line(fill=1.0)
    params = oracle.build_grid("cmp", [2000.0], [4000.0], [16])
    sel = np.arange(6, dtype=np.uint32)
    sem, stk, _ = oracle.ls_eval("cmp", smp, mid, hoff, sel, 1000.0, 0.004, 2, params)
    inner = sem[50:120]
    assert np.all(inner == 1.0)
    assert np.all(stk[50:120] == 1.0)
    idx = oracle.argmax(sem)
    assert np.all(idx[50:120] == 0)


def test_window_outside_trace_is_skipped():
    # t0 = 0 with tau = 2: k = 0 -> k - tau < 0, every trace skipped,
    # used = 0 -> semblance = stack = 0; the first candidate wins (0 > -1)
    smp, mid, hoff = _line(fill=1.0)
    hoff[:] = 0.0
    params = oracle.build_grid("cmp", [2000.0], [4000.0], [4])
    sem, stk, _ = oracle.ls_eval("cmp", smp, mid, hoff, np.arange(6, dtype=np.uint32),
                                 1000.0, 0.004, 2, params, precision="f64")
    assert np.all(sem[0] == 0) and np.all(stk[0] == 0)
    assert oracle.argmax(sem)[0] == 0
    # last samples: k + tau + 1 >= S -> skipped as well
    assert np.all(sem[-2:] == 0)


def test_ramp_interpolation_is_exact():
    # y[k] = k: linear interpolation is exact, and the symmetric window's mean
    # is tIndex, so stack = mean over traces of t_i / dt
    S, dt, tau = 300, 0.004, 3
    smp, mid, hoff = _line(n_tr=5, S=S)
    smp[:] = np.arange(S, dtype=np.float32)[None, :]
    v = 2500.0
    params = np.array([[4.0 / (v * v)]], np.float32)
    sem, stk, _ = oracle.ls_eval("cmp", smp, mid, hoff, np.arange(5, dtype=np.uint32),
                                 1000.0, dt, tau, params, precision="f64")
    s = 150
    t0 = float(np.float32(s)) * float(np.float32(dt))
    c = float(params[0, 0])
    tidx = np.sqrt(t0 * t0 + c * hoff.astype(np.float64) ** 2) / float(np.float32(dt))
    ok = (np.floor(tidx) >= tau) & (np.floor(tidx) + tau + 1 < S)
    assert abs(stk[s, 0] - tidx[ok].mean()) < 1e-9


def test_grid_order_and_steps():
    # ZO-CRS: velocity slowest, then A, B fastest (zocrs/linear_search.cu:21-23);
    # step = (U - L) / G so U is never reached
    lo, hi, g = [1500.0, -1e-3, -1e-7], [4500.0, 1e-3, 1e-7], [3, 4, 5]
    p = oracle.build_grid("zocrs", lo, hi, g)
    assert p.shape == (60, 3)
    f32 = np.float32
    for i in [0, 7, 23, 59]:
        iv, ia, ib = i // 20, (i // 5) % 4, i % 5
        steps = [f32((f32(hi[j]) - f32(lo[j])) / f32(g[j])) for j in range(3)]
        v = f32(np.float64(f32(lo[0])) + np.float64(f32(iv)) * np.float64(steps[0]))
        assert p[i, 0] == f32(f32(4.0) / f32(v * v))
        # min + idx*inc as one fused multiply-add (the reference's device code)
        assert p[i, 1] == f32(np.float64(f32(lo[1])) + np.float64(f32(ia)) * np.float64(steps[1]))
        assert p[i, 2] == f32(np.float64(f32(lo[2])) + np.float64(f32(ib)) * np.float64(steps[2]))
    v_last = f32(f32(lo[0]) + f32(2) * f32((f32(hi[0]) - f32(lo[0])) / f32(3)))
    assert v_last < hi[0]


def test_selection_rules():
    mid = np.array([975, 1000, 1000, 1025, 1375, 1376], np.float32)
    hoff = np.array([50, 25, 75, 50, 50, 50], np.float32)
    assert oracle.select("cmp", mid, hoff, 1000.0).tolist() == [0, 1, 1, 0, 0, 0]
    assert oracle.select("zocrs", mid, hoff, 1000.0, apm=375.0).tolist() == [1, 1, 1, 1, 1, 0]


def test_oct_displaced_midpoint_bound():
    # |mh - m0| <= sqrt(h^2 + h0^2): the engine's OCT prefilter relies on it.
    rng = np.random.default_rng(3)
    lo, hi = [1200.0, -1e-3], [5000.0, 1e-3]
    cands = oracle.oct_selection_candidates(lo, hi, 64)
    mid = np.full(1, 10000.0, np.float32)
    for h in [0.0, 10.0, 500.0, 3000.0]:
        for h0 in [0.0, 500.0, 1000.0]:
            far = float(np.sqrt(h * h + h0 * h0)) * 1.001 + 1.0
            # a trace just beyond apm + bound can never be selected
            m = np.float32(10000.0 + 20.0 + far + 0.5)
            sel = oracle.select("oct", np.array([m], np.float32), np.array([h], np.float32),
                                10000.0, apm=20.0, h0=h0, S=200, dt=0.004, cands=cands)
            assert not sel[0]


def test_fp32_matches_fp64_argmax_on_small_cmp_line():
    w = synthetic.WORKLOADS["cmp-small"]
    line = synthetic.cmp_line(n_cmp=2, halfoffsets=list(range(25, 1176, 50)), ns=1000,
                              dt_us=4000, n_reflectors=5, n_multiples=0, f=25.0, snr=10.0,
                              seed=1001)
    from parity import Report, compare_block
    params = oracle.build_grid("cmp", w.lower, w.upper, w.granularity)
    rep = Report()
    for m0 in line.cdp_midpoints:
        sel = np.nonzero(line.midpoints == m0)[0].astype(np.uint32)
        args = ("cmp", line.samples, line.midpoints, line.halfoffsets, sel, m0,
                float(line.dt), 2, params)
        s32, k32, _ = oracle.ls_eval(*args)
        s64, k64, _ = oracle.ls_eval(*args, precision="f64")
        got, _ = oracle.ls_result("cmp", s32, k32, params)
        rms = float(np.sqrt(np.mean(line.samples[sel] ** 2)))
        compare_block(rep, got, s64, k64, params, rms)
    rep.check()
    assert rep.mismatches <= 0.001 * rep.samples, rep.summary()


def test_oct_candidates_match_libstdcxx_restatement():
    c = oracle.oct_selection_candidates([450.0, -0.001], [6000.0, 0.001])
    # values printed by a std::default_random_engine / uniform_real_distribution
    # <float> program compiled with GCC 13's libstdc++
    assert np.float32(c[0, 0]) == np.float32(1.97492755e-05)
    assert np.float32(c[1023, 0]) == np.float32(1.48173527e-07)
    assert np.float32(c[0, 1]) == np.float32(-0.000258325541)
    assert np.float32(c[1023, 1]) == np.float32(-0.000674933894)


def test_inclusive_grid():
    """Inclusive grid: G values per parameter, both bounds included, the
    velocity uniform in c = 4/v^2 from 4/L^2 (index 0) to 4/U^2."""
    lo, hi, g = [1500.0, -1e-3, -1e-7], [6000.0, 1e-3, 1e-7], [41, 21, 21]
    p = oracle.build_grid("zocrs", lo, hi, g, "inclusive")
    assert p.shape == (41 * 21 * 21, 3)
    c = p[:: 21 * 21, 0]
    assert c[0] == np.float32(4.0) / np.float32(np.float32(1500.0) * np.float32(1500.0))
    assert c[-1] == np.float32(4.0) / np.float32(np.float32(6000.0) * np.float32(6000.0))
    np.testing.assert_allclose(np.diff(c), (c[-1] - c[0]) / 40, rtol=1e-4)
    a = p[:21 * 21:21, 1]
    assert a[0] == np.float32(-1e-3) and a[-1] == np.float32(1e-3)
    bb = p[:21, 2]
    assert bb[0] == np.float32(-1e-7) and bb[-1] == np.float32(1e-7)
    # G = 1: the lower bound only
    one = oracle.build_grid("cmp", [2000.0], [3000.0], [1], "inclusive")
    assert one.shape == (1, 1) and one[0, 0] == np.float32(4.0) / np.float32(4e6)
