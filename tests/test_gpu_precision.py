"""Precision modes of the linear search (hpss_set_precision): FP64 traveltime
and compensated window sums, judged against the FP64 oracle on the ZO-CRS
workload's geometry (~1900 traces per midpoint, window 5: about 9500 window
x trace terms, above the 4096 at which the compensated sums switch on).

Reported per mode and kernel family: the fraction of samples whose chosen
parameters differ from the FP64 oracle's, and the p99.9 relative error of
the chosen semblance.  Bounds: no mode is worse than the reference's FP32
arithmetic; the FP64 traveltime is closer to FP64 on ZO-CRS and OCT (the
tuned kernels' FP64 traveltime gives the plain kernel's results); the
compensated sums are much closer to FP64 where summation error dominates (a
gather with a large constant amplitude) -- per term in the plain kernel,
per staging round in the tuned kernel.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from highperformanceseismicstacking_gb300.su import tau_index
from oracle import oracle
from parity import assert_same_but_stack

pytestmark = pytest.mark.gpu

MODES = {"fp32": (False, False), "fp64-traveltime": (True, False),
         "compensated": (False, True), "both": (True, True)}


@pytest.fixture(scope="module")
def zocrs_case():
    w = synthetic.WORKLOADS["zocrs-ls"]
    line = w.make_line(n_cmp=120)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    m0s = line.cdp_midpoints[59:61]
    gran = [5, 5, 9]
    ref, _, counts = oracle.linear_search("zocrs", line.samples, line.midpoints,
                                          line.halfoffsets, m0s, float(line.dt), tau, lower,
                                          upper, gran, w.apm, precision="f64")
    return w, line, lower, upper, tau, m0s, gran, ref, counts


def _score(got, ref):
    changed = float(np.mean(np.any(~np.isclose(got[:, 2:], ref[:, 2:], rtol=1e-6), axis=1)))
    rel = np.abs(got[:, 0] - ref[:, 0]) / np.maximum(np.abs(ref[:, 0]), 1e-3)
    return changed, float(np.quantile(rel, 0.999))


def test_precision_modes_against_fp64(engine, zocrs_case):
    w, line, lower, upper, tau, m0s, gran, ref, counts = zocrs_case
    assert np.all(counts * (2 * tau + 1) > 4096)
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("zocrs", lower, upper, w.apm)
    engine.set_window(tau)
    scores = {}
    try:
        for name, (tt64, comp) in MODES.items():
            engine.set_precision(tt64, comp)
            got, st = engine.linear_search(m0s, gran, "plain")
            assert st["device_error"] == 0
            scores[name] = _score(got, ref)
            tuned, st_t = engine.linear_search(m0s, gran, "tuned")
            assert st_t["device_error"] == 0
            scores[name + " (tuned)"] = _score(tuned, ref)
            if name != "fp32":
                # the tuned kernel's precision instantiations (fixed shape)
                assert st_t["kernel_variant"] == 1
            if not comp:
                # same traveltime arithmetic, same window sums
                assert_same_but_stack(tuned, got, 3)
    finally:
        engine.set_precision(False, False)
    for name, (changed, p999) in scores.items():
        print(f"precision {name}: chosen parameters changed vs FP64 {changed:.5f}, "
              f"semblance rel. error p99.9 {p999:.2e}")
    fp32_changed, fp32_err = scores["fp32"]
    for name in ("fp64-traveltime", "compensated", "both"):
        for k in (name, name + " (tuned)"):
            assert scores[k][0] <= fp32_changed + 0.002, (k, scores)
    # on this line the FP32 error is the traveltime's: FP64 traveltime helps,
    # compensated sums neither help nor hurt (see the DC-heavy case below)
    assert scores["fp64-traveltime"][1] <= fp32_err, scores
    assert scores["compensated"][1] <= 1.05 * fp32_err, scores


def test_compensated_sums_on_large_dc_gather(engine):
    """A CMP gather of 1600 traces of amplitude ~1000 with a small signal:
    the FP32 sums of 1600 x 5 terms lose ~N eps relative; the compensated
    sums stay at ~eps (semblance against the FP64 oracle)."""
    rng = np.random.default_rng(3)
    n, S, dt = 1600, 300, 0.004
    mid = np.full(n, 5000.0, np.float32)
    hoff = np.sort(rng.uniform(0, 1500, n)).astype(np.float32)
    t = np.arange(S) * dt
    base = 1000.0 + 0.5 * np.sin(2 * np.pi * 7.0 * t)
    smp = (base[None, :] + 0.01 * rng.standard_normal((n, S))).astype(np.float32)
    lower, upper, gran, tau = [1500.0], [4500.0], [6], 2
    engine.upload_gather(smp, mid, hoff, dt)
    engine.set_traveltime("cmp", lower, upper)
    engine.set_window(tau)
    ref, _, _ = oracle.linear_search("cmp", smp, mid, hoff, [5000.0], dt, tau, lower, upper,
                                     gran, precision="f64")
    try:
        fp32, _ = engine.linear_search([5000.0], gran, "plain")
        engine.set_precision(False, True)
        comp, _ = engine.linear_search([5000.0], gran, "plain")
        comp_t, st = engine.linear_search([5000.0], gran, "tuned")
        assert st["kernel_variant"] == 1 and st["device_error"] == 0
    finally:
        engine.set_precision(False, False)
    live = ref[0, 0] > 0.5
    e32 = np.abs(fp32[0, 0][live] - ref[0, 0][live]) / ref[0, 0][live]
    ec = np.abs(comp[0, 0][live] - ref[0, 0][live]) / ref[0, 0][live]
    et = np.abs(comp_t[0, 0][live] - ref[0, 0][live]) / ref[0, 0][live]
    print(f"DC-heavy gather: semblance rel. error vs FP64, FP32 sums median {np.median(e32):.2e} "
          f"max {e32.max():.2e}; compensated (plain, per term) median {np.median(ec):.2e} "
          f"max {ec.max():.2e}; compensated (tuned, per staging round) median "
          f"{np.median(et):.2e} max {et.max():.2e}")
    assert np.median(ec) < 0.1 * np.median(e32)
    # rounds of a few tens of traces summed plainly, the rounds compensated
    assert np.median(et) < 0.3 * np.median(e32)


def test_precision_oct_fp64_traveltime(engine):
    line = synthetic.structured_line(n_cmp=16, fold_range=(4, 8), h_max=800, ns=200,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=12)
    lower, upper, gran = [1200.0, -1e-3], [5000.0, 1e-3], [6, 5]
    apm, tau, h0 = 60.0, 2, 300.0
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("oct", lower, upper, apm, h0)
    engine.set_window(tau)
    m0s = line.cdp_midpoints[::4]
    cands = oracle.oct_selection_candidates(lower, upper)
    ref, _, _ = oracle.linear_search("oct", line.samples, line.midpoints, line.halfoffsets, m0s,
                                     float(line.dt), tau, lower, upper, gran, apm, h0,
                                     precision="f64", oct_cands=cands)
    try:
        fp32, _ = engine.linear_search(m0s, gran, "plain")
        engine.set_precision(True, False)
        f64, st = engine.linear_search(m0s, gran, "plain")
        f64t, st_t = engine.linear_search(m0s, gran, "tuned")
    finally:
        engine.set_precision(False, False)
    assert st["device_error"] == 0 and st_t["device_error"] == 0
    # the OCT kernel's FP64 traveltime: the plain kernel's results bit for bit
    assert np.array_equal(f64t, f64)
    assert st_t["not_used"] == st["not_used"]
    a, b = _score(fp32, ref), _score(f64, ref)
    print(f"OCT fp32 {a}, fp64 traveltime {b}")
    assert b[0] <= a[0] + 0.002
    with pytest.raises(Exception):
        engine._check(engine._lib.hpss_set_precision(engine.h, 16))
