"""Every step in FP64 (hpss_set_precision HPSS_PREC_FP64) and the agreement
of the FP32 modes with it.

The FP64 search is the FP64 reference of the agreement measurement (the
host oracle cannot evaluate 10^4 samples of the 21 x 21 x 41 ZO-CRS grid in
reasonable time), so it is pinned first: against the host oracle's FP64
evaluation on small cases of all three models.  The engine's candidate grid
holds the device's fast-math 4/v^2 (the reference's grid, within one FP32
ulp of the IEEE quotient the oracle's grid holds), so the two evaluate
candidates up to 1.2e-7 apart: semblances agree within 1e-5 relative, and the
chosen candidate is the oracle's wherever the oracle's two best are not
within 1e-5 of each other.  The FP64 stretch-free pass, which recomputes
4/v^2 from the given velocities in FP64, matches the oracle's to the
rounding of its FP32 output.

Then, on every sample of one midpoint of the ZO-CRS workload line at the
full grid, each FP32 mode must choose the FP64 reference's candidate on
>= 99.9 % of the samples, near-ties (another candidate within 1e-4 x
max(best, 1e-3) of the FP64 best, as the FP64 semblances show) counted
apart.  BF16 storage (8 significant bits) is reported, not held to the bar.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from highperformanceseismicstacking_gb300.su import tau_index
from oracle import oracle
from parity import chosen_index

pytestmark = pytest.mark.gpu


def _cases():
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    return {
        "cmp": (synthetic.cmp_line(n_cmp=3, halfoffsets=list(range(25, 1176, 50)), ns=300,
                                   dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0,
                                   seed=91), [1000.0], [5040.0], [41], 0.0, 0.0),
        "zocrs": (synthetic.structured_line(n_cmp=12, fold_range=(6, 10), h_max=1000, ns=200,
                                            dt_us=4000, n_reflectors=3, f=20.0, snr=5.0,
                                            seed=92),
                  [1414.2136, -a, -b], [6324.5553, a, b], [7, 5, 5], 125.0, 0.0),
        "oct": (synthetic.structured_line(n_cmp=10, fold_range=(4, 8), h_max=800, ns=200,
                                          dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=93),
                [1200.0, -1e-3], [5000.0, 1e-3], [8, 5], 60.0, 500.0),
    }


@pytest.mark.parametrize("model", ["cmp", "zocrs", "oct"])
def test_fp64_search_matches_fp64_oracle(engine, model):
    line, lower, upper, gran, apm, h0 = _cases()[model]
    tau = 2
    m0s = line.cdp_midpoints[len(line.cdp_midpoints) // 2:][:2]
    engine.set_oct_half_offsets([])
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime(model, lower, upper, apm, h0)
    engine.set_window(tau)
    try:
        engine.set_precision(fp64=True)
        got, st = engine.linear_search(m0s, gran, "tuned")  # FP64 whatever is asked
    finally:
        engine.set_precision()
    assert st["device_error"] == 0 and st["kernel_variant"] == -1
    params = oracle.build_grid(model, lower, upper, gran)
    cands = oracle.oct_selection_candidates(lower, upper) if model == "oct" else None
    S = line.samples_per_trace
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(oracle.select(model, line.midpoints, line.halfoffsets, m0, apm, h0, S,
                                       float(line.dt), cands))[0].astype(np.uint32)
        sem, stk, _ = oracle.ls_eval(model, line.samples, line.midpoints, line.halfoffsets, sel,
                                     float(m0), float(line.dt), tau, params, apm, h0,
                                     precision="f64")
        ref, idx = oracle.ls_result(model, sem, stk, params)
        top = np.sort(sem, axis=1)[:, -2:]
        tied = (top[:, 1] - top[:, 0]) <= 1e-5 * np.maximum(top[:, 1], 1e-3)
        same = chosen_index(params, got[i]) == idx
        assert np.all(same | tied), np.nonzero(~(same | tied))[0][:10]
        np.testing.assert_allclose(got[i, 0], ref[0], rtol=1e-5, atol=1e-9)
        np.testing.assert_allclose(got[i, 1][same], ref[1][same], rtol=1e-4, atol=1e-6)


@pytest.mark.parametrize("model", ["cmp", "zocrs", "oct"])
def test_fp64_stretch_free_matches_fp64_oracle(engine, model):
    line, lower, upper, gran, apm, h0 = _cases()[model]
    tau, nmax = 2, 6
    m0s = line.cdp_midpoints[len(line.cdp_midpoints) // 2:][:2]
    engine.set_oct_half_offsets([])
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime(model, lower, upper, apm, h0)
    engine.set_window(tau)
    ls, _ = engine.linear_search(m0s, gran, "tuned")
    prior = np.ascontiguousarray(ls[:, 2:])
    try:
        engine.set_precision(fp64=True)
        got, st = engine.stretch_free(m0s, prior, nmax)
    finally:
        engine.set_precision()
    assert st["device_error"] == 0
    S = line.samples_per_trace
    for i, m0 in enumerate(m0s):
        if model == "oct":
            init = np.stack([prior[i, 0], prior[i, 1]], axis=1)[:, None, :]
            sel = np.nonzero(oracle.select_oct_per_sample(line.midpoints, line.halfoffsets, m0,
                                                          apm, h0, S, float(line.dt), init))[0]
        else:
            sel = np.nonzero(oracle.select(model, line.midpoints, line.halfoffsets, m0, apm))[0]
        sem, _, _ = oracle.sf_eval(model, line.samples, line.midpoints, line.halfoffsets,
                                   sel.astype(np.uint32), m0, float(line.dt), tau, prior[i],
                                   nmax, apm, h0, precision="f64")
        idx = oracle.argmax(sem)
        best = sem[np.arange(S), idx]
        np.testing.assert_allclose(got[i, 0], best, rtol=2e-7, atol=1e-12)
        top = np.sort(sem, axis=1)[:, -2:]
        tied = (top[:, 1] - top[:, 0]) <= 1e-9 * np.maximum(top[:, 1], 1e-3)
        assert np.all((got[i, 2] == idx - nmax) | tied)


def test_fp32_modes_agree_with_fp64_on_the_zocrs_grid(engine):
    """One midpoint of the ZO-CRS workload line (fold U{30..90}, +-15-CMP
    aperture, 1500 samples), the full 21 x 21 x 41 grid, window 5."""
    w = synthetic.WORKLOADS["zocrs-ls"]
    line = w.make_line(n_cmp=64)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    m0s = line.cdp_midpoints[32:33]
    engine.set_oct_half_offsets([])
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("zocrs", lower, upper, w.apm)
    engine.set_window(tau)

    def semb64(params):
        out, _ = engine.stretch_free(m0s, np.ascontiguousarray(params), 0)
        return out[:, 0].astype(np.float64)

    outs = {}
    try:
        engine.set_precision(fp64=True)
        ref, st = engine.linear_search(m0s, w.granularity, "plain")
        s_best = semb64(ref[:, 2:])
        for name, kw in {"fp32": {}, "fp64-traveltime": {"fp64_traveltime": True},
                         "compensated": {"compensated": True}}.items():
            engine.set_precision(**kw)
            outs[name], _ = engine.linear_search(m0s, w.granularity, "tuned")
        engine.set_precision()
        for storage in ("fp16", "bf16"):
            engine.upload_gather(line.samples, line.midpoints, line.halfoffsets,
                                 float(line.dt), storage=storage)
            outs[storage], _ = engine.linear_search(m0s, w.granularity, "tuned")
        engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        engine.set_precision(fp64=True)
        report = {}
        for name, got in outs.items():
            diff = np.any(got[:, 2:] != ref[:, 2:], axis=1)
            near = 0
            if diff.any():
                s_alt = semb64(got[:, 2:])
                near = int(np.sum(diff & (s_alt >= s_best - 1e-4 * np.maximum(s_best, 1e-3))))
            report[name] = ((int(diff.sum()) - near) / diff.size, near / diff.size)
    finally:
        engine.set_precision()
    for name, (changed, near) in report.items():
        print(f"{name}: changed vs FP64 {changed:.5f}, near-ties {near:.5f}")
    for name in ("fp32", "fp64-traveltime", "compensated", "fp16"):
        assert report[name][0] <= 1e-3, (name, report)
