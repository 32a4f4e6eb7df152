"""16-bit amplitude storage (BF16; FP16 with a per-trace FP32 scale).

The line is resident in 16-bit rows only (half the bytes); the tuned kernel
widens the staged windows to FP32 in shared memory, the other kernels as
they read them; interpolation and all sums stay FP32.  Rounding the
amplitudes is a precision loss, so these modes are judged against the FP64
oracle: the fraction of samples whose chosen candidate differs (printed;
bounded here) and the error of the chosen semblance.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from oracle import oracle
from parity import assert_same_but_stack

pytestmark = pytest.mark.gpu

# storage -> (max fraction of changed chosen candidates, p99.9 rel. semblance error)
BOUNDS = {"fp32": (0.001, 2e-4), "fp16": (0.01, 2e-3), "bf16": (0.05, 2e-2)}


@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
def test_storage_modes_against_fp64(engine, storage):
    w = synthetic.WORKLOADS["cmp-small"]
    line = w.make_line()
    m0s = line.cdp_midpoints[:6]
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)
    engine.set_traveltime("cmp", w.lower, w.upper)
    engine.set_window(2)
    got, st = engine.linear_search(m0s, w.granularity, "tuned")
    assert st["device_error"] == 0
    ref, idx, _ = oracle.linear_search("cmp", line.samples, line.midpoints, line.halfoffsets, m0s,
                                       float(line.dt), 2, w.lower, w.upper, w.granularity,
                                       precision="f64")
    changed = float(np.mean(~np.isclose(got[:, 2], ref[:, 2], rtol=1e-5)))
    rel = np.abs(got[:, 0] - ref[:, 0]) / np.maximum(np.abs(ref[:, 0]), 1e-3)
    p999 = float(np.quantile(rel, 0.999))
    print(f"storage {storage}: changed chosen candidates {changed:.5f}, "
          f"semblance rel. error p99.9 {p999:.2e}")
    max_changed, max_err = BOUNDS[storage]
    assert changed <= max_changed
    assert p999 <= max_err
    # the plain kernel widens the same 16-bit rows (the line is resident in
    # one storage only): the same semblances and chosen parameters
    plain, _ = engine.linear_search(m0s, w.granularity, "plain")
    assert_same_but_stack(got, plain, 1)


@pytest.mark.parametrize("storage", ["bf16", "fp16"])
@pytest.mark.parametrize("model", ["cmp", "zocrs"])
def test_16bit_bulk_staging_equals_plain(engine, monkeypatch, storage, model):
    """16-bit rows reach the tuned kernel's stage by bulk copies of the raw
    spans (rounded to 8 samples), widened in place in shared memory: for
    every tuned shape, windows 3 / 7 / 11 (windows at the trace ends) and
    rows whose length is not a multiple of 8, the semblances and chosen
    parameters equal the plain kernel's on the same 16-bit rows, and no
    device error is reported."""
    line = synthetic.structured_line(n_cmp=14, fold_range=(6, 12), h_max=1000, ns=203,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=81)
    if model == "cmp":
        lower, upper, gran, apm = [1000.0], [5040.0], [37], 0.0
    else:
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, gran, apm = [1414.2136, -a, -b], [6324.5553, a, b], [5, 5, 5], 125.0
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)
    engine.set_traveltime(model, lower, upper, apm)
    m0s = line.cdp_midpoints[2:12]
    for tau in (1, 3, 5):
        engine.set_window(tau)
        plain, _ = engine.linear_search(m0s, gran, "plain")
        for variant in ("0", "1", "2"):
            monkeypatch.setenv("HPSS_LS_VARIANT", variant)
            got, st = engine.linear_search(m0s, gran, "tuned")
            assert st["device_error"] == 0
            assert st["kernel_variant"] == int(variant)
            assert_same_but_stack(got, plain, 1)
        monkeypatch.delenv("HPSS_LS_VARIANT", raising=False)
