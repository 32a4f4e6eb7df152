"""OCT over several target half-offsets in one call, and 16-bit amplitude
storage in the OCT, differential-evolution and stretch-free kernels.

The reference holds one h0 per OffsetContinuationTrajectory
(common/src/traveltime/OffsetContinuationTrajectory.cpp:5-25), so a job per
h0.  hpss_set_oct_half_offsets makes every OCT call run all of them in one
launch, result blocks h0-major; each block must equal the one-h0 call bit
for bit (the DE random stream is keyed by the midpoint's value).

With BF16 / FP16 storage the line is resident in 16-bit rows only and every
kernel widens the amplitudes as it reads them: the tuned and plain linear
searches then agree with each other exactly, and the results stay within the
storage's rounding of the FP32-storage results.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from parity import assert_same_but_stack

pytestmark = pytest.mark.gpu

H0S = [0.0, 500.0, 1000.0]
LOWER, UPPER = [1200.0, -1e-3], [5000.0, 1e-3]
APM, TAU = 150.0, 4  # window 9, as the OCT workload


def _line():
    return synthetic.structured_line(n_cmp=14, fold_range=(6, 10), h_max=1500, ns=300,
                                     dt_us=2000, n_reflectors=3, f=30.0, snr=8.0, seed=81,
                                     v0=1800.0, kz=0.5, kx=0.1)


def _setup(eng, line, h0=0.0, storage="fp32"):
    eng.set_oct_half_offsets([])
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                      storage=storage)
    eng.set_traveltime("oct", LOWER, UPPER, APM, h0)
    eng.set_window(TAU)


@pytest.mark.parametrize("kernel", ["tuned", "plain"])
def test_h0_batch_linear_search_equals_one_h0_calls(engine, kernel):
    line = _line()
    m0s = line.cdp_midpoints[4:7]
    singles, nu = [], 0.0
    for h0 in H0S:
        _setup(engine, line, h0)
        out, st = engine.linear_search(m0s, [9, 7], kernel)
        singles.append(out)
        nu += st["not_used"]
    _setup(engine, line, 123.0)  # the traveltime's own h0 is not used with a list
    engine.set_oct_half_offsets(H0S)
    counts = engine.select_traces(m0s)
    batch, st = engine.linear_search(m0s, [9, 7], kernel)
    engine.set_oct_half_offsets([])
    assert st["device_error"] == 0
    assert batch.shape == (len(H0S) * m0s.size, 4, line.samples_per_trace)
    assert np.array_equal(batch, np.concatenate(singles))
    assert st["not_used"] == nu
    want = []
    for h0 in H0S:
        _setup(engine, line, h0)
        want.append(engine.select_traces(m0s))
    assert np.array_equal(counts, np.concatenate(want))


def test_h0_batch_de_and_stretch_free_equal_one_h0_calls(engine):
    """The OCT DE workload's pipeline on a small line: DE over all h0 in one
    launch, then the stretch-free stack over the chosen parameters in one
    launch -- block for block the one-h0 calls' results."""
    line = _line()
    m0s = line.cdp_midpoints[5:7]
    S = line.samples_per_trace
    de1, sf1 = [], []
    for h0 in H0S:
        _setup(engine, line, h0)
        de, _ = engine.differential_evolution(m0s, 24, 10, 0.5, 0.9, seed=5)
        sf, _ = engine.stretch_free(m0s, np.ascontiguousarray(de[:, 2:]), 10)
        de1.append(de)
        sf1.append(sf)
    _setup(engine, line)
    engine.set_oct_half_offsets(H0S)
    de, st = engine.differential_evolution(m0s, 24, 10, 0.5, 0.9, seed=5)
    assert st["device_error"] == 0
    assert st["evals"] == pytest.approx(st["selected_traces"] * S * 24 * 10)
    sf, st2 = engine.stretch_free(m0s, np.ascontiguousarray(de[:, 2:]), 10)
    engine.set_oct_half_offsets([])
    assert np.array_equal(de, np.concatenate(de1))
    assert np.array_equal(sf, np.concatenate(sf1))
    assert st2["device_error"] == 0


def test_half_offset_list_arguments(engine):
    from highperformanceseismicstacking_gb300 import capi
    with pytest.raises(capi.HpssError):
        engine.set_oct_half_offsets([0.0] * 65)
    with pytest.raises(capi.HpssError):
        engine.set_oct_half_offsets([float("nan")])
    engine.set_oct_half_offsets([])


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_oct_and_de_read_16bit_storage(engine, storage):
    """16-bit storage: tuned and plain OCT searches read the same widened
    amplitudes (identical results); DE and stretch-free stay within the
    rounding of the amplitudes of their FP32-storage results."""
    from highperformanceseismicstacking_gb300 import capi
    line = _line()
    m0s = line.cdp_midpoints[4:8]
    _setup(engine, line, 500.0)
    ls32, _ = engine.linear_search(m0s, [9, 7], "tuned")
    de32, _ = engine.differential_evolution(m0s, 24, 12, 0.5, 0.9, seed=9)
    sf32, _ = engine.stretch_free(m0s, np.ascontiguousarray(de32[:, 2:]), 10)
    # the line is resident in one storage only: switching a handle to 16-bit
    # rows releases the FP32 rows (but for a bounded staging area)
    with capi.Engine(0) as fresh:
        fresh.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        b32 = fresh.device_bytes()
        fresh.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                            storage=storage)
        b16 = fresh.device_bytes()
    line_bytes = line.samples.shape[0] * ((line.samples.shape[1] + 7) // 8 * 8) * 4
    assert b32 - b16 >= line_bytes // 2 - 4096, (b32, b16, line_bytes)
    _setup(engine, line, 500.0, storage)
    ls16, st = engine.linear_search(m0s, [9, 7], "tuned")
    plain16, _ = engine.linear_search(m0s, [9, 7], "plain")
    assert st["device_error"] == 0
    assert np.array_equal(ls16, plain16)
    changed = float(np.mean(np.any(ls16[:, 2:] != ls32[:, 2:], axis=1)))
    rel = np.abs(ls16[:, 0] - ls32[:, 0]) / np.maximum(ls32[:, 0], 1e-3)
    tol = {"fp16": (0.02, 5e-3), "bf16": (0.10, 5e-2)}[storage]
    print(f"OCT LS {storage}: changed {changed:.4f}, semblance p99 {np.quantile(rel, 0.99):.2e}")
    assert changed <= tol[0]
    assert np.quantile(rel, 0.99) <= tol[1]
    de16, st = engine.differential_evolution(m0s, 24, 12, 0.5, 0.9, seed=9)
    assert st["device_error"] == 0
    strong = de32[:, 0] > 0.1
    ratio = float(np.median(de16[:, 0][strong] / de32[:, 0][strong]))
    print(f"OCT DE {storage}: median best-semblance ratio to FP32 storage {ratio:.4f}")
    assert abs(ratio - 1.0) <= tol[1] * 4
    sf16, _ = engine.stretch_free(m0s, np.ascontiguousarray(de32[:, 2:]), 10)
    rel = np.abs(sf16[:, 0] - sf32[:, 0]) / np.maximum(sf32[:, 0], 1e-3)
    assert np.quantile(rel, 0.99) <= tol[1]


@pytest.mark.parametrize("storage", ["fp16", "bf16"])
def test_cmp_zocrs_16bit_storage_tuned_equals_plain(engine, storage):
    """CMP / ZO-CRS with 16-bit storage: the tuned kernel's staging and the
    plain kernel widen the same way (semblance and parameters identical,
    stack within parity.STACK_REL); DE runs on the same rows."""
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    line = synthetic.structured_line(n_cmp=16, fold_range=(6, 10), h_max=1000, ns=300,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=82)
    engine.set_oct_half_offsets([])
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)
    engine.set_traveltime("zocrs", [1414.2136, -a, -b], [6324.5553, a, b], 125.0)
    engine.set_window(2)
    m0s = line.cdp_midpoints[5:9]
    tuned, st = engine.linear_search(m0s, [7, 5, 5], "tuned")
    plain, _ = engine.linear_search(m0s, [7, 5, 5], "plain")
    assert st["device_error"] == 0
    assert_same_but_stack(tuned, plain, 3)
    de, st = engine.differential_evolution(m0s, 16, 8, 0.5, 0.9, seed=3)
    assert st["device_error"] == 0 and np.all(np.isfinite(de))
