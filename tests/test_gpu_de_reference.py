"""Differential evolution against the reference's own DE (its CUDA kernels,
built from the reference sources by oracle/build_ref.py, replayed by
oracle/ref_runner.py with F = 0.5, CR = 0.9).

The two random streams differ (curand XORWOW vs the engine's Philox), so the
comparison is statistical, as the DE workloads ask: per (m0, t0) sample, the
engine's best semblance (median over seeds) against the reference DE's median
over 16 seeds, both against the exhaustive-grid optimum of the same line.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from oracle import ref_runner

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not ref_runner.available(),
                                 reason="reference kernels not built (oracle/build_ref.py)")]

SEEDS = 16
F, CR = 0.5, 0.9
OPS = "common_differential_evolution_f05cr09"


@pytest.fixture(scope="module")
def rk():
    if not (ref_runner.REF_DIR / f"{OPS}.fatbin").exists():
        pytest.skip("F/CR shim of the reference DE operators not built")
    return ref_runner.ReferenceKernels()


def _compare(name, ours, ref, grid):
    """ours, ref: [seeds][nM0][S] best semblances; grid: [nM0][S] optimum."""
    o = np.median(ours, axis=0).ravel()
    r = np.median(ref, axis=0).ravel()
    g = grid.ravel()
    strong = g > 0.1
    diff = o[strong] - r[strong]
    print(f"{name}: samples {strong.sum()}, engine/grid median {np.median(o[strong] / g[strong]):.4f}"
          f", reference/grid median {np.median(r[strong] / g[strong]):.4f}, "
          f"engine/reference median {np.median(o[strong] / r[strong]):.4f}, "
          f"mean(engine - reference) {diff.mean():+.5f}, "
          f"engine below reference by > 0.05: {np.mean(diff < -0.05):.4f}, "
          f"above by > 0.05: {np.mean(diff > 0.05):.4f}")
    return o[strong], r[strong], g[strong]


def _assert_no_worse(o, r):
    """The engine's DE finds what the reference's does: medians over 16 seeds
    agree, and the engine is far (> 0.05) below the reference on at most 2 %
    of the samples, or no more often than it is far above it (+1 %): a
    16-seed median still scatters on a rugged landscape, in both directions."""
    assert np.median(o / r) >= 0.99
    assert np.mean(o - r) >= -0.01
    below, above = np.mean(o - r < -0.05), np.mean(o - r > 0.05)
    assert below <= 0.02 or below <= above + 0.01, (below, above)


def test_de_cmp_vs_reference_de_16_seeds(engine, rk):
    line = synthetic.cmp_line(n_cmp=3, halfoffsets=list(range(25, 1176, 50)), ns=400,
                              dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0,
                              seed=41)
    lower, upper = [1000.0], [5040.0]
    pop, gens, tau = 32, 60, 2
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("cmp", lower, upper)
    engine.set_window(tau)
    m0s = line.cdp_midpoints
    grid, _ = engine.linear_search(m0s, [404], "tuned")
    ours = np.stack([engine.differential_evolution(m0s, pop, gens, F, CR, seed=1000 + k)[0][:, 0]
                     for k in range(SEEDS)])
    ref = np.zeros_like(ours)
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(line.midpoints == m0)[0]
        for k in range(SEEDS):
            res, _, _ = rk.differential_evolution_midpoint(
                "cmp", line.samples, line.midpoints, line.halfoffsets, float(m0),
                float(line.dt), tau, lower, upper, pop, gens, seed=77 + k, sel=sel,
                operators=OPS)
            ref[k, i] = res[0]
            assert np.all((res[2] >= 1000.0) & (res[2] <= 5040.0))
    o, r, g = _compare("cmp", ours, ref, grid[:, 0])
    _assert_no_worse(o, r)


def test_de_zocrs_vs_reference_de_16_seeds(engine, rk):
    line = synthetic.structured_line(n_cmp=20, fold_range=(8, 14), h_max=1000, ns=250,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=42)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    lower, upper = [1414.2136, -a, -b], [6324.5553, a, b]
    # the ZO-CRS DE workload's population and generations
    apm, tau, pop, gens = 125.0, 2, 32, 60
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("zocrs", lower, upper, apm)
    engine.set_window(tau)
    m0s = line.cdp_midpoints[8:11]
    grid, _ = engine.linear_search(m0s, [11, 11, 11], "tuned")
    ours = np.stack([engine.differential_evolution(m0s, pop, gens, F, CR, seed=2000 + k)[0][:, 0]
                     for k in range(SEEDS)])
    ref = np.zeros_like(ours)
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(np.abs(np.float32(m0) - line.midpoints) <= np.float32(apm))[0]
        for k in range(SEEDS):
            res, _, _ = rk.differential_evolution_midpoint(
                "zocrs", line.samples, line.midpoints, line.halfoffsets, float(m0),
                float(line.dt), tau, lower, upper, pop, gens, seed=99 + k, apm=apm, sel=sel,
                operators=OPS)
            ref[k, i] = res[0]
    o, r, g = _compare("zocrs", ours, ref, grid[:, 0])
    _assert_no_worse(o, r)


@pytest.mark.parametrize("h0", [0.0, 500.0])
def test_de_oct_vs_reference_de_16_seeds(engine, rk, h0):
    """OCT DE (the OCT DE workload's population 48 and 80 generations, slope
    within +-1e-3 s/m) against the reference's OCT DE kernels
    (oct/differential_evolution.cu:4-128, its own trace selection on the
    initial population), medians over 16 seeds."""
    line = synthetic.structured_line(n_cmp=10, fold_range=(6, 10), h_max=1200, ns=250,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=43)
    lower, upper = [1200.0, -1e-3], [5000.0, 1e-3]
    apm, tau, pop, gens = 60.0, 2, 48, 80
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("oct", lower, upper, apm, h0)
    engine.set_window(tau)
    m0s = line.cdp_midpoints[3:7]
    grid, _ = engine.linear_search(m0s, [40, 21], "tuned")
    ours = np.stack([engine.differential_evolution(m0s, pop, gens, F, CR, seed=3000 + k)[0][:, 0]
                     for k in range(SEEDS)])
    ref = np.zeros_like(ours)
    for i, m0 in enumerate(m0s):
        for k in range(SEEDS):
            res, _, _ = rk.differential_evolution_midpoint(
                "oct", line.samples, line.midpoints, line.halfoffsets, float(m0),
                float(line.dt), tau, lower, upper, pop, gens, seed=123 + k, apm=apm, h0=h0,
                operators=OPS)
            ref[k, i] = res[0]
            assert np.all((res[3] >= -1e-3) & (res[3] <= 1e-3))
    o, r, g = _compare(f"oct h0={h0:g}", ours, ref, grid[:, 0])
    assert o.size > 50
    _assert_no_worse(o, r)
