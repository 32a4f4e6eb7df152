"""Differential evolution on the GPU, through the C ABI.

The random stream differs from the reference's (curand seeded from
time(NULL)), so DE is judged by what it finds: its best semblance against the
exhaustive-grid optimum of the same line, the reported semblance against the
oracle's evaluation of the reported parameters, and exact checks of the parts
that do not depend on the stream's values: the initial population (regenerated
by the oracle from the same counter-based stream), determinism per seed, the
bounds, and OCT trace selection from the initial population.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu


def _cmp_line():
    return synthetic.cmp_line(n_cmp=3, halfoffsets=list(range(25, 1176, 50)), ns=400,
                              dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0,
                              seed=31)


def _setup(eng, line, model, lower, upper, tau=2, apm=0.0, h0=0.0):
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    eng.set_traveltime(model, lower, upper, apm, h0)
    eng.set_window(tau)


def test_de_cmp_finds_grid_optimum(engine):
    line = _cmp_line()
    lower, upper = [1000.0], [5040.0]
    _setup(engine, line, "cmp", lower, upper)
    m0s = line.cdp_midpoints
    de, st = engine.differential_evolution(m0s, 32, 32, 0.85, 0.5, seed=1)
    assert st["evals"] == 3 * 24 * 400 * 32 * 32
    ls, _ = engine.linear_search(m0s, [404], "tuned")       # 10 m/s grid
    assert np.all((de[:, 2] >= 1000.0) & (de[:, 2] <= 5040.0))
    strong = ls[:, 0] > 0.1
    ratio = de[:, 0][strong] / ls[:, 0][strong]
    assert np.median(ratio) >= 0.99, np.median(ratio)
    assert np.mean(ratio) >= 0.95, np.mean(ratio)


def test_de_reported_semblance_is_the_parameters_semblance(engine):
    line = _cmp_line()
    _setup(engine, line, "cmp", [1000.0], [5040.0])
    m0s = line.cdp_midpoints
    de, _ = engine.differential_evolution(m0s, 16, 8, 0.85, 0.5, seed=5)
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(line.midpoints == m0)[0].astype(np.uint32)
        cands = de[i, 2:].T.reshape(-1, 1, 1)
        sem, stk = oracle.eval_raw("cmp", line.samples, line.midpoints, line.halfoffsets, sel,
                                   m0, float(line.dt), 2, cands, precision="f32")
        rel = np.abs(sem[:, 0] - de[i, 0]) / np.maximum(np.abs(sem[:, 0]), 1e-3)
        assert np.quantile(rel, 0.999) <= 2e-4


def test_de_single_generation_is_best_initial_individual(engine):
    line = _cmp_line()
    lower, upper = [1000.0], [5040.0]
    _setup(engine, line, "cmp", lower, upper)
    m0s = line.cdp_midpoints[:1]
    seed, pop = 77, 24
    de, _ = engine.differential_evolution(m0s, pop, 1, 0.85, 0.5, seed=seed)
    init = oracle.de_initial_population(seed, oracle.de_key(m0s[0]), line.samples_per_trace,
                                        pop, lower, upper)
    sel = np.nonzero(line.midpoints == m0s[0])[0].astype(np.uint32)
    sem, _ = oracle.eval_raw("cmp", line.samples, line.midpoints, line.halfoffsets, sel,
                             m0s[0], float(line.dt), 2, init, precision="f32")
    # the reported velocity is one of that sample's initial individuals, bit for bit
    S = line.samples_per_trace
    member = np.array([np.any(init[s, :, 0] == de[0, 2, s]) for s in range(S)])
    assert member.all()
    best = sem.max(axis=1)
    chosen = np.array([sem[s, np.nonzero(init[s, :, 0] == de[0, 2, s])[0][0]] for s in range(S)])
    assert np.all(np.abs(chosen - best) <= 1e-4 * np.maximum(best, 1e-3))


def test_de_is_deterministic_per_seed(engine):
    line = _cmp_line()
    _setup(engine, line, "cmp", [1000.0], [5040.0])
    m0s = line.cdp_midpoints
    a, _ = engine.differential_evolution(m0s, 16, 6, 0.5, 0.9, seed=11)
    b, _ = engine.differential_evolution(m0s, 16, 6, 0.5, 0.9, seed=11)
    c, _ = engine.differential_evolution(m0s, 16, 6, 0.5, 0.9, seed=12)
    assert np.array_equal(a, b)
    assert not np.array_equal(a, c)


@pytest.mark.parametrize("pop", [1, 48, 128])
def test_de_population_sizes(engine, pop):
    line = _cmp_line()
    _setup(engine, line, "cmp", [1000.0], [5040.0])
    de, _ = engine.differential_evolution(line.cdp_midpoints[:1], pop, 4, 0.5, 0.9, seed=3)
    assert np.all((de[0, 2] >= 1000.0) & (de[0, 2] <= 5040.0))
    assert np.all(np.isfinite(de))


def test_de_zocrs_small_line(engine):
    line = synthetic.structured_line(n_cmp=20, fold_range=(6, 10), h_max=1000, ns=300,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=41)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    lower, upper = [1414.2136, -a, -b], [6324.5553, a, b]
    _setup(engine, line, "zocrs", lower, upper, apm=125.0)
    m0s = line.cdp_midpoints[5:8]
    de, st = engine.differential_evolution(m0s, 32, 40, 0.5, 0.9, seed=2)
    for j in range(3):
        assert np.all((de[:, 2 + j] >= lower[j]) & (de[:, 2 + j] <= upper[j]))
    ls, _ = engine.linear_search(m0s, [21, 11, 11], "tuned")
    strong = ls[:, 0] > 0.1
    ratio = de[:, 0][strong] / ls[:, 0][strong]
    # DE searches the continuous box; the grid is coarse -- DE should match or beat it
    assert np.median(ratio) >= 0.97, np.median(ratio)


def test_de_oct_selection_from_initial_population(engine):
    """OCT DE selects a trace if any sample's initial individual reaches it
    (oct/differential_evolution.cu selectTraces...): the engine's count per
    midpoint equals the oracle's on the same initial population.  The device
    forms c = 4/v^2 with the fast-math division, so a trace whose test sits
    within rounding of the aperture may flip: a midpoint is well-conditioned
    when the oracle's count is unchanged with every velocity moved by
    +-5e-7 (c by ~1e-6, well above the division's error); those must match
    exactly, the others within one trace."""
    line = synthetic.structured_line(n_cmp=10, fold_range=(4, 8), h_max=800, ns=120,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=51)
    lower, upper = [1200.0, -1e-3], [5000.0, 1e-3]
    apm, h0, seed, pop = 50.0, 300.0, 9, 8
    _setup(engine, line, "oct", lower, upper, apm=apm, h0=h0)
    S = line.samples_per_trace
    exact = 0
    for m0 in line.cdp_midpoints[2:8]:
        de, st = engine.differential_evolution([m0], pop, 3, 0.5, 0.9, seed=seed)
        assert np.all(np.isfinite(de))
        init = oracle.de_initial_population(seed, oracle.de_key(m0), S, pop, lower, upper)
        counts = []
        for f in (1.0, 1.0 - 5e-7, 1.0 + 5e-7):
            pert = init.copy()
            pert[..., 0] = (pert[..., 0].astype(np.float64) * f).astype(np.float32)
            counts.append(int(oracle.select_oct_per_sample(
                line.midpoints, line.halfoffsets, m0, apm, h0, S, float(line.dt),
                pert).sum()))
        if len(set(counts)) == 1:
            assert st["selected_traces"] == counts[0], m0
            exact += 1
        else:
            assert abs(st["selected_traces"] - counts[0]) <= 1, m0
    assert exact >= 4


def test_de_multi_wave_call_maps_units_to_midpoints(engine):
    """A call with more (midpoint, sample group) units than resident CTAs
    takes them from the work queue, midpoints ordered by selected traces
    (uneven fold here); every unit must still work on its own midpoint: with
    one generation, every reported velocity is one of the initial individuals
    the counter-based stream gives that midpoint."""
    line = synthetic.structured_line(n_cmp=40, fold_range=(6, 20), h_max=1200, ns=400,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=33)
    lower, upper = [1000.0], [5040.0]
    _setup(engine, line, "cmp", lower, upper)
    m0s = line.cdp_midpoints
    assert m0s.size == 40
    seed, pop = 91, 16
    de, st = engine.differential_evolution(m0s, pop, 1, 0.85, 0.5, seed=seed)
    assert st["device_error"] == 0
    S = line.samples_per_trace
    for i in (0, 7, 23, 39):
        init = oracle.de_initial_population(seed, oracle.de_key(m0s[i]), S, pop, lower,
                                            upper)
        member = np.array([np.any(init[s, :, 0] == de[i, 2, s]) for s in range(S)])
        assert member.all(), i


@pytest.mark.parametrize("slope,h0", [(1e-3, 0.0), (5e-3, 0.0), (1e-3, 500.0), (5e-3, 1000.0)])
def test_de_oct_box_test_keeps_results(engine, monkeypatch, slope, h0):
    """OCT DE: warps drop traces by the displaced-midpoint box test (the
    range of their evaluations' t0 and slope, or theta and t0^2 - c h0^2)
    before the per-sample test.  Blocks and not-used counts equal those with
    the box test off (HPSS_OCT_BOX_TEST=0: every trace through the
    per-sample test)."""
    line = synthetic.structured_line(n_cmp=24, fold_range=(6, 12), h_max=2500, ns=400,
                                     dt_us=2000, n_reflectors=4, f=20.0, snr=8.0, seed=14)
    lower, upper = [1200.0, -slope], [5000.0, slope]
    _setup(engine, line, "oct", lower, upper, apm=150.0, h0=h0)
    m0s = line.cdp_midpoints[2::5]
    de, st = engine.differential_evolution(m0s, 32, 12, 0.5, 0.9, seed=4)
    monkeypatch.setenv("HPSS_OCT_BOX_TEST", "0")
    de0, st0 = engine.differential_evolution(m0s, 32, 12, 0.5, 0.9, seed=4)
    assert st["device_error"] == 0 and st0["device_error"] == 0
    assert st0["not_used"] > 0
    # the selection's per-sample box test keeps the selected traces
    assert st["selected_traces"] == st0["selected_traces"]
    assert st["not_used"] == st0["not_used"]
    assert np.array_equal(de, de0)


@pytest.mark.parametrize("model", ["cmp", "zocrs"])
@pytest.mark.parametrize("storage", ["fp32", "fp16", "bf16"])
@pytest.mark.parametrize("tau", [0, 2, 5])
def test_de_staged_spans_equal_unstaged(engine, monkeypatch, model, storage, tau):
    """CMP / ZO-CRS DE reads its windows from trace spans staged in shared
    memory (the spans any window of the CTA's trials can touch), two
    individuals per thread when the population is even (HPSS_DE_PAIRS=1);
    the results equal one individual per thread (HPSS_DE_PAIRS=0) and the
    evaluation through
    L1 (HPSS_DE_STAGED=0) bit for bit, with uneven fold (rounds of different
    trace counts), odd trace counts per round, windows at the trace ends,
    several sample groups per midpoint and populations 32, 48 and 7, and no
    device error."""
    line = synthetic.structured_line(n_cmp=14, fold_range=(5, 13), h_max=1100, ns=260,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=71)
    if model == "cmp":
        lower, upper, apm = [1000.0], [5040.0], 0.0
    else:
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, apm = [1414.2136, -a, -b], [6324.5553, a, b], 150.0
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)
    engine.set_traveltime(model, lower, upper, apm)
    engine.set_window(tau)
    m0s = line.cdp_midpoints[3:11]
    for pop in (32, 48, 7):
        runs = {}
        # default: staged spans, two individuals per thread for an even
        # population; then one per thread; then through L1
        for name, env in (("pairs", {"HPSS_DE_PAIRS": "1"}), ("single", {"HPSS_DE_PAIRS": "0"}),
                          ("l1", {"HPSS_DE_STAGED": "0"})):
            for k in ("HPSS_DE_PAIRS", "HPSS_DE_STAGED"):
                monkeypatch.delenv(k, raising=False)
            for k, v in env.items():
                monkeypatch.setenv(k, v)
            runs[name] = engine.differential_evolution(m0s, pop, 12, 0.5, 0.9, seed=5)
        for k in ("HPSS_DE_PAIRS", "HPSS_DE_STAGED"):
            monkeypatch.delenv(k, raising=False)
        want, st0 = runs["l1"]
        for name in ("pairs", "single"):
            got, st = runs[name]
            assert st["device_error"] == 0, (name, pop)
            assert np.array_equal(got, want), (name, pop)
