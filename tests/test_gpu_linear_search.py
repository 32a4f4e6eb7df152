"""Linear-search parity on the GPU, through the C ABI.

* plain kernel vs the oracle (FP32 restatement, IEEE): semblance and stack
  within tolerance, chosen candidate identical except near-ties (counted);
* tuned_exact kernel vs plain kernel: identical bits (same per-candidate
  arithmetic, same trace order); tuned kernel: semblance and chosen
  parameters identical, stack within parity.STACK_REL (its linear sum is the
  sum of the per-tap sums);
* FP64 oracle: chosen parameters agree on >= 99.9% of samples;
* edge cases the reference has: no selected trace, windows at the trace
  edges, window sizes 1..15, constant traces (semblance exactly 1, lowest
  index wins ties), argument errors.
"""
import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import capi, synthetic
from oracle import oracle
from parity import Report, assert_same_but_stack, compare_block, count_near_ties

pytestmark = pytest.mark.gpu


def _setup(eng, line, model, lower, upper, tau, apm=0.0, h0=0.0):
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    eng.set_traveltime(model, lower, upper, apm, h0)
    eng.set_window(tau)


def _check_against_oracle(model, line, m0s, got, lower, upper, gran, tau, apm=0.0, h0=0.0,
                          cands=None, precision="f32", grid_mode="reference"):
    """Engine blocks vs the oracle for every midpoint; tolerances in parity.py."""
    params = oracle.build_grid(model, lower, upper, gran, grid_mode)
    S = line.samples_per_trace
    rep = Report()
    for i, m0 in enumerate(m0s):
        mask = oracle.select(model, line.midpoints, line.halfoffsets, m0, apm, h0, S,
                             float(line.dt), cands)
        sel = np.nonzero(mask)[0].astype(np.uint32)
        if sel.size == 0:
            assert np.all(got[i] == 0)
            continue
        sem, stk, _ = oracle.ls_eval(model, line.samples, line.midpoints, line.halfoffsets,
                                     sel, m0, float(line.dt), tau, params, apm, h0,
                                     precision=precision)
        rms = float(np.sqrt(np.mean(line.samples[sel] ** 2)))
        compare_block(rep, got[i], sem, stk, params, rms)
    rep.check()
    return rep


@pytest.fixture(scope="module")
def c1_line():
    return synthetic.WORKLOADS["cmp-small"].make_line()


def test_cmp_small_line_plain_vs_oracle_and_tuned(engine, c1_line):
    w = synthetic.WORKLOADS["cmp-small"]
    tau = 2
    _setup(engine, c1_line, "cmp", w.lower, w.upper, tau)
    m0s = np.concatenate([c1_line.cdp_midpoints, [np.float32(12345.0)]])
    plain, st_p = engine.linear_search(m0s, w.granularity, "plain")
    tuned, st_t = engine.linear_search(m0s, w.granularity, "tuned")
    exact, st_e = engine.linear_search(m0s, w.granularity, "tuned_exact")
    assert st_t["device_error"] == 0 and st_p["device_error"] == 0 and st_e["device_error"] == 0
    assert np.array_equal(plain, exact)
    assert_same_but_stack(tuned, plain, 1)
    # identical semblances: identical near-tie counts
    assert st_p["near_ties"] == st_t["near_ties"] == st_e["near_ties"]
    print(f"cmp-small near-ties: {st_p['near_ties']:.0f} of {plain.shape[0] * plain.shape[2]}")
    assert np.all(plain[-1] == 0)          # midpoint without traces: zeros
    assert st_p["evals"] == 50 * 24 * 1000 * 101
    _check_against_oracle("cmp", c1_line, m0s, plain, w.lower, w.upper, w.granularity, tau)


@pytest.mark.parametrize("tau", [0, 1, 3, 5, 7])
def test_cmp_window_sizes_tuned_equals_plain(engine, c1_line, tau):
    w = synthetic.WORKLOADS["cmp-small"]
    _setup(engine, c1_line, "cmp", w.lower, w.upper, tau)
    m0s = c1_line.cdp_midpoints[:6]
    plain, _ = engine.linear_search(m0s, w.granularity, "plain")
    tuned, st = engine.linear_search(m0s, w.granularity, "tuned")
    exact, st_e = engine.linear_search(m0s, w.granularity, "tuned_exact")
    assert st["device_error"] == 0 and st_e["device_error"] == 0
    assert np.array_equal(plain, exact)
    assert_same_but_stack(tuned, plain, 1)


def test_cmp_fp64_oracle_agreement(engine, c1_line):
    w = synthetic.WORKLOADS["cmp-small"]
    _setup(engine, c1_line, "cmp", w.lower, w.upper, 2)
    m0s = c1_line.cdp_midpoints[:5]
    got, _ = engine.linear_search(m0s, w.granularity, "tuned")
    rep = _check_against_oracle("cmp", c1_line, m0s, got, w.lower, w.upper, w.granularity, 2,
                                precision="f64")
    # chosen parameters agree with the FP64 oracle on >= 99.9% of samples
    assert rep.mismatches <= 0.001 * rep.samples, rep.summary()


def test_constant_traces_known_answer(engine):
    S, n = 256, 8
    mid = np.full(n, 2000.0, np.float32)
    hoff = (np.arange(n) * 100 + 50).astype(np.float32)
    smp = np.ones((n, S), np.float32)
    engine.upload_gather(smp, mid, hoff, 0.004)
    engine.set_traveltime("cmp", [2000.0], [4000.0])
    engine.set_window(2)
    sem, _, _ = oracle.ls_eval("cmp", smp, mid, hoff, np.arange(n, dtype=np.uint32), 2000.0,
                               0.004, 2, oracle.build_grid("cmp", [2000.0], [4000.0], [16]))
    ties = count_near_ties(sem)
    assert ties > 0
    for k in ("plain", "tuned", "tuned_exact"):
        out, st = engine.linear_search([2000.0], [16], k)
        # every candidate whose windows fit gives semblance exactly 1: near-ties
        assert st["near_ties"] == ties, (k, st["near_ties"], ties)
        # mid-trace samples: semblance exactly 1, stack 1, lowest index (v = 2000)
        assert np.all(out[0, 0, 60:150] == 1.0)
        assert np.all(out[0, 1, 60:150] == 1.0)
        np.testing.assert_allclose(out[0, 2, 60:150], 2000.0, rtol=1e-6)
        # last samples: t >= t0, so every window ends past the trace -> used = 0,
        # semblance = stack = 0 and the first candidate is reported
        assert np.all(out[0, 0, -3:] == 0.0) and np.all(out[0, 1, -3:] == 0.0)
        np.testing.assert_allclose(out[0, 2, -3:], 2000.0, rtol=1e-6)


def test_zocrs_small_line(engine):
    line = synthetic.structured_line(n_cmp=30, fold_range=(8, 14), h_max=1000, ns=300,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=11)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    lower, upper, gran = [1414.2136, -a, -b], [6324.5553, a, b], [5, 5, 5]
    apm, tau = 125.0, 2
    _setup(engine, line, "zocrs", lower, upper, tau, apm)
    m0s = line.cdp_midpoints[::3]
    plain, st_p = engine.linear_search(m0s, gran, "plain")
    tuned, st_t = engine.linear_search(m0s, gran, "tuned")
    exact, st_e = engine.linear_search(m0s, gran, "tuned_exact")
    assert st_t["device_error"] == 0 and st_e["device_error"] == 0
    assert np.array_equal(plain, exact)
    assert_same_but_stack(tuned, plain, 3)
    counts = engine.select_traces(m0s)
    for i, m0 in enumerate(m0s):
        assert counts[i] == oracle.select("zocrs", line.midpoints, line.halfoffsets, m0,
                                          apm).sum()
    _check_against_oracle("zocrs", line, m0s, plain, lower, upper, gran, tau, apm)


@pytest.mark.parametrize("h0", [0.0, 300.0])
def test_oct_small_line(engine, h0):
    line = synthetic.structured_line(n_cmp=16, fold_range=(4, 8), h_max=800, ns=200,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=12)
    lower, upper, gran = [1200.0, -1e-3], [5000.0, 1e-3], [6, 5]
    apm, tau = 60.0, 2
    _setup(engine, line, "oct", lower, upper, tau, apm, h0)
    m0s = line.cdp_midpoints[::4]
    cands = oracle.oct_selection_candidates(lower, upper)
    counts = engine.select_traces(m0s)
    for i, m0 in enumerate(m0s):
        assert counts[i] == oracle.select("oct", line.midpoints, line.halfoffsets, m0, apm, h0,
                                          line.samples_per_trace, float(line.dt), cands).sum()
    plain, st_p = engine.linear_search(m0s, gran, "plain")
    tuned, st_t = engine.linear_search(m0s, gran, "tuned")
    assert st_t["device_error"] == 0
    assert np.array_equal(plain, tuned)
    assert st_p["not_used"] == st_t["not_used"]
    _check_against_oracle("oct", line, m0s, plain, lower, upper, gran, tau, apm, h0, cands)


@pytest.mark.parametrize("slope,dt_us,h0", [(5e-3, 2000, 0.0), (2e-4, 1000, 0.0),
                                             (2e-2, 4000, 0.0), (5e-3, 2000, 500.0),
                                             (1e-3, 1000, 1000.0), (2e-2, 4000, 0.5)])
def test_oct_selection_box_test_keeps_the_selection(engine, monkeypatch, slope, dt_us, h0):
    """OCT trace selection: per sample, the box test over all sampled
    candidates (their slope and c ranges) rules out samples at which no
    candidate can reach the trace, before the per-candidate tests; the
    selected traces equal those of the per-candidate tests alone
    (HPSS_OCT_BOX_TEST=0), counts midpoint by midpoint."""
    line = synthetic.structured_line(n_cmp=40, fold_range=(6, 12), h_max=2500, ns=300,
                                     dt_us=dt_us, n_reflectors=3, f=20.0, snr=8.0, seed=19)
    lower, upper = [1200.0, -slope], [5000.0, slope]
    _setup(engine, line, "oct", lower, upper, 2, 150.0, h0)
    m0s = line.cdp_midpoints[3::5]
    on = engine.select_traces(m0s)
    monkeypatch.setenv("HPSS_OCT_BOX_TEST", "0")
    off = engine.select_traces(m0s)
    monkeypatch.delenv("HPSS_OCT_BOX_TEST")
    assert off.sum() > 0
    assert np.array_equal(on, off)


@pytest.mark.parametrize("slope,dt_us,h0", [(5e-3, 2000, 0.0), (2e-4, 1000, 0.0),
                                             (2e-2, 4000, 0.0), (5e-3, 2000, 500.0),
                                             (1e-3, 1000, 1000.0), (2e-2, 4000, 0.5)])
def test_oct_tile_test_keeps_per_sample_results(engine, slope, dt_us, h0):
    """The OCT kernel drops, per 32-sample tile and candidate, the traces
    whose midpoint is farther than apm from every displaced midpoint the
    tile can reach; the rest go through the per-sample test.  Blocks and
    not-used counts equal the plain kernel's (every trace through the
    per-sample test) on wide apertures, steep and shallow slopes, fine
    sampling, h0 = 0 and h0 > 0 (tiles where t0^2 - c h0^2 changes sign run
    without the test)."""
    line = synthetic.structured_line(n_cmp=24, fold_range=(6, 12), h_max=2500, ns=400,
                                     dt_us=dt_us, n_reflectors=4, f=20.0, snr=8.0, seed=13)
    lower, upper, gran = [1200.0, -slope], [5000.0, slope], [5, 9]
    apm, tau = 150.0, 2
    _setup(engine, line, "oct", lower, upper, tau, apm, h0)
    m0s = line.cdp_midpoints[1::3]
    plain, st_p = engine.linear_search(m0s, gran, "plain")
    tuned, st_t = engine.linear_search(m0s, gran, "tuned")
    assert st_t["device_error"] == 0
    assert st_p["not_used"] > 0
    assert np.array_equal(plain, tuned)
    assert st_p["not_used"] == st_t["not_used"]


@pytest.mark.parametrize("h0", [0.0, 300.0])
def test_oct_negative_halfoffsets(engine, h0):
    """Half-offsets of either sign (x sin(az) + y cos(az) of the offset
    vector can be negative): the OCT formulas see h through h^2 and |h|, the
    box test through h^2; tuned equals plain, and the oracle agrees (the
    line and candidates of test_oct_small_line, where the FP32 formula is
    well conditioned, with the sign of half of the offsets flipped)."""
    base = synthetic.structured_line(n_cmp=16, fold_range=(4, 8), h_max=800, ns=200,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=12)
    rng = np.random.default_rng(3)
    h = base.halfoffsets * np.where(rng.random(base.halfoffsets.size) < 0.5, -1, 1)
    order = np.lexsort((h, base.midpoints))
    line = synthetic.Line(samples=np.ascontiguousarray(base.samples[order]),
                          midpoints=np.ascontiguousarray(base.midpoints[order]),
                          halfoffsets=np.ascontiguousarray(h[order].astype(np.float32)),
                          headers=base.headers[order], cdp_midpoints=base.cdp_midpoints,
                          dt_us=base.dt_us, seed=base.seed)
    lower, upper, gran = [1200.0, -1e-3], [5000.0, 1e-3], [6, 5]
    apm, tau = 60.0, 2
    _setup(engine, line, "oct", lower, upper, tau, apm, h0)
    m0s = line.cdp_midpoints[::4]
    plain, st_p = engine.linear_search(m0s, gran, "plain")
    tuned, st_t = engine.linear_search(m0s, gran, "tuned")
    assert st_t["device_error"] == 0
    assert np.array_equal(plain, tuned)
    assert st_p["not_used"] == st_t["not_used"]
    cands = oracle.oct_selection_candidates(lower, upper)
    _check_against_oracle("oct", line, m0s, plain, lower, upper, gran, tau, apm, h0, cands)


def test_argument_errors(engine, c1_line):
    with pytest.raises(capi.HpssError) as e:
        engine.set_traveltime("zocrs", [1000.0], [2000.0])
    assert e.value.code == -2            # logic_error: bound count
    with pytest.raises(capi.HpssError) as e:
        engine.set_window(16)            # w = 33 > MAX_WINDOW_SIZE
    assert e.value.code == -1
    rev = c1_line.midpoints[::-1].copy()
    with pytest.raises(capi.HpssError) as e:
        engine.upload_gather(c1_line.samples, rev, c1_line.halfoffsets, float(c1_line.dt))
    assert e.value.code == -1
    # velocity bounds must give a finite 4/v^2; geometry must be finite;
    # traces longer than 2^22 samples are refused
    for lo, hi in (([0.0], [2000.0]), ([-1000.0], [2000.0]), ([1e-30], [2000.0]),
                   ([1000.0], [float("inf")])):
        with pytest.raises(capi.HpssError) as e:
            engine.set_traveltime("cmp", lo, hi)
        assert e.value.code == -1
    bad = c1_line.halfoffsets.copy()
    bad[-1] = np.inf
    with pytest.raises(capi.HpssError) as e:
        engine.upload_gather(c1_line.samples, c1_line.midpoints, bad, float(c1_line.dt))
    assert e.value.code == -1
    import ctypes as C
    lib = engine._lib
    z = np.zeros(1, np.float32)
    rc = lib.hpss_upload_gather(engine.h, z.ctypes.data_as(C.POINTER(C.c_float)),
                                z.ctypes.data_as(C.POINTER(C.c_float)),
                                z.ctypes.data_as(C.POINTER(C.c_float)), 0, (1 << 22) + 1,
                                C.c_float(0.004), 0)
    assert rc == -1


def test_inclusive_grid_zocrs(engine):
    """HPSS_GRID_INCLUSIVE: both bounds included, velocity uniform in 4/v^2;
    the engine's grid equals the oracle's bit for bit (chosen parameters are
    reported from it) and the search passes the parity bar against the
    oracle on that grid."""
    line = synthetic.structured_line(n_cmp=30, fold_range=(8, 14), h_max=1000, ns=300,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=11)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    lower, upper, gran = [1414.2136, -a, -b], [6324.5553, a, b], [6, 5, 5]
    apm, tau = 125.0, 2
    _setup(engine, line, "zocrs", lower, upper, tau, apm)
    m0s = line.cdp_midpoints[::5]
    try:
        engine.set_grid_mode("inclusive")
        plain, _ = engine.linear_search(m0s, gran, "plain")
        tuned, st = engine.linear_search(m0s, gran, "tuned")
    finally:
        engine.set_grid_mode("reference")
    assert st["device_error"] == 0
    assert_same_but_stack(tuned, plain, 3)
    grid = oracle.build_grid("zocrs", lower, upper, gran, "inclusive")
    # reported A and B lie on the inclusive grid, whose ends are the bounds
    assert set(np.unique(plain[:, 3])) <= set(np.unique(grid[:, 1]))
    assert np.float32(-a) in grid[:, 1] and np.float32(a) in grid[:, 1]
    _check_against_oracle("zocrs", line, m0s, plain, lower, upper, gran, tau, apm,
                          grid_mode="inclusive")
    assert engine._lib.hpss_set_grid_mode(engine.h, 7) == -1     # unknown mode


@pytest.mark.parametrize("kernel", ["tuned", "tuned_exact"])
def test_candidate_split_equals_unsplit(engine, kernel):
    """A call with few midpoints splits the candidates of every (midpoint,
    32-sample tile) into ranges merged in candidate order, so that it fills
    the GPU; one-midpoint calls (the reference's per-midpoint interface) give
    the unsplit batched call's blocks bit for bit, near-tie counts included."""
    w = synthetic.WORKLOADS["cmp-production"]
    line = w.make_line(n_cmp=72)
    tau = 3
    _setup(engine, line, "cmp", w.lower, w.upper, tau)
    m0s = line.cdp_midpoints
    batched, st_b = engine.linear_search(m0s, w.granularity, kernel)
    assert st_b["candidate_parts"] == 1 and st_b["device_error"] == 0
    picks = [0, 17, 40, 71]
    ties = 0.0
    for i in picks:
        one, st = engine.linear_search(m0s[i:i + 1], w.granularity, kernel)
        assert st["candidate_parts"] > 1 and st["device_error"] == 0
        assert np.array_equal(one[0], batched[i]), i
        ties += st["near_ties"]
    few, st_f = engine.linear_search(m0s[picks], w.granularity, kernel)
    assert 1 < st_f["candidate_parts"] and np.array_equal(few, batched[picks])
    plain, st_p = engine.linear_search(m0s[picks], w.granularity, "plain")
    assert ties == st_f["near_ties"] == st_p["near_ties"]
    if kernel == "tuned_exact":
        assert np.array_equal(few, plain)
    else:
        assert_same_but_stack(few, plain, 1)
    print(f"{kernel}: one-midpoint calls split into {st['candidate_parts']} candidate ranges, "
          f"{len(picks)} midpoints into {st_f['candidate_parts']}")


def test_candidate_split_zocrs_and_empty_midpoint(engine):
    """ZO-CRS (three parameters) through the split, and a midpoint without
    traces inside a split call (its block stays zero)."""
    line = synthetic.structured_line(n_cmp=24, fold_range=(8, 14), h_max=1500, ns=400,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=6.0, seed=5)
    lower, upper, gran = [1500.0, -1e-3, -1e-7], [4500.0, 1e-3, 1e-7], [6, 5, 9]
    apm, tau = 60.0, 2
    _setup(engine, line, "zocrs", lower, upper, tau, apm)
    m0s = np.concatenate([line.cdp_midpoints[10:12], [np.float32(-5000.0)]])
    tuned, st = engine.linear_search(m0s, gran, "tuned")
    exact, st_e = engine.linear_search(m0s, gran, "tuned_exact")
    plain, st_p = engine.linear_search(m0s, gran, "plain")
    assert st["candidate_parts"] > 1 and st_e["candidate_parts"] > 1
    assert st["device_error"] == 0 and st_e["device_error"] == 0
    assert np.array_equal(exact, plain)
    assert_same_but_stack(tuned, plain, 3)
    assert np.all(tuned[-1] == 0) and np.all(exact[-1] == 0)
    assert st["near_ties"] == st_p["near_ties"]


def test_grid_reuse_across_calls(engine, c1_line):
    """The handle keeps the candidate grid and chunk bounds of its last call
    and reuses them when the next call has the same grid; a change of bounds,
    granularity or grid mode rebuilds them.  Every call equals the same call
    on a fresh handle."""
    w = synthetic.WORKLOADS["cmp-small"]
    tau = 2
    m0s = c1_line.cdp_midpoints[:4]
    seq = [(w.lower, [101], "reference"), (w.lower, [101], "reference"),
           (w.lower, [57], "reference"), ([1200.0], [101], "reference"),
           ([1200.0], [101], "inclusive"), (w.lower, [101], "reference")]
    _setup(engine, c1_line, "cmp", w.lower, w.upper, tau)
    try:
        for lower, gran, mode in seq:
            engine.set_traveltime("cmp", lower, w.upper)
            engine.set_grid_mode(mode)
            for kernel in ("tuned", "plain"):
                got, st = engine.linear_search(m0s, gran, kernel)
                with capi.Engine(0) as fresh:
                    _setup(fresh, c1_line, "cmp", lower, w.upper, tau)
                    fresh.set_grid_mode(mode)
                    want, _ = fresh.linear_search(m0s, gran, kernel)
                assert np.array_equal(got, want), (lower, gran, mode, kernel)
    finally:
        engine.set_grid_mode("reference")


def test_reupload_reuses_line_buffers(engine):
    """A re-upload keeps the device line buffers when the new line fits them
    (no allocation for a line of the same size); lines of other sizes,
    sample counts and storages in between give the results of a fresh
    handle."""
    w = synthetic.WORKLOADS["cmp-small"]
    big = synthetic.cmp_line(n_cmp=8, halfoffsets=list(range(25, 1176, 50)), ns=600,
                             dt_us=4000, n_reflectors=4, n_multiples=0, f=25.0, snr=10.0, seed=31)
    small = synthetic.cmp_line(n_cmp=5, halfoffsets=list(range(25, 776, 50)), ns=301,
                               dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0, seed=32)
    tau = 2

    def run(eng, line, storage):
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          storage=storage)
        eng.set_traveltime("cmp", w.lower, w.upper)
        eng.set_window(tau)
        return eng.linear_search(line.cdp_midpoints, w.granularity, "tuned")[0]

    with capi.Engine(0) as eng:
        first = run(eng, big, "fp32")
        held = eng.device_bytes()
        again = run(eng, big, "fp32")
        assert eng.device_bytes() == held
        assert np.array_equal(first, again)
        for line, storage in [(small, "fp16"), (big, "bf16"), (small, "fp32"), (big, "fp32")]:
            got = run(eng, line, storage)
            with capi.Engine(0) as fresh:
                want = run(fresh, line, storage)
            assert np.array_equal(got, want), (line.samples.shape, storage)


def _line_cases():
    cmp_line = synthetic.cmp_line(n_cmp=20, halfoffsets=list(range(25, 1176, 50)), ns=301,
                                  dt_us=4000, n_reflectors=4, n_multiples=0, f=25.0, snr=10.0,
                                  seed=41)
    w = synthetic.WORKLOADS["cmp-small"]
    zl = synthetic.structured_line(n_cmp=30, fold_range=(8, 14), h_max=1000, ns=300,
                                   dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=42)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    ol = synthetic.structured_line(n_cmp=16, fold_range=(4, 8), h_max=800, ns=200,
                                   dt_us=4000, n_reflectors=3, f=20.0, snr=8.0, seed=43)
    return [("cmp", cmp_line, w.lower, w.upper, w.granularity, 0.0, 0.0),
            ("zocrs", zl, [1414.2136, -a, -b], [6324.5553, a, b], [5, 5, 5], 125.0, 0.0),
            ("oct", ol, [1200.0, -1e-3], [5000.0, 1e-3], [6, 5], 60.0, 300.0)]


@pytest.mark.parametrize("storage, chunks, groups", [("fp32", None, None), ("bf16", None, None),
                                                     ("fp32", "5", "3"), ("fp32", "1", "64")])
def test_linear_search_line_equals_upload_then_search(storage, chunks, groups, monkeypatch):
    """hpss_linear_search_line (upload streamed in trace ranges, midpoints
    searched in groups as their traces arrive) gives the blocks and
    statistics of hpss_upload_gather followed by hpss_linear_search, for all
    three models, rows with padding (301 samples), calls with more and fewer
    midpoints than groups and a midpoint outside the line, with the default
    numbers of trace ranges and groups and with others (HPSS_STREAM_CHUNKS,
    HPSS_STREAM_GROUPS); the line stays resident afterwards."""
    if chunks:
        monkeypatch.setenv("HPSS_STREAM_CHUNKS", chunks)
        monkeypatch.setenv("HPSS_STREAM_GROUPS", groups)
    tau = 2
    for model, line, lower, upper, gran, apm, h0 in _line_cases():
        for m0s in (line.cdp_midpoints,
                    np.concatenate([line.cdp_midpoints[3:5], [np.float32(-777.0)]])):
            with capi.Engine(0) as ref_eng, capi.Engine(0) as eng:
                _setup(ref_eng, line, model, lower, upper, tau, apm, h0)
                ref_eng.upload_gather(line.samples, line.midpoints, line.halfoffsets,
                                      float(line.dt), storage=storage)
                want, st_w = ref_eng.linear_search(m0s, gran, "tuned")
                eng.set_traveltime(model, lower, upper, apm, h0)
                eng.set_window(tau)
                got, st = eng.linear_search_line(line.samples, line.midpoints, line.halfoffsets,
                                                 float(line.dt), m0s, gran, "tuned", storage)
                assert np.array_equal(got, want), (model, storage, m0s.size)
                for k in ("evals", "selected_traces", "not_used", "near_ties", "device_error"):
                    assert st[k] == st_w[k], (model, k, st[k], st_w[k])
                again, _ = eng.linear_search(m0s, gran, "tuned")
                assert np.array_equal(again, want)
                plain, _ = eng.linear_search_line(line.samples, line.midpoints,
                                                  line.halfoffsets, float(line.dt), m0s, gran,
                                                  "plain", storage)
                want_plain, _ = ref_eng.linear_search(m0s, gran, "plain")
                assert np.array_equal(plain, want_plain), (model, storage, "plain")


@pytest.mark.parametrize("storage", ["fp32", "bf16"])
@pytest.mark.parametrize("ns, tau, tuned_runs", [(16376, 3, True), (16377, 3, False),
                                                 (2000, 15, False)])
def test_size_limits_of_the_tuned_kernel(engine, ns, tau, tuned_runs, storage):
    """Sizes at the tuned kernel's limits: a trace row must fit its shared-
    memory stage (stride + 8 <= 16384 floats) and the window must be at most
    15 samples; beyond either the tuned call runs the plain kernel
    (kernel_variant -1).  Either way the results are the plain kernel's
    (semblance and chosen parameters bit for bit, stack within parity)."""
    w = synthetic.WORKLOADS["cmp-small"]
    line = synthetic.cmp_line(n_cmp=2, halfoffsets=list(range(25, 1176, 50)), ns=ns, dt_us=250,
                              n_reflectors=6, n_multiples=0, f=25.0, snr=10.0, seed=51)
    _setup(engine, line, "cmp", w.lower, w.upper, tau)
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)  # 16-bit rows: the bulk-copied staging at its limit
    m0s = line.cdp_midpoints
    tuned, st = engine.linear_search(m0s, [61], "tuned")
    plain, st_p = engine.linear_search(m0s, [61], "plain")
    assert st["device_error"] == 0 and st_p["device_error"] == 0
    assert (st["kernel_variant"] >= 0) == tuned_runs, st["kernel_variant"]
    assert_same_but_stack(tuned, plain, 1)
    assert st["near_ties"] == st_p["near_ties"]


def test_work_queue_multi_wave_calls(engine):
    """Calls with more units than resident CTAs take them from the work
    queue: an uneven-fold ZO-CRS line (midpoints ordered by selected traces)
    and a CMP line of 4200 midpoints (beyond the ordered batch size, queue in
    midpoint order).  The stack-exact tuned kernel equals the plain kernel bit
    for bit in both."""
    zl = synthetic.structured_line(n_cmp=60, fold_range=(4, 30), h_max=1500, ns=600,
                                   dt_us=4000, n_reflectors=4, f=20.0, snr=6.0, seed=61)
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    lower, upper, gran = [1414.2136, -a, -b], [6324.5553, a, b], [5, 3, 3]
    _setup(engine, zl, "zocrs", lower, upper, 2, 125.0)
    m0s = zl.cdp_midpoints
    exact, st = engine.linear_search(m0s, gran, "tuned_exact")
    plain, _ = engine.linear_search(m0s, gran, "plain")
    assert st["device_error"] == 0 and np.array_equal(exact, plain)
    cl = synthetic.cmp_line(n_cmp=4200, halfoffsets=[100, 400, 700, 1000], ns=64, dt_us=4000,
                            n_reflectors=2, n_multiples=0, f=25.0, snr=10.0, seed=62)
    w = synthetic.WORKLOADS["cmp-small"]
    _setup(engine, cl, "cmp", w.lower, w.upper, 2)
    m0s = cl.cdp_midpoints
    assert m0s.size > 4096
    exact, st = engine.linear_search(m0s, [21], "tuned_exact")
    plain, _ = engine.linear_search(m0s, [21], "plain")
    tuned, _ = engine.linear_search(m0s, [21], "tuned")
    assert st["device_error"] == 0 and np.array_equal(exact, plain)
    assert_same_but_stack(tuned, plain, 1)


def test_autotuner_decision_shared_across_handles(c1_line):
    """A handle opened after another one of the same device reuses the
    shape the first one tuned for the same call (the decision table is
    shared by the handles of the process); its results equal the first
    handle's."""
    w = synthetic.WORKLOADS["cmp-small"]
    m0s = c1_line.cdp_midpoints
    with capi.Engine(0) as first:
        _setup(first, c1_line, "cmp", w.lower, w.upper, 2)
        want, st0 = first.linear_search(m0s, w.granularity, "tuned")
    assert st0["kernel_variant"] >= 0
    for _ in range(3):
        with capi.Engine(0) as later:
            _setup(later, c1_line, "cmp", w.lower, w.upper, 2)
            got, st = later.linear_search(m0s, w.granularity, "tuned")
        assert st["kernel_variant"] == st0["kernel_variant"]
        assert np.array_equal(got, want)
