"""Stretch-free stack on the GPU, through the C ABI.

CMP is checked against the reference's own stretch-free kernels (golden
fixture: the reference's semblance + best-n kernels fed with the reference's
linear-search velocities).  ZO-CRS and OCT, which the reference's CUDA path
does not run (its OCT case falls through into `throw`), are checked against
the oracle's restatement of the reference kernels.
"""
from pathlib import Path

import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import synthetic
from oracle import oracle

pytestmark = pytest.mark.gpu
GOLDEN = Path(__file__).resolve().parent / "golden"


def _check_sf(out, sem, stk, nmax, near_tie=1e-4):
    """out: engine block [3][S]; sem/stk: oracle tables [S][2*nmax+1]."""
    idx = oracle.argmax(sem)
    S = sem.shape[0]
    rows = np.arange(S)
    ref0 = sem[rows, idx]
    rel = np.abs(out[0] - ref0) / np.maximum(np.abs(ref0), 1e-3)
    assert np.quantile(rel, 0.999) <= 2e-4
    n_got = out[2].astype(int)
    far = 0
    for s in np.nonzero(n_got != idx - nmax)[0]:
        alt = sem[s, n_got[s] + nmax]
        if abs(float(ref0[s]) - float(alt)) > near_tie * max(float(ref0[s]), 1e-3):
            far += 1
    assert far <= 0.002 * S, far


SF_FIXTURES = sorted(p.stem[4:] for p in GOLDEN.glob("ref_*.npz")
                     if "sf_results" in np.load(p).files)


@pytest.mark.parametrize("name", SF_FIXTURES)
def test_cmp_stretch_free_matches_reference_kernels(engine, name):
    """The reference's CMP stretch-free kernels on its own linear-search
    velocities (window 5 on the small line; window 9 on the production-line
    slice, whose search ran with window 7)."""
    from test_golden import load
    z = load(name)
    engine.upload_gather(z["samples"], z["midpoints"], z["halfoffsets"], float(z["dt"]))
    engine.set_traveltime("cmp", z["lower"], z["upper"])
    engine.set_window(int(z["sf_tau"]) if "sf_tau" in z else int(z["tau"]))
    sf = z["sf_results"]
    m0s = z["m0s"][: sf.shape[0]]
    prior = z["results"][: sf.shape[0], 2:3]        # reference LS velocities [nM0][1][S]
    out, st = engine.stretch_free(m0s, prior, 10)
    assert st["evals"] == float(np.sum(z["counts"][: sf.shape[0]])) * sf.shape[2] * 21
    exact = float(np.mean(np.all(out == sf, axis=1)))
    print(f"stretch-free {name}: bit-identical samples {exact:.6f}")
    assert exact == 1.0


@pytest.mark.parametrize("model", ["zocrs", "oct"])
def test_stretch_free_other_models_vs_oracle(engine, model):
    line = synthetic.structured_line(n_cmp=12, fold_range=(6, 10), h_max=900, ns=250,
                                     dt_us=4000, n_reflectors=3, f=20.0, snr=6.0, seed=61)
    if model == "zocrs":
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, gran, apm, h0 = [1414.2136, -a, -b], [6324.5553, a, b], [8, 5, 5], 100.0, 0.0
    else:
        lower, upper, gran, apm, h0 = [1200.0, -1e-3], [5000.0, 1e-3], [10, 5], 60.0, 200.0
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime(model, lower, upper, apm, h0)
    engine.set_window(2)
    m0s = line.cdp_midpoints[4:7]
    ls, _ = engine.linear_search(m0s, gran, "plain")
    prior = np.ascontiguousarray(ls[:, 2:])
    out, st = engine.stretch_free(m0s, prior, 10)
    S = line.samples_per_trace
    cands = oracle.oct_selection_candidates(lower, upper) if model == "oct" else None
    for i, m0 in enumerate(m0s):
        if model == "oct":
            init = np.stack([prior[i, 0], prior[i, 1]], axis=1)[:, None, :]
            sel = np.nonzero(oracle.select_oct_per_sample(line.midpoints, line.halfoffsets, m0,
                                                          apm, h0, S, float(line.dt), init))[0]
        else:
            sel = np.nonzero(oracle.select(model, line.midpoints, line.halfoffsets, m0, apm))[0]
        sem, stk, _ = oracle.sf_eval(model, line.samples, line.midpoints, line.halfoffsets,
                                     sel.astype(np.uint32), m0, float(line.dt), 2, prior[i],
                                     10, apm, h0)
        _check_sf(out[i], sem, stk, 10)


@pytest.mark.parametrize("model, wide", [("cmp", False), ("zocrs", False), ("zocrs", True),
                                         ("oct", False), ("oct", True)])
@pytest.mark.parametrize("storage", ["fp32", "fp16"])
def test_block_kernels_equal_warp_kernel(engine, monkeypatch, model, wide, storage):
    """The stretch-free block kernels (warp = n value, lane = sample): the
    per-pair one (CMP; HPSS_SF_KERNEL=block for any model) and the one that
    shares each (s - n, trace) traveltime among the pairs (ZO-CRS, OCT, in
    batches of 64 traces: `wide` apertures hold more than one batch) give
    the warp-per-sample kernel's block (lanes = n values) bit for bit,
    not-used counts included; a window or n count outside the block
    kernels' instantiations (window 13, 33 n values) runs the warp kernel."""
    line = synthetic.structured_line(n_cmp=16 if wide else 10, fold_range=(5, 9), h_max=900,
                                     ns=300, dt_us=4000, n_reflectors=3, f=20.0, snr=6.0,
                                     seed=67)
    if model == "cmp":
        lower, upper, gran, apm, h0 = [1200.0], [5000.0], [41], 0.0, 0.0
    elif model == "zocrs":
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, gran, apm, h0 = [1414.2136, -a, -b], [6324.5553, a, b], [6, 5, 5], 100.0, 0.0
    else:
        lower, upper, gran, apm, h0 = [1200.0, -1e-3], [5000.0, 1e-3], [8, 5], 60.0, 300.0
    if wide:
        apm *= 8.0
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                         storage=storage)
    engine.set_traveltime(model, lower, upper, apm, h0)
    engine.set_window(3)
    m0s = line.cdp_midpoints[2:8]
    ls, _ = engine.linear_search(m0s, gran, "plain")
    prior = np.ascontiguousarray(ls[:, 2:])
    for nmax in (0, 7, 15):
        monkeypatch.delenv("HPSS_SF_KERNEL", raising=False)
        dflt, st_d = engine.stretch_free(m0s, prior, nmax)
        monkeypatch.setenv("HPSS_SF_KERNEL", "block")
        blk, st_b = engine.stretch_free(m0s, prior, nmax)
        monkeypatch.setenv("HPSS_SF_KERNEL", "warp")
        wrp, st_w = engine.stretch_free(m0s, prior, nmax)
        assert np.array_equal(dflt, wrp), (model, storage, nmax, "default")
        assert np.array_equal(blk, wrp), (model, storage, nmax, "block")
        assert st_d["not_used"] == st_w["not_used"] == st_b["not_used"]
        if wide:  # more than one batch of traces per midpoint
            assert st_d["selected_traces"] > 64 * len(m0s), st_d["selected_traces"]
    monkeypatch.delenv("HPSS_SF_KERNEL", raising=False)
    # warp kernel by shape: 33 n values, and window 13
    big, _ = engine.stretch_free(m0s, prior, 16)
    assert np.all(np.isfinite(big)) and np.all(np.abs(big[:, 2]) <= 16)
    engine.set_window(6)
    w13, _ = engine.stretch_free(m0s, prior, 10)
    assert np.all(np.isfinite(w13)) and np.all(np.abs(w13[:, 2]) <= 10)


def test_stretch_free_argument_errors(engine):
    z = np.load(GOLDEN / "ref_cmp.npz")
    engine.upload_gather(z["samples"], z["midpoints"], z["halfoffsets"], float(z["dt"]))
    engine.set_traveltime("cmp", z["lower"], z["upper"])
    engine.set_window(int(z["tau"]))
    from highperformanceseismicstacking_gb300 import capi
    with pytest.raises(capi.HpssError):
        engine.stretch_free(z["m0s"][:1], z["results"][:1, 2:3], -1)


@pytest.mark.parametrize("slope,h0", [(1e-3, 0.0), (5e-3, 0.0), (1e-3, 500.0), (5e-3, 1000.0)])
def test_oct_stretch_free_box_test_keeps_results(engine, monkeypatch, slope, h0):
    """OCT stretch-free: a warp (one sample, lanes over n) drops, per block of
    32 traces, those no lane's displaced midpoint can reach (the box of the
    lanes' t0 and parameters) before the per-lane tests; blocks and
    not-used counts equal those with the box test off
    (HPSS_OCT_BOX_TEST=0)."""
    line = synthetic.structured_line(n_cmp=24, fold_range=(6, 12), h_max=2500, ns=400,
                                     dt_us=2000, n_reflectors=4, f=20.0, snr=8.0, seed=14)
    lower, upper = [1200.0, -slope], [5000.0, slope]
    engine.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    engine.set_traveltime("oct", lower, upper, 150.0, h0)
    engine.set_window(4)
    m0s = line.cdp_midpoints[2::5]
    ls, _ = engine.linear_search(m0s, [9, 7], "tuned")
    prior = np.ascontiguousarray(ls[:, 2:])
    sf, st = engine.stretch_free(m0s, prior, 10)
    monkeypatch.setenv("HPSS_OCT_BOX_TEST", "0")
    sf0, st0 = engine.stretch_free(m0s, prior, 10)
    monkeypatch.delenv("HPSS_OCT_BOX_TEST")
    assert st0["not_used"] > 0
    assert st["not_used"] == st0["not_used"]
    assert st["selected_traces"] == st0["selected_traces"]
    assert np.array_equal(sf, sf0)
