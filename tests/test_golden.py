"""Golden fixtures made by the reference's own CUDA kernels
(tests/golden/make_reference_golden.py, run on a GB300 with kernels compiled
from the reference sources).

* CPU: the oracle against the fixtures (this pins the oracle);
* GPU: the engine's plain, tuned and tuned_exact kernels against the
  fixtures through the C ABI -- chosen candidates and values bit-identical
  where the arithmetic is pinned (the tuned kernel's stack, whose linear sum
  is summed in another order, within parity.STACK_REL), within the parity
  tolerances everywhere.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import oracle
from parity import Report, assert_same_but_stack, compare_block, index_scale

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = sorted(p.stem[4:] for p in GOLDEN.glob("ref_*.npz"))


def load(name):
    z = np.load(GOLDEN / f"ref_{name}.npz")
    d = {k: z[k] for k in z.files}
    if "samples16" in d:  # FP16-valued amplitudes, stored as FP16
        d["samples"] = d.pop("samples16").astype(np.float32)
    return d


# Oracle comparisons of a fixture cost P x S x selected traces evaluations
# per midpoint; above this many the oracle runs on a fixed subset of the
# samples (every one of them is still compared bit for bit with the
# reference's results by the GPU test).
ORACLE_EVALS_MAX = 3e8


def oracle_tables(z, i, m0, sel):
    """Oracle semblance / stack tables of midpoint i and the sample indices
    they cover (all samples, or an evenly spaced subset for large cases)."""
    model = str(z["model"])
    S = z["samples"].shape[1]
    P = z["params"].shape[0]
    args = (model, z["samples"], z["midpoints"], z["halfoffsets"], sel, float(m0),
            float(z["dt"]), int(z["tau"]), z["params"])
    if float(P) * S * sel.size <= ORACLE_EVALS_MAX:
        sem, stk, nu = oracle.ls_eval(*args, float(z["apm"]), float(z["h0"]))
        return sem, stk, nu, np.arange(S)
    n = max(8, int(ORACLE_EVALS_MAX / (float(P) * sel.size)))
    sidx = np.unique(np.linspace(0, S - 1, n).astype(np.uint32))
    sem, stk = oracle.ls_eval_samples(*args, sidx, float(z["apm"]), float(z["h0"]))
    return sem, stk, None, sidx


def selection(z, m0):
    model = str(z["model"])
    if model == "cmp":
        return np.nonzero(z["midpoints"] == np.float32(m0))[0]
    if model == "zocrs":
        return np.nonzero(oracle.select("zocrs", z["midpoints"], z["halfoffsets"], m0,
                                        float(z["apm"])))[0]
    cands = oracle.oct_selection_candidates(z["lower"], z["upper"])
    return np.nonzero(oracle.select("oct", z["midpoints"], z["halfoffsets"], m0,
                                    float(z["apm"]), float(z["h0"]), z["samples"].shape[1],
                                    float(z["dt"]), cands))[0]


def test_fixtures_present():
    assert set(CASES) >= {"cmp", "zocrs", "oct_h0_0", "oct_h0_300", "oct_h0_500",
                          "oct_h0_1000", "cmp_production_w7", "zocrs_full_grid"}


@pytest.mark.parametrize("name", CASES)
def test_oracle_grid_and_selection_match_reference(name):
    z = load(name)
    model = str(z["model"])
    grid = oracle.build_grid(model, z["lower"], z["upper"], z["gran"])
    # the reference builds its grid on the device with fast-math 4/v^2: equal to
    # IEEE within one ulp
    np.testing.assert_allclose(grid, z["params"], rtol=2.5e-7, atol=0)
    for i, m0 in enumerate(z["m0s"]):
        assert selection(z, m0).size == z["counts"][i]


@pytest.mark.parametrize("name", CASES)
def test_oracle_matches_reference_kernels(name):
    z = load(name)
    model = str(z["model"])
    params = z["params"]
    rep = Report(sembl_p999=index_scale(z["samples"].shape[1], model) * Report.sembl_p999)
    for i, m0 in enumerate(z["m0s"]):
        sel = selection(z, m0).astype(np.uint32)
        if sel.size == 0:
            assert np.all(z["results"][i] == 0)
            continue
        sem, stk, nu, sidx = oracle_tables(z, i, m0, sel)
        rms = float(np.sqrt(np.mean(z["samples"][sel] ** 2)))
        compare_block(rep, z["results"][i][:, sidx], sem, stk, params, rms)
        if model == "oct":
            # IEEE FP32 (the oracle) against the fast-math build (the
            # reference): a trace within rounding of the aperture may flip;
            # the engine's count is checked for equality on the GPU
            assert abs(float(nu.sum()) - z["not_used"][i]) <= max(2.0, 1e-5 * z["not_used"][i])
    rep.check()


@pytest.mark.gpu
@pytest.mark.parametrize("kernel", ["plain", "tuned", "tuned_exact"])
@pytest.mark.parametrize("name", CASES)
def test_engine_matches_reference_kernels(engine, name, kernel):
    z = load(name)
    model = str(z["model"])
    engine.upload_gather(z["samples"], z["midpoints"], z["halfoffsets"], float(z["dt"]))
    engine.set_traveltime(model, z["lower"], z["upper"], float(z["apm"]), float(z["h0"]))
    engine.set_window(int(z["tau"]))
    out, st = engine.linear_search(z["m0s"], z["gran"], kernel)
    assert st["device_error"] == 0
    assert np.array_equal(engine.select_traces(z["m0s"]), z["counts"])
    ref = z["results"]
    cmp_rows = out == ref
    if kernel == "tuned" and model != "oct":
        # stack: same values summed in another order
        cmp_rows[:, 1] = True
        if model in ("cmp", "zocrs"):
            assert_same_but_stack(out, ref, ref.shape[1] - 2)
    exact = np.all(cmp_rows, axis=1)           # per (midpoint, sample)
    frac = float(exact.mean())
    print(f"{name} {kernel}: bit-identical samples {frac:.6f}")
    # midpoints without traces: zeros, as the reference's reset result
    for i in np.nonzero(z["counts"] == 0)[0]:
        assert np.all(out[i] == 0)
    if model == "oct":
        assert st["not_used"] == float(np.sum(z["not_used"]))
    # every sample: the reference's chosen candidate and values within the
    # parity tolerances (tests/parity.py), judged against the reference's table
    params = z["params"]
    rep = Report(sembl_p999=index_scale(z["samples"].shape[1], model) * Report.sembl_p999)
    for i, m0 in enumerate(z["m0s"]):
        sel = selection(z, m0).astype(np.uint32)
        if sel.size == 0:
            continue
        sem, stk, _, sidx = oracle_tables(z, i, m0, sel)
        rms = float(np.sqrt(np.mean(z["samples"][sel] ** 2)))
        compare_block(rep, out[i][:, sidx], sem, stk, params, rms)
    rep.check()
    # traveltime arithmetic pinned to the reference's (CMP, ZO-CRS and the
    # OCT displaced midpoint and time): bit-identical results
    assert frac == 1.0, frac
