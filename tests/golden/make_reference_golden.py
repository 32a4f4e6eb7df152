#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference's own CUDA
kernels.

Needs a GPU and oracle/_ref/*.fatbin (built from the reference sources by
oracle/build_ref.py).  For each case it makes a small seeded line, runs the
reference's selection, grid, semblance and argmax kernels with the launch
sequence of CudaLinearSearchAlgorithm (and, for CMP, CudaStretchFreeAlgorithm),
and stores inputs and outputs in one compressed .npz:

    python tests/golden/make_reference_golden.py OUT_DIR [CASE ...]

(all cases by default).  Cases marked store16 keep FP16-valued amplitudes
(rounded before the reference runs, stored as FP16: exact in FP32).

The fixtures are committed; the tests read them without the reference.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from highperformanceseismicstacking_gb300 import synthetic  # noqa: E402
from oracle import oracle, ref_runner  # noqa: E402

CASES = {
    "cmp": dict(model="cmp", lower=[1000.0], upper=[5040.0], gran=[101], tau=2, apm=0.0,
                h0=0.0, line=lambda: synthetic.cmp_line(
                    n_cmp=4, halfoffsets=list(range(25, 1176, 50)), ns=500, dt_us=4000,
                    n_reflectors=4, n_multiples=0, f=25.0, snr=10.0, seed=2001)),
    "zocrs": dict(model="zocrs", lower=None, upper=None, gran=[5, 5, 5], tau=2, apm=125.0,
                  h0=0.0, line=lambda: synthetic.structured_line(
                      n_cmp=12, fold_range=(6, 10), h_max=1000, ns=300, dt_us=4000,
                      n_reflectors=4, f=20.0, snr=5.0, seed=2002)),
    "oct_h0_0": dict(model="oct", lower=[1200.0, -1e-3], upper=[5000.0, 1e-3], gran=[6, 5],
                     tau=2, apm=60.0, h0=0.0, line=lambda: synthetic.structured_line(
                         n_cmp=10, fold_range=(4, 8), h_max=800, ns=200, dt_us=4000,
                         n_reflectors=3, f=20.0, snr=8.0, seed=2003)),
    "oct_h0_300": dict(model="oct", lower=[1200.0, -1e-3], upper=[5000.0, 1e-3], gran=[6, 5],
                       tau=2, apm=60.0, h0=300.0, line=lambda: synthetic.structured_line(
                           n_cmp=10, fold_range=(4, 8), h_max=800, ns=200, dt_us=4000,
                           n_reflectors=3, f=20.0, snr=8.0, seed=2003)),
    # OCT target half-offsets of the OCT DE workload (h0 = 500 / 1000 m)
    "oct_h0_500": dict(model="oct", lower=[1200.0, -1e-3], upper=[5000.0, 1e-3], gran=[6, 5],
                       tau=2, apm=60.0, h0=500.0, line=lambda: synthetic.structured_line(
                           n_cmp=10, fold_range=(4, 8), h_max=800, ns=200, dt_us=4000,
                           n_reflectors=3, f=20.0, snr=8.0, seed=2003)),
    "oct_h0_1000": dict(model="oct", lower=[1200.0, -1e-3], upper=[5000.0, 1e-3],
                        gran=[6, 5], tau=2, apm=60.0, h0=1000.0,
                        line=lambda: synthetic.structured_line(
                            n_cmp=10, fold_range=(4, 8), h_max=800, ns=200, dt_us=4000,
                            n_reflectors=3, f=20.0, snr=8.0, seed=2003)),
    # A slice of the CMP production line (fold 60 at 0..2950 m, 2000 samples
    # at 2 ms, 12 reflectors + 3 multiples, 401 velocities 1000..6012.5 m/s,
    # window 7), plus the stretch-free stack with window 9 over its
    # velocities.  Amplitudes rounded to FP16 values (exact in FP32) and
    # stored as FP16 to keep the fixture small.
    "cmp_production_w7": dict(
        model="cmp", lower=[1000.0], upper=[6012.5], gran=[401], tau=3, apm=0.0, h0=0.0,
        store16=True, sf_tau=4,
        line=lambda: synthetic.cmp_line(
            n_cmp=4, halfoffsets=list(range(0, 2951, 50)), ns=2000, dt_us=2000,
            n_reflectors=12, n_multiples=3, f=25.0, snr=10.0, seed=2005)),
    # ZO-CRS at the full 21 x 21 x 41 candidate grid of the ZO-CRS workload
    # (fold U{30..90}, half-offsets up to 2000 m, +-15-CMP aperture, w 5),
    # two midpoints whose apertures lie inside the 32-CMP line; 300 samples
    # (4 ms) instead of 1500 keep the fixture small.  FP16-valued amplitudes.
    "zocrs_full_grid": dict(
        model="zocrs", lower=None, upper=None, gran=[41, 21, 21], tau=2, apm=375.0, h0=0.0,
        store16=True, m0_index=[15, 16], no_empty=True,
        line=lambda: synthetic.structured_line(
            n_cmp=32, fold_range=(30, 90), h_max=2000, ns=300, dt_us=4000,
            n_reflectors=8, f=20.0, snr=5.0, seed=2006)),
}


def main(out_dir: str, names=()):
    out = Path(out_dir)
    out.mkdir(parents=True, exist_ok=True)
    rk = ref_runner.ReferenceKernels()
    for name, c in CASES.items():
        if names and name not in names:
            continue
        line = c["line"]()
        if c.get("store16"):
            line.samples = line.samples.astype(np.float16).astype(np.float32)
        model = c["model"]
        lower, upper = c["lower"], c["upper"]
        if model == "zocrs":
            a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
            lower, upper = [1414.2136, -a, -b], [6324.5553, a, b]
        S = line.samples_per_trace
        dt = float(line.dt)
        params = rk.build_grid(model, lower, upper, c["gran"])
        cands = (oracle.oct_selection_candidates(lower, upper) if model == "oct" else None)
        if "m0_index" in c:
            m0s = line.cdp_midpoints[c["m0_index"]]
        else:
            m0s = line.cdp_midpoints
        if not c.get("no_empty"):
            # one midpoint without traces: the reference's all-zero result
            m0s = np.concatenate([m0s, [np.float32(line.cdp_midpoints[-1] + 7.0)]])
        results, counts, not_used = [], [], []
        for m0 in m0s:
            mask = rk.select(model, line.midpoints, line.halfoffsets, float(m0), c["apm"],
                             c["h0"], S, dt, cands)
            sel = np.nonzero(mask)[0]
            counts.append(sel.size)
            res, sem, stk, nu = rk.linear_search_midpoint(
                model, line.samples, line.midpoints, line.halfoffsets, sel, float(m0), dt,
                c["tau"], params, c["apm"], c["h0"])
            results.append(res)
            not_used.append(float(np.sum(nu)))
        extra = {}
        if model == "cmp":
            # stretch-free over the linear-search velocities of each midpoint
            sf_tau = c.get("sf_tau", c["tau"])
            sf = []
            for i, m0 in enumerate(line.cdp_midpoints):
                sel = np.nonzero(line.midpoints == m0)[0]
                sf.append(rk.stretch_free_midpoint_cmp(line.samples, line.halfoffsets, sel, dt,
                                                       sf_tau, results[i][2]))
            extra["sf_results"] = np.stack(sf)
            extra["sf_tau"] = sf_tau
        if c.get("store16"):
            extra["samples16"] = line.samples.astype(np.float16)
        else:
            extra["samples"] = line.samples
        np.savez_compressed(
            out / f"ref_{name}.npz", midpoints=line.midpoints,
            halfoffsets=line.halfoffsets, dt=np.float32(dt), tau=c["tau"],
            model=model, lower=np.float32(lower), upper=np.float32(upper),
            gran=np.uint32(c["gran"]), apm=np.float32(c["apm"]), h0=np.float32(c["h0"]),
            params=params, m0s=m0s.astype(np.float32), counts=np.asarray(counts),
            results=np.stack(results), not_used=np.asarray(not_used), **extra)
        print(name, "midpoints", len(m0s), "selected", counts)


if __name__ == "__main__":
    if len(sys.argv) < 2:
        sys.exit("usage: make_reference_golden.py OUT_DIR [CASE ...]")
    main(sys.argv[1], sys.argv[2:])
