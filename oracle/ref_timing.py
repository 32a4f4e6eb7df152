"""Timing of the reference's own CUDA kernels on the GB300 (the reference's
CUDA build as a reported baseline beside the engine's numbers).

TEST INFRASTRUCTURE / BASELINE ONLY: the kernels are the reference's, built
from its sources by oracle/build_ref.py into oracle/_ref/ and replayed by
oracle/ref_runner.py with the launch sequences of the reference's
Cuda*Algorithm classes, one midpoint at a time, as the reference runs them.
Device time of the evaluation and argmax (or the whole DE) launches is taken
with CUDA events; trace selection and packing are excluded, as in the
reference's own total_kernel_exec_time.  Nothing of the engine runs here.
The midpoints are those of the engine's bench side measurements, so the
evals/s compare directly.

    python oracle/ref_timing.py          # one JSON object, every workload
"""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

from highperformanceseismicstacking_gb300 import synthetic  # noqa: E402
from highperformanceseismicstacking_gb300.su import tau_index  # noqa: E402
from oracle import oracle, ref_runner  # noqa: E402


def _line(name, cache, n_cmp=None):
    key = (name, n_cmp)
    if key not in cache:
        cache[key] = synthetic.WORKLOADS[name].make_line(n_cmp=n_cmp)
    return cache[key]


def cmp_ls(rk, cache, n_mid=100):
    """CMP production line, 401 velocities, window 7: per midpoint
    computeSemblancesForCommonMidPoint + selectBestSemblancesForCommonMidPoint
    (CudaLinearSearchAlgorithm.cu:35-163).  Returns the timing and the
    reference's velocities (the stretch-free prior)."""
    w = synthetic.WORKLOADS["cmp-production"]
    line = _line("cmp-production", cache)
    tau = tau_index(w.tau, line.dt)
    params = rk.build_grid("cmp", w.lower, w.upper, w.granularity)
    S, P = line.samples_per_trace, params.shape[0]
    ms, evals, vel = 0.0, 0.0, []
    for i, m0 in enumerate(line.cdp_midpoints[:n_mid]):
        sel = np.nonzero(line.midpoints == m0)[0]
        call = lambda: rk.linear_search_midpoint("cmp", line.samples, line.midpoints,
                                                 line.halfoffsets, sel, float(m0),
                                                 float(line.dt), tau, params, timing=True)
        if i == 0:
            call()  # module load
        res, _, _, _, t = call()
        ms += t
        evals += float(sel.size) * S * P
        vel.append(res[2])
    return ({"workload": "cmp-production", "midpoints": int(n_mid), "ms": ms, "evals": evals,
             "value": evals / (ms / 1e3)}, np.stack(vel))


def zocrs_ls(rk, cache, n_mid=2):
    w = synthetic.WORKLOADS["zocrs-ls"]
    line = _line("zocrs-ls", cache)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    params = rk.build_grid("zocrs", lower, upper, w.granularity)
    S = line.samples_per_trace
    mid = len(line.cdp_midpoints) // 2
    ms, evals = 0.0, 0.0
    for i, m0 in enumerate(line.cdp_midpoints[mid:mid + n_mid]):
        sel = np.nonzero(rk.select("zocrs", line.midpoints, line.halfoffsets, float(m0), w.apm,
                                   0.0, S, float(line.dt)))[0]
        call = lambda: rk.linear_search_midpoint("zocrs", line.samples, line.midpoints,
                                                 line.halfoffsets, sel, float(m0),
                                                 float(line.dt), tau, params, w.apm, 0.0,
                                                 timing=True)
        if i == 0:
            call()
        _, _, _, _, t = call()
        ms += t
        evals += float(sel.size) * S * params.shape[0]
    return {"workload": "zocrs-ls (21 x 21 x 41 candidates)", "midpoints": int(n_mid),
            "ms": ms, "evals": evals, "value": evals / (ms / 1e3)}


def oct_ls(rk, cache, n_mid=1, h0=0.0):
    w = synthetic.WORKLOADS["oct-de"]
    line = _line("oct-de", cache)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    gran = [11, 5]
    params = rk.build_grid("oct", lower, upper, gran)
    cands = oracle.oct_selection_candidates(lower, upper)
    S = line.samples_per_trace
    mid = len(line.cdp_midpoints) // 2
    ms, evals = 0.0, 0.0
    for i, m0 in enumerate(line.cdp_midpoints[mid:mid + n_mid]):
        sel = np.nonzero(rk.select("oct", line.midpoints, line.halfoffsets, float(m0), w.apm,
                                   h0, S, float(line.dt), cands))[0]
        call = lambda: rk.linear_search_midpoint("oct", line.samples, line.midpoints,
                                                 line.halfoffsets, sel, float(m0),
                                                 float(line.dt), tau, params, w.apm, h0,
                                                 timing=True)
        if i == 0:
            call()
        _, _, _, _, t = call()
        ms += t
        evals += float(sel.size) * S * params.shape[0]
    return {"workload": "oct-de line, 11 x 5 candidates", "h0": h0, "midpoints": int(n_mid),
            "ms": ms, "evals": evals, "value": evals / (ms / 1e3)}


def de(rk, cache, name, n_mid=2, h0=None):
    """The reference's whole DE sequence per midpoint
    (CudaDifferentialEvolutionAlgorithm.cu:35-353, F 0.5 / CR 0.9 shim)."""
    w = synthetic.WORKLOADS[name]
    h0 = w.h0 if h0 is None else float(h0)
    line = _line(name, cache)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    S = line.samples_per_trace
    mid = len(line.cdp_midpoints) // 2
    ms, evals, best = 0.0, 0.0, []
    for i, m0 in enumerate(line.cdp_midpoints[mid:mid + n_mid]):
        sel = None
        if w.model == "zocrs":
            sel = np.nonzero(np.abs(np.float32(m0) - line.midpoints) <= np.float32(w.apm))[0]
        res, t, n_sel = rk.differential_evolution_midpoint(
            w.model, line.samples, line.midpoints, line.halfoffsets, float(m0), float(line.dt),
            tau, lower, upper, w.population, w.generations, seed=11 + i, apm=w.apm, h0=h0,
            sel=sel, operators="common_differential_evolution_f05cr09")
        ms += t
        evals += float(n_sel) * S * w.population * w.generations
        best.append(float(np.mean(res[0])))
    return {"workload": name, "h0": h0, "midpoints": int(n_mid), "population": w.population,
            "generations": w.generations, "ms": ms, "evals": evals,
            "value": evals / (ms / 1e3), "mean_best_semblance": float(np.mean(best))}


def cmp_sf(rk, cache, prior, n_mid=20):
    """CMP stretch-free (21 n, window 7) over the reference's own velocities."""
    w = synthetic.WORKLOADS["cmp-production"]
    line = _line("cmp-production", cache)
    tau = tau_index(w.tau, line.dt)
    S = line.samples_per_trace
    ms, evals = 0.0, 0.0
    for i, m0 in enumerate(line.cdp_midpoints[:n_mid]):
        sel = np.nonzero(line.midpoints == m0)[0]
        _, t = rk.stretch_free_midpoint_cmp(line.samples, line.halfoffsets, sel, float(line.dt),
                                            tau, prior[i], timing=True)
        ms += t
        evals += float(sel.size) * S * 21
    return {"workload": "cmp-production stretch-free (21 n, window 7)", "midpoints": int(n_mid),
            "ms": ms, "evals": evals, "value": evals / (ms / 1e3)}


def reference_cuda() -> dict:
    """Every workload above, on the current GPU."""
    if not ref_runner.available():
        return {"unavailable": "reference kernels not built (oracle/build_ref.py needs the "
                               "reference source tree)"}
    rk = ref_runner.ReferenceKernels()
    cache = {}
    ls, vel = cmp_ls(rk, cache)
    out = {"cmp_linear_search": ls,
           "cmp_stretch_free": cmp_sf(rk, cache, vel),
           "zocrs_linear_search": zocrs_ls(rk, cache),
           "oct_linear_search": oct_ls(rk, cache),
           "zocrs_de": de(rk, cache, "zocrs-de"),
           "oct_de": de(rk, cache, "oct-de")}
    return out


if __name__ == "__main__":
    print(json.dumps(reference_cuda()))
