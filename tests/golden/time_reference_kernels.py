#!/usr/bin/env python3
"""Time the reference's own CUDA kernels (fatbins built from the reference
sources by oracle/build_ref.py) on the workloads of the engine's bench, next
to the engine on the same midpoints.  Prints one JSON line per workload.

  ls [n]  CMP production line, 401 velocities, window 7: per midpoint the
          reference's launch sequence (computeSemblancesForCommonMidPoint +
          selectBestSemblancesForCommonMidPoint, CudaLinearSearchAlgorithm.cu
          :35-163) timed with CUDA events; trace selection and packing are
          excluded, as in the reference's own total_kernel_exec_time.
  de [n]  ZO-CRS and OCT differential evolution workloads (population 32 / 48,
          60 / 80 generations, F 0.5, CR 0.9): the reference's whole DE
          sequence per midpoint (CudaDifferentialEvolutionAlgorithm.cu:35-353,
          one synchronised launch per operator and generation, as the
          reference runs it) against the engine's fused DE launch.

  oct [n] OCT linear search on the OCT DE line's geometry (11 x 5 candidates).
  (de and oct take an optional third argument: the OCT reference half-offset
  h0, default the workload's 0 m.)
  zocrs [n] ZO-CRS linear search on the ZO-CRS line (21 x 21 x 41 candidates).
  sf [n]  CMP stretch-free stack on the CMP production line.

    python tests/golden/time_reference_kernels.py ls 40
    python tests/golden/time_reference_kernels.py de 2
    python tests/golden/time_reference_kernels.py oct 1
    python tests/golden/time_reference_kernels.py oct 1 500
    python tests/golden/time_reference_kernels.py sf 20
    python tests/golden/time_reference_kernels.py zocrs 2
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from highperformanceseismicstacking_gb300 import capi, synthetic  # noqa: E402
from highperformanceseismicstacking_gb300.su import tau_index  # noqa: E402
from oracle import ref_runner  # noqa: E402


def time_ls(n_mid: int = 20):
    import torch
    w = synthetic.WORKLOADS["cmp-production"]
    line = w.make_line(n_cmp=n_mid)
    tau = tau_index(w.tau, line.dt)
    rk = ref_runner.ReferenceKernels()
    params = rk.build_grid("cmp", w.lower, w.upper, w.granularity)
    S = line.samples_per_trace
    P = params.shape[0]
    mod = rk.d.module("cmp_linear_search")
    comp = mod["computeSemblancesForCommonMidPoint"]
    best = mod["selectBestSemblancesForCommonMidPoint"]
    dp = torch.from_numpy(params.ravel().copy()).cuda()
    sem = torch.zeros(S * P, device="cuda")
    stk = torch.zeros(S * P, device="cuda")
    res = torch.zeros(3 * S, device="cuda")
    total_ms = 0.0
    evals = 0.0
    g = ref_runner._grid(S * P)
    gb = ref_runner._grid(S)
    for i, m0 in enumerate(line.cdp_midpoints):
        sel = np.nonzero(line.midpoints == m0)[0]
        smp = torch.from_numpy(np.ascontiguousarray(line.samples[sel]).ravel()).cuda()
        h = line.halfoffsets[sel]
        h2 = torch.from_numpy((h * h).astype(np.float32)).cuda()
        args = [C.c_void_p(smp.data_ptr()), C.c_void_p(h2.data_ptr()), C.c_uint(sel.size),
                C.c_uint(S), C.c_float(float(line.dt)), C.c_int(tau), C.c_int(2 * tau + 1),
                C.c_void_p(dp.data_ptr()), C.c_uint(P), C.c_void_p(sem.data_ptr()),
                C.c_void_p(stk.data_ptr())]
        bargs = [C.c_void_p(sem.data_ptr()), C.c_void_p(stk.data_ptr()),
                 C.c_void_p(dp.data_ptr()), C.c_uint(P), C.c_uint(S), C.c_void_p(res.data_ptr())]
        if i == 0:  # warm-up
            rk.d.launch(comp, g, ref_runner.THREADS, args)
            rk.d.launch(best, gb, ref_runner.THREADS, bargs)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        rk.d.launch(comp, g, ref_runner.THREADS, args)
        rk.d.launch(best, gb, ref_runner.THREADS, bargs)
        e1.record()
        torch.cuda.synchronize()
        total_ms += e0.elapsed_time(e1)
        evals += float(sel.size) * S * P
    print(json.dumps({"impl": "reference CUDA kernels (sm_103a build of the reference sources)",
                      "workload": "cmp-production", "algorithm": "linear-search",
                      "midpoints": n_mid, "evals": evals, "kernel_ms": total_ms,
                      "value": evals / (total_ms / 1e3), "unit": "evals/s"}))


def time_zocrs(n_mid: int = 2):
    """ZO-CRS linear search on the ZO-CRS line (1000 CMPs, +-15-CMP aperture,
    21 x 21 x 41 candidates, window 5): the reference's evaluation + argmax
    per midpoint (computeSemblancesForZeroOffsetCommonReflectionSurface +
    selectBest..., CudaLinearSearchAlgorithm.cu:35-163) against the engine's
    plain and tuned kernels on the same midpoints."""
    w = synthetic.WORKLOADS["zocrs-ls"]
    line = w.make_line()
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    rk = ref_runner.ReferenceKernels()
    params = rk.build_grid("zocrs", lower, upper, w.granularity)
    S = line.samples_per_trace
    mid = len(line.cdp_midpoints) // 2
    m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_mid])
    ref_ms, ref_evals, ref_out = 0.0, 0.0, []
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(rk.select("zocrs", line.midpoints, line.halfoffsets, float(m0), w.apm,
                                   0.0, S, float(line.dt)))[0]
        call = lambda: rk.linear_search_midpoint("zocrs", line.samples, line.midpoints,
                                                 line.halfoffsets, sel, float(m0),
                                                 float(line.dt), tau, params, w.apm, 0.0,
                                                 timing=True)
        if i == 0:
            call()  # warm-up (module load)
        res, _, _, _, ms = call()
        ref_ms += ms
        ref_evals += float(sel.size) * S * params.shape[0]
        ref_out.append(res)
    out = {"workload": "zocrs-ls (1000-CMP ZO-CRS line, 21 x 21 x 41 candidates, window 5)",
           "midpoints": int(len(m0s)), "samples": S,
           "reference": {"ms": ref_ms, "evals": ref_evals, "value": ref_evals / (ref_ms / 1e3)}}
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("zocrs", lower, upper, w.apm)
        eng.set_window(tau)
        for kernel in ("plain", "tuned"):
            eng.linear_search(m0s, w.granularity, kernel)
            got, st = eng.linear_search(m0s, w.granularity, kernel)
            same = float(np.mean(np.all(got[:, 2:] == np.stack(ref_out)[:, 2:], axis=1)))
            out[kernel] = {"ms": st["kernel_ms"], "evals": st["evals"],
                           "value": st["evals"] / (st["kernel_ms"] / 1e3),
                           "parameters_equal_to_reference": same,
                           "speedup_vs_reference": ref_ms / st["kernel_ms"]}
    print(json.dumps(out))


def time_de(n_mid: int = 2, oct_h0=None):
    rk = ref_runner.ReferenceKernels()
    ops = "common_differential_evolution_f05cr09"
    for name in ("zocrs-de", "oct-de"):
        w = synthetic.WORKLOADS[name]
        h0 = float(oct_h0) if (name == "oct-de" and oct_h0 is not None) else w.h0
        line = w.make_line()
        lower, upper = synthetic.workload_bounds(w)
        tau = tau_index(w.tau, line.dt)
        S = line.samples_per_trace
        mid = len(line.cdp_midpoints) // 2
        m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_mid])
        ref_ms, ref_evals, ref_best = 0.0, 0.0, []
        for i, m0 in enumerate(m0s):
            sel = None
            if w.model == "zocrs":
                sel = np.nonzero(np.abs(np.float32(m0) - line.midpoints) <= np.float32(w.apm))[0]
            res, ms, n_sel = rk.differential_evolution_midpoint(
                w.model, line.samples, line.midpoints, line.halfoffsets, float(m0),
                float(line.dt), tau, lower, upper, w.population, w.generations, seed=11 + i,
                apm=w.apm, h0=h0, sel=sel, operators=ops)
            ref_ms += ms
            ref_best.append(res[0])
            ref_evals += float(n_sel) * S * w.population * w.generations
        with capi.Engine(0) as eng:
            eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
            eng.set_traveltime(w.model, lower, upper, w.apm, h0)
            eng.set_window(tau)
            eng.differential_evolution(m0s, w.population, 2, w.de_f, w.de_cr, seed=1)
            got, st = eng.differential_evolution(m0s, w.population, w.generations, w.de_f,
                                                 w.de_cr, seed=7)
        line_out = {"workload": name, "algorithm": "differential-evolution", "h0": h0,
                    "midpoints": int(len(m0s)), "samples": S, "population": w.population,
                    "generations": w.generations,
                    "reference": {"ms": ref_ms,
                                  "mean_best_semblance": float(np.mean(ref_best))},
                    "engine": {"ms": st["kernel_ms"], "evals": st["evals"],
                               "value": st["evals"] / (st["kernel_ms"] / 1e3),
                               "mean_best_semblance": float(np.mean(got[:, 0]))},
                    "speedup_engine_vs_reference": ref_ms / st["kernel_ms"]}
        line_out["reference"]["evals"] = ref_evals
        line_out["reference"]["value"] = ref_evals / (ref_ms / 1e3)
        print(json.dumps(line_out))


def time_oct(n_mid: int = 1, h0=None):
    """OCT linear search (the OCT DE line's geometry, 11 x 5 candidates,
    h0 = 0 unless given): the reference's per-midpoint evaluation + argmax against the
    engine's plain and tuned kernels on the same midpoints."""
    from oracle import oracle
    w = synthetic.WORKLOADS["oct-de"]
    h0 = w.h0 if h0 is None else float(h0)
    line = w.make_line(n_cmp=60)
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    gran = [11, 5]
    rk = ref_runner.ReferenceKernels()
    params = rk.build_grid("oct", lower, upper, gran)
    cands = oracle.oct_selection_candidates(lower, upper)
    S = line.samples_per_trace
    mid = len(line.cdp_midpoints) // 2
    m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_mid])
    ref_ms, ref_evals, ref_out = 0.0, 0.0, []
    for m0 in m0s:
        sel = np.nonzero(rk.select("oct", line.midpoints, line.halfoffsets, float(m0), w.apm,
                                   h0, S, float(line.dt), cands))[0]
        res, _, _, _, ms = rk.linear_search_midpoint("oct", line.samples, line.midpoints,
                                                     line.halfoffsets, sel, float(m0),
                                                     float(line.dt), tau, params, w.apm, h0,
                                                     timing=True)
        ref_ms += ms
        ref_evals += float(sel.size) * S * params.shape[0]
        ref_out.append(res)
    out = {"workload": "oct-ls (OCT DE line geometry, 60 CMPs, 11 x 5 candidates)", "h0": h0,
           "midpoints": int(len(m0s)), "samples": S,
           "reference": {"ms": ref_ms, "evals": ref_evals, "value": ref_evals / (ref_ms / 1e3)}}
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("oct", lower, upper, w.apm, h0)
        eng.set_window(tau)
        for kernel in ("plain", "tuned"):
            eng.linear_search(m0s, gran, kernel)
            got, st = eng.linear_search(m0s, gran, kernel)
            same = float(np.mean(np.isclose(got[:, 2], np.stack(ref_out)[:, 2], rtol=1e-6)))
            out[kernel] = {"ms": st["kernel_ms"], "evals": st["evals"],
                           "value": st["evals"] / (st["kernel_ms"] / 1e3),
                           "velocity_equal_to_reference": same}
    print(json.dumps(out))


def time_sf(n_mid: int = 20):
    """CMP stretch-free stack (21 n values, window 7) on the CMP production
    line, prior velocities from the engine's linear search: the reference's
    per-midpoint evaluation + argmax against the engine's stretch-free."""
    w = synthetic.WORKLOADS["cmp-production"]
    line = w.make_line(n_cmp=n_mid)
    tau = tau_index(w.tau, line.dt)
    S = line.samples_per_trace
    m0s = line.cdp_midpoints
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("cmp", w.lower, w.upper)
        eng.set_window(tau)
        ls, _ = eng.linear_search(m0s, w.granularity, "tuned")
        prior = np.ascontiguousarray(ls[:, 2:3, :])
        eng.stretch_free(m0s, prior)
        got, st = eng.stretch_free(m0s, prior)
    rk = ref_runner.ReferenceKernels()
    ref_ms, evals, same = 0.0, 0.0, []
    for i, m0 in enumerate(m0s):
        sel = np.nonzero(line.midpoints == m0)[0]
        res, ms = rk.stretch_free_midpoint_cmp(line.samples, line.halfoffsets, sel,
                                               float(line.dt), tau, prior[i, 0], timing=True)
        ref_ms += ms
        evals += float(sel.size) * S * 21
        same.append(np.array_equal(res, got[i]))
    print(json.dumps({"workload": "cmp-production stretch-free (21 n)", "midpoints": int(n_mid),
                      "reference": {"ms": ref_ms, "value": evals / (ref_ms / 1e3)},
                      "engine": {"ms": st["kernel_ms"], "value": evals / (st["kernel_ms"] / 1e3)},
                      "identical_to_reference": bool(all(same)),
                      "speedup_engine_vs_reference": ref_ms / st["kernel_ms"]}))


if __name__ == "__main__":
    mode = sys.argv[1] if len(sys.argv) > 1 else "ls"
    n = int(sys.argv[2]) if len(sys.argv) > 2 else {"ls": 20, "de": 2, "oct": 1, "sf": 20,
                                                      "zocrs": 2}[mode]
    if mode == "ls":
        time_ls(n)
    elif mode == "zocrs":
        time_zocrs(n)
    elif mode == "de":
        time_de(n, float(sys.argv[3]) if len(sys.argv) > 3 else None)
    elif mode == "oct":
        time_oct(n, float(sys.argv[3]) if len(sys.argv) > 3 else None)
    elif mode == "sf":
        time_sf(n)
    else:
        raise SystemExit(f"unknown mode {mode}")
