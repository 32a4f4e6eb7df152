#!/usr/bin/env python3
"""Benchmark: semblance evaluations per second (trace x sample x candidate).

Workload (default): CMP linear search at production size -- 2000 CMPs, fold
60 (half-offsets 0..2950 m), 2000 samples at dt = 2 ms, 401 velocities
1000..6000 m/s, window 7.  One step = the whole line in one call.

  value : device-resident line and midpoints, the tuned kernel, timed with CUDA
          events on the engine's stream (the line, 960 MB, exceeds the 129 MB L2
          so no flush is needed between steps);
  e2e   : the same step through the public C ABI with host buffers, one call of
          hpss_linear_search_line: the line goes up from page-locked memory in
          trace ranges while the midpoints whose traces have arrived are
          searched, and the results come back to a page-locked block;
  plain : the plain one-(sample, candidate)-per-thread FP32 kernel, same line.

`--impl reference` times the reference algorithm on the host CPU (the oracle's
C restatement, all cores): the reference's only CPU path is its OpenCL build
on a host OpenCL device, which this machine does not have.  Beside it, the
same line carries `reference_cuda`: the reference's own CUDA kernels (built
from its sources) timed on the same GPU over the midpoints of this arm's
side measurements.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "semblance evals/s (trace*sample*param), tuned vs plain, 1 GB300, <=1e-4 err"
UNIT = "evals/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="cmp-production")
    ap.add_argument("--n-cmp", type=int, default=None, help="smaller line (profiling only)")
    ap.add_argument("--plain-steps", type=int, default=1)
    ap.add_argument("--e2e-steps", type=int, default=2)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--de-cmps", type=int, default=2,
                    help="midpoints of the OCT DE side measurement (0: skip)")
    ap.add_argument("--zocrs-de-cmps", type=int, default=16,
                    help="midpoints of the ZO-CRS DE side measurement (16 midpoints x 1500 "
                         "samples = 1500 CTAs of sixteen populations, about 2.5 waves)")
    ap.add_argument("--per-midpoint-calls", type=int, default=64,
                    help="one-midpoint calls timed beside the batched call (0: skip)")
    ap.add_argument("--no-storage-side", action="store_true",
                    help="skip the BF16 / FP16 storage side measurement")
    ap.add_argument("--zocrs-cmps", type=int, default=32,
                    help="midpoints of the ZO-CRS line measured beside the main workload "
                         "(0 = skip); 32 midpoints = 1504 (midpoint, tile) units, about five "
                         "waves of the persistent grid, so the last partial wave is small")
    ap.add_argument("--oct-cmps", type=int, default=4,
                    help="midpoints of the OCT linear-search side measurement (0: skip)")
    ap.add_argument("--c5-cmps", type=int, default=2,
                    help="midpoints of the OCT DE + stretch-free pipeline over three h0 "
                         "(0: skip)")
    ap.add_argument("--fp64-cmps", type=int, default=7,
                    help="midpoints of the ZO-CRS line (1500 samples each) on which every "
                         "FP32 mode is compared with the FP64 search (0: skip)")
    ap.add_argument("--sf-cmps", type=int, default=2000,
                    help="midpoints of the CMP stretch-free side measurement (0: skip); "
                         "the default is the whole production line")
    ap.add_argument("--no-io-side", action="store_true", help="skip the SU input/output side")
    ap.add_argument("--no-whole-lines", action="store_true",
                    help="skip the whole-line ZO-CRS DE (500 midpoints) and ZO-CRS linear "
                         "search (1000 midpoints, about a minute) calls")
    ap.add_argument("--no-reference-cuda", action="store_true",
                    help="reference arm: skip timing the reference's CUDA kernels")
    ap.add_argument("--profile-case", default=None, choices=sorted(PROFILE_CASES),
                    help="run one small case of one kernel instead of the benchmark: a "
                         "warm-up call, then the call an ncu capture takes "
                         "(-k <kernel> -s 1 -c 1)")
    return ap.parse_args()


# ----------------------------------------------------------------- helpers

def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except (OSError, FileNotFoundError):
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        return json.loads(p.read_text())
    return {"hbm_gbs": 6800.0, "sm_max_mhz": 2070.0, "fallback": True}


def profile_traffic(kernel_tag: str):
    """DRAM bytes per launch of the dominant kernel from the committed ncu
    summary (profiles/<kernel_tag>.md, line 'traffic_bytes_per_launch: N')."""
    p = ROOT / "profiles" / f"{kernel_tag}.md"
    if not p.exists():
        return None, None
    scale = None
    val = None
    for ln in p.read_text().splitlines():
        if ln.startswith("traffic_bytes_per_launch:"):
            try:
                val = float(ln.split(":", 1)[1].split()[0])
            except ValueError:
                pass
        if ln.startswith("traffic_scale_units:"):
            scale = ln.split(":", 1)[1].strip()
    return val, scale


# ----------------------------------------------------------------- workload

_LINES = {}


def make_workload(name: str, n_cmp=None):
    """A workload's settings and its seeded synthetic line (generated once
    per process and shared by the measurements that use it)."""
    from highperformanceseismicstacking_gb300 import synthetic
    from highperformanceseismicstacking_gb300.su import tau_index
    w = synthetic.WORKLOADS[name]
    key = (name, n_cmp)
    if key not in _LINES:
        _LINES[key] = w.make_line(n_cmp=n_cmp)
    line = _LINES[key]
    lower, upper = synthetic.workload_bounds(w)
    tau = tau_index(w.tau, line.dt)
    return w, line, lower, upper, tau


def evals_per_step(counts, S, P):
    return float(np.sum(counts)) * S * P


def compare_outputs(a, b):
    """Tuned result table a against b ([nM0][2+np][S]): semblance and chosen
    parameters identical?  Largest stack difference relative to
    |b| + max |b| of the midpoint (the tuned kernel sums the linear sum in
    another order)."""
    same = bool(np.array_equal(a[:, 0], b[:, 0]) and np.array_equal(a[:, 2:], b[:, 2:]))
    sa, sb = a[:, 1].astype(np.float64), b[:, 1].astype(np.float64)
    scale = np.abs(sb) + np.max(np.abs(sb), axis=1, keepdims=True)
    err = float(np.max(np.abs(sa - sb) / np.maximum(scale, 1e-30))) if sa.size else 0.0
    return {"semblance_and_parameters_identical": same, "stack_max_rel_err": err,
            "all_identical": bool(np.array_equal(a, b))}


def zocrs_side_measure(n_cmp, local):
    """ZO-CRS linear search on midpoints of the 1000-CMP ZO-CRS line (full
    +-15-CMP apertures, 21 x 21 x 41 grid): tuned vs plain, device-resident,
    CUDA events on the engine's stream."""
    import torch
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("zocrs-ls")
    P = int(np.prod(w.granularity))
    mid = len(line.cdp_midpoints) // 2
    m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_cmp])
    eng = capi.Engine(local)
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
    eng.set_window(tau)
    evals = evals_per_step(eng.select_traces(m0s), line.samples_per_trace, P)
    dev = torch.device("cuda", local)
    d_m0 = torch.from_numpy(m0s).to(dev)
    outs = {}
    res = {}
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)
    for kernel in ("tuned", "plain"):
        d_out = torch.empty((len(m0s), 2 + eng.np, line.samples_per_trace), dtype=torch.float32,
                            device=dev)
        ms = time_call(eng, stream, d_m0, len(m0s), w.granularity, d_out, kernel)
        res[kernel] = {"value": evals / (ms / 1e3), "ms": ms}
        outs[kernel] = d_out.cpu().numpy()
    storage = storage_side(eng, line, stream, d_m0, len(m0s), w.granularity, evals,
                           outs["tuned"])
    eng.close()
    # FP32-pipe roofline of the tuned kernel (3w + 5 instructions per eval)
    props = torch.cuda.get_device_properties(dev)
    peak = props.multi_processor_count * 128 * float(measured_peaks().get("sm_max_mhz", 2070.0)) * 1e6
    instr = 3 * (2 * tau + 1) + 5
    res["tuned"]["roofline_frac"] = res["tuned"]["value"] * instr / peak
    res["tuned"]["roofline"] = fp32_roofline("zocrs", 2 * tau + 1, evals, 0.0,
                                             res["tuned"]["ms"], local)
    return {"workload": "zocrs-ls", "cmps": int(len(m0s)), "evals": evals,
            "candidates": P, "mean_traces_per_midpoint": evals / P / line.samples_per_trace / len(m0s),
            "tuned": res["tuned"], "plain": res["plain"],
            "speedup_tuned_vs_plain": res["tuned"]["value"] / res["plain"]["value"],
            "tuned_vs_plain": compare_outputs(outs["tuned"], outs["plain"]),
            "storage": storage}


def whole_workloads_side(local):
    """Two workloads end to end in one call each: C4, the ZO-CRS DE over all
    500 midpoints of the ZO-CRS DE line (population 32, 60 generations), and
    C3, the tuned ZO-CRS linear search over all 1000 midpoints of the ZO-CRS
    line (21 x 21 x 41 candidates).  Each after a short warm-up call on the
    same engine (module load, autotuning); device time from the engine's
    events, wall time of the call on the host."""
    from highperformanceseismicstacking_gb300 import capi
    out = {}
    w, line, lower, upper, tau = make_workload("zocrs-de")
    m0s = np.ascontiguousarray(line.cdp_midpoints)
    with capi.Engine(local) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
        eng.set_window(tau)
        eng.differential_evolution(m0s[:8], w.population, 2, w.de_f, w.de_cr, seed=1)
        t0 = time.perf_counter()
        res, st = eng.differential_evolution(m0s, w.population, w.generations, w.de_f, w.de_cr,
                                             seed=7)
        wall = time.perf_counter() - t0
    sel = st["selected_traces"]
    out["zocrs_de_whole_line"] = {
        "cmps": int(len(m0s)), "population": w.population, "generations": w.generations,
        "evals": st["evals"], "kernel_ms": st["kernel_ms"], "selection_ms": st["selection_ms"],
        "call_wall_s": wall, "value": st["evals"] / (st["kernel_ms"] / 1e3),
        "mean_best_semblance": float(np.mean(res[:, 0])),
        "roofline": fp32_roofline(w.model, 2 * tau + 1, st["evals"], 0.0, st["kernel_ms"], local,
                                  alg_bytes=sel * line.samples_per_trace * 4 + sel * 16)}
    w, line, lower, upper, tau = make_workload("zocrs-ls")
    m0s = np.ascontiguousarray(line.cdp_midpoints)
    with capi.Engine(local) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
        eng.set_window(tau)
        mid = len(m0s) // 2
        eng.linear_search(m0s[mid:mid + 4], w.granularity, "tuned")
        t0 = time.perf_counter()
        _, st = eng.linear_search(m0s, w.granularity, "tuned")
        wall = time.perf_counter() - t0
    out["zocrs_ls_whole_line"] = {
        "cmps": int(len(m0s)), "candidates": int(np.prod(w.granularity)), "evals": st["evals"],
        "kernel_ms": st["kernel_ms"], "selection_ms": st["selection_ms"], "call_wall_s": wall,
        "kernel_variant": st["kernel_variant"], "value": st["evals"] / (st["kernel_ms"] / 1e3),
        "roofline": fp32_roofline("zocrs", 2 * tau + 1, st["evals"], 0.0, st["kernel_ms"],
                                  local)}
    return out


def de_side_measure(n_cmp, local, n_cmp_zocrs=None):
    """Fused differential evolution on midpoints of the DE workloads: ZO-CRS
    (500-CMP line, 1500 samples, population 32, 60 generations, F 0.5, CR 0.9)
    and OCT (800-CMP line, 3000 samples, population 48, 80 generations,
    h0 = 0).  Device time of the DE launch from the engine's own events."""
    from highperformanceseismicstacking_gb300 import capi
    out = {}
    for name in ("zocrs-de", "oct-de"):
        w, line, lower, upper, tau = make_workload(name)
        mid = len(line.cdp_midpoints) // 2
        k = n_cmp_zocrs if (name == "zocrs-de" and n_cmp_zocrs) else n_cmp
        m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + k])
        with capi.Engine(local) as eng:
            eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
            eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
            eng.set_window(tau)
            eng.differential_evolution(m0s, w.population, 2, w.de_f, w.de_cr, seed=1)
            res, st = eng.differential_evolution(m0s, w.population, w.generations, w.de_f,
                                                 w.de_cr, seed=7)
        sel = st["selected_traces"]
        out[name] = {"cmps": int(len(m0s)), "samples": line.samples_per_trace,
                     "population": w.population, "generations": w.generations,
                     "evals": st["evals"], "not_used": st["not_used"],
                     "kernel_ms": st["kernel_ms"], "selection_ms": st["selection_ms"],
                     "value": st["evals"] / (st["kernel_ms"] / 1e3),
                     "mean_best_semblance": float(np.mean(res[:, 0])),
                     "roofline": fp32_roofline(w.model, 2 * tau + 1, st["evals"], st["not_used"],
                                               st["kernel_ms"], local,
                                               alg_bytes=sel * line.samples_per_trace * 4 +
                                               sel * 16)}
    return out


def oct_ls_side(n_cmp, local):
    """OCT linear search on midpoints of the OCT DE workload's line (11 x 5
    candidates over the workload's bounds, window 9, h0 0): tuned vs plain,
    device time from the engine's events (the first call tunes / loads)."""
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("oct-de")
    mid = len(line.cdp_midpoints) // 2
    m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_cmp])
    gran = [11, 5]
    S = line.samples_per_trace
    out = {"cmps": int(len(m0s)), "candidates": 55, "window": 2 * tau + 1, "h0": 0.0}
    with capi.Engine(local) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("oct", lower, upper, w.apm, 0.0)
        eng.set_window(tau)
        res = {}
        for kernel in ("tuned", "plain"):
            eng.linear_search(m0s, gran, kernel)
            got, st = eng.linear_search(m0s, gran, kernel)
            res[kernel] = got
            sel = st["selected_traces"]
            out[kernel] = {"kernel_ms": st["kernel_ms"], "selection_ms": st["selection_ms"],
                           "evals": st["evals"], "not_used": st["not_used"],
                           "value": st["evals"] / (st["kernel_ms"] / 1e3),
                           "roofline": fp32_roofline("oct", 2 * tau + 1, st["evals"],
                                                     st["not_used"], st["kernel_ms"], local,
                                                     alg_bytes=sel * S * 4 + sel * 16)}
    out["speedup_tuned_vs_plain"] = out["plain"]["kernel_ms"] / out["tuned"]["kernel_ms"]
    out["tuned_equals_plain"] = bool(np.array_equal(res["tuned"], res["plain"]))
    return out


def sf_side(n_cmp, local):
    """CMP stretch-free stack (n in [-10, 10], window 7) on midpoints of the
    CMP production line over the tuned search's velocities."""
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("cmp-production")
    m0s = np.ascontiguousarray(line.cdp_midpoints[:n_cmp])
    S = line.samples_per_trace
    with capi.Engine(local) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("cmp", lower, upper)
        eng.set_window(tau)
        ls, _ = eng.linear_search(m0s, w.granularity, "tuned")
        prior = np.ascontiguousarray(ls[:, 2:3])
        eng.stretch_free(m0s, prior, 10)
        sf, st = eng.stretch_free(m0s, prior, 10)
    sel = st["selected_traces"]
    return {"cmps": int(n_cmp), "n_values": 21, "window": 2 * tau + 1,
            "kernel_ms": st["kernel_ms"], "evals": st["evals"],
            "value": st["evals"] / (st["kernel_ms"] / 1e3),
            "roofline": fp32_roofline("cmp", 2 * tau + 1, st["evals"], 0.0, st["kernel_ms"],
                                      local, extra_per_eval=1,
                                      alg_bytes=sel * S * 4 + sel * 8 + n_cmp * 4 * S * 4)}


def su_io_side(line, d_out, n_m0, rows, S, n_cmp=200):
    """SU input / output throughput on the host: the line's first n_cmp CMP
    gathers written as one SU file and read back with the reference's gather
    semantics (su.read_gather: filters, CDP map, sort), and the result files
    of the whole line (rows SU files of one trace per CDP) written from the
    device result slab by the batched writer (hpss_write_result_files)
    against the reference's per-CDP loop of header and trace writes
    (Dumper::dumpResult, common/src/output/Dumper.cpp:77-114), restated in
    Python."""
    import shutil
    import tempfile
    from highperformanceseismicstacking_gb300 import capi, su
    tmp = Path(tempfile.mkdtemp(prefix="hpss_su_"))
    try:
        sel = np.isin(line.midpoints, line.cdp_midpoints[:n_cmp])
        hdr, smp = line.headers[sel], line.samples[sel]
        path = tmp / "line.su"
        t0 = time.perf_counter()
        su.write_su(str(path), hdr, smp)
        t_w = time.perf_counter() - t0
        nbytes = path.stat().st_size
        t0 = time.perf_counter()
        g = su.read_gather(str(path), aph=1e9, apm=0.0, tau=0.0, emulate_eof_cdp=False)
        t_r = time.perf_counter() - t0
        assert g.trace_count == smp.shape[0]
        # result files of the whole line from the device slab
        cdp_hdr = np.zeros(n_m0, su.SU_HEADER_DTYPE)
        cdp_hdr["ns"] = S
        cdp_hdr["cdp"] = np.arange(1, n_m0 + 1)
        paths = [str(tmp / f"r{r}.su") for r in range(rows)]
        slab_shape = np.empty((n_m0, rows, S), np.float32)  # shape only
        t0 = time.perf_counter()
        capi.write_result_files(slab_shape, cdp_hdr, paths, device_ptr=d_out.data_ptr())
        t_b = time.perf_counter() - t0
        res_bytes = sum(Path(p).stat().st_size for p in paths)
        host = d_out.cpu().numpy()
        t0 = time.perf_counter()
        for r in range(rows):
            with open(tmp / f"loop{r}.su", "wb") as f:
                for i in range(n_m0):
                    f.write(cdp_hdr[i].tobytes())
                    f.write(host[i, r].tobytes())
        t_l = time.perf_counter() - t0
        same = all((tmp / f"loop{r}.su").read_bytes() == Path(paths[r]).read_bytes()
                   for r in range(rows))
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return {"line_sample": f"{n_cmp} CMP gathers, {smp.shape[0]} traces, {nbytes / 1e6:.0f} MB",
            "write_su_MBps": nbytes / t_w / 1e6, "read_gather_MBps": nbytes / t_r / 1e6,
            "result_files": {"files": rows, "bytes": res_bytes,
                             "batched_from_device_MBps": res_bytes / t_b / 1e6,
                             "per_cdp_loop_MBps": res_bytes / t_l / 1e6,
                             "identical_bytes": bool(same)}}


# Algorithmic FP32-pipe instructions per evaluation (one (m0, t0, candidate,
# selected trace) tuple): 3 per window tap (interpolation with a precomputed
# slope, numerator add, denominator fma) plus the traveltime -- 2 CMP, 5
# ZO-CRS, 40 OCT (displaced midpoint and time).  An OCT trace that fails the
# displaced-midpoint test costs the test alone: 9 (its per-(t0, candidate,
# trace) operations once the trace-only and candidate-only factors are
# hoisted).  Stretch-free adds the time shift (1).
T_MODEL = {"cmp": 2, "zocrs": 5, "oct": 40}
T_OCT_SKIP = 9


def fp32_roofline(model, w, evals, not_used, ms, local, extra_per_eval=0, alg_bytes=None):
    """FP32-pipe roofline of one launch: algorithmic instructions / time over
    SMs x 128 lanes x max SM clock; plus the HBM view of its algorithmic
    bytes when given."""
    import torch
    peaks = measured_peaks()
    sms = torch.cuda.get_device_properties(local).multi_processor_count
    peak = sms * 128 * float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    used = evals - not_used
    instr = used * (3 * w + T_MODEL[model] + extra_per_eval) + not_used * T_OCT_SKIP
    r = {"bound": "fp32", "achieved": instr / (ms / 1e3) / 1e12, "peak": peak / 1e12,
         "unit": "Tinstr/s", "frac": instr / (ms / 1e3) / peak, "kernel_ms": ms,
         "instr_per_launch": instr}
    if alg_bytes is not None:
        hbm = float(peaks.get("hbm_gbs", 6800.0))
        gbs = alg_bytes / (ms / 1e3) / 1e9
        r["hbm"] = {"achieved": gbs, "peak": hbm, "unit": "GB/s", "frac": gbs / hbm,
                    "bytes_per_launch": alg_bytes}
    return r


def c5_side_measure(n_cmp, local, h0s=(0.0, 500.0, 1000.0), storages=("fp16", "fp32")):
    """The OCT DE workload as one pipeline on a bounded sample of its
    midpoints: OCT differential evolution (population 48, 80 generations, F
    0.5, CR 0.9, window 9) over every target half-offset in ONE launch, then
    the stretch-free stack (window 9, n in [-10, 10]) over the chosen
    parameters in one launch; FP16 amplitude storage (the workload's) and
    FP32 storage for comparison.  Device time from the engine's events."""
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("oct-de")
    mid = len(line.cdp_midpoints) // 2
    m0s = np.ascontiguousarray(line.cdp_midpoints[mid:mid + n_cmp])
    S = line.samples_per_trace
    wsz = 2 * tau + 1
    out = {"cmps": int(len(m0s)), "h0s": list(h0s), "samples": S, "population": w.population,
           "generations": w.generations, "window": wsz, "launches_per_pipeline": None}
    res = {}
    for storage in storages:
        with capi.Engine(local) as eng:
            eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                              storage=storage)
            eng.set_traveltime("oct", lower, upper, w.apm, 0.0)
            eng.set_window(tau)
            eng.set_oct_half_offsets(list(h0s))
            eng.differential_evolution(m0s, w.population, 2, w.de_f, w.de_cr, seed=1)
            de, st = eng.differential_evolution(m0s, w.population, w.generations, w.de_f,
                                                w.de_cr, seed=7)
            prior = np.ascontiguousarray(de[:, 2:])
            sf, st2 = eng.stretch_free(m0s, prior, 10)
            dev_bytes = eng.device_bytes()
        sel = st["selected_traces"]
        bpv = 2 if storage != "fp32" else 4
        de_bytes = sel * S * bpv + sel * 16
        r = {"de": {"kernel_ms": st["kernel_ms"], "selection_ms": st["selection_ms"],
                    "evals": st["evals"], "not_used": st["not_used"],
                    "value": st["evals"] / (st["kernel_ms"] / 1e3),
                    "mean_best_semblance": float(np.mean(de[:, 0])),
                    "roofline": fp32_roofline("oct", wsz, st["evals"], st["not_used"],
                                              st["kernel_ms"], local, alg_bytes=de_bytes)},
             "stretch_free": {"kernel_ms": st2["kernel_ms"], "selection_ms": st2["selection_ms"],
                              "evals": st2["evals"], "not_used": st2["not_used"],
                              "value": st2["evals"] / (st2["kernel_ms"] / 1e3),
                              "mean_semblance": float(np.mean(sf[:, 0])),
                              "roofline": fp32_roofline("oct", wsz, st2["evals"], st2["not_used"],
                                                        st2["kernel_ms"], local, extra_per_eval=1)},
             "device_bytes": dev_bytes}
        r["pipeline_ms"] = (st["kernel_ms"] + st["selection_ms"] + st2["kernel_ms"] +
                            st2["selection_ms"])
        res[storage] = (r, de, sf)
    for storage in storages:
        out[storage] = res[storage][0]
    if "fp16" in res and "fp32" in res:
        d16, d32 = res["fp16"][1], res["fp32"][1]
        strong = d32[:, 0] > 0.1
        out["fp16_vs_fp32"] = {
            "de_median_best_semblance_ratio": float(np.median(d16[:, 0][strong] /
                                                              d32[:, 0][strong])),
            "de_speedup": res["fp32"][0]["de"]["kernel_ms"] / res["fp16"][0]["de"]["kernel_ms"]}
    # per pipeline: DE selection (flags + compaction), DE, stretch-free
    # selection (flags + compaction), stretch-free
    out["launches_per_pipeline"] = 6
    return out


def fp64_agreement_side(n_mid, local):
    """Chosen parameters of every FP32 mode against the FP64 reference on
    n_mid midpoints of the ZO-CRS line (every sample of each, 21 x 21 x 41
    candidates, window 5): the FP64 reference is the search with every step
    in FP64 on the device (HPSS_PREC_FP64).  Per mode, a sample is
    'agree' (the FP64 choice), 'near_tie' (another candidate whose FP64
    semblance is within 1e-4 x max(best, 1e-3) of the FP64 best -- evaluated
    by the FP64 stretch-free pass with n = 0 on both choices) or 'changed'.
    Modes: FP32 (the reference's arithmetic), FP64 traveltime, compensated
    sums, both (tuned kernels), and BF16 / FP16 amplitude storage."""
    import torch
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("zocrs-ls")
    cdp = line.cdp_midpoints
    pick = np.linspace(40, len(cdp) - 41, n_mid).round().astype(int)
    m0s = np.ascontiguousarray(cdp[pick])
    S = line.samples_per_trace
    gran = w.granularity
    eng = capi.Engine(local)
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
    eng.set_window(tau)
    eng.set_precision(fp64=True)
    t0 = time.perf_counter()
    ref, st64 = eng.linear_search(m0s, gran, "plain")
    fp64_s = time.perf_counter() - t0

    def semb64(params):
        # FP64 semblance of explicit per-sample parameters (raw) at n = 0
        out, _ = eng.stretch_free(m0s, np.ascontiguousarray(params), 0)
        return out[:, 0].astype(np.float64)

    s_best = semb64(ref[:, 2:])
    modes = {"fp32": {}, "fp64_traveltime": {"fp64_traveltime": True},
             "compensated": {"compensated": True},
             "fp64_traveltime+compensated": {"fp64_traveltime": True, "compensated": True}}
    outs = {}
    for name, kw in modes.items():
        eng.set_precision(**kw)
        outs[name], _ = eng.linear_search(m0s, gran, "tuned")
    eng.set_precision()
    for storage in ("bf16", "fp16"):
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          storage=storage)
        outs[storage], _ = eng.linear_search(m0s, gran, "tuned")
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    res = {"midpoints": int(n_mid), "samples": int(n_mid * S), "candidates": int(np.prod(gran)),
           "fp64_reference_s": fp64_s, "fp64_reference_evals": st64["evals"],
           "fp64_near_ties": st64["near_ties"], "modes": {}}
    eng.set_precision(fp64=True)
    for name, got in outs.items():
        diff = np.any(got[:, 2:] != ref[:, 2:], axis=1)  # [nM0][S]
        n = int(diff.sum())
        near = 0
        if n:
            s_alt = semb64(got[:, 2:])
            tol = 1e-4 * np.maximum(s_best, 1e-3)
            near = int(np.sum(diff & (s_alt >= s_best - tol)))
        tot = diff.size
        res["modes"][name] = {"changed": (n - near) / tot, "near_tie": near / tot,
                              "agree": 1.0 - n / tot,
                              "meets_99_9": (n - near) / tot <= 1e-3}
    eng.set_precision()
    eng.close()
    return res


def _case_ls(workload, n_cmp, mid_count, gran=None, storage="fp32", kernel="tuned",
             fp64=False):
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload(workload, n_cmp)
    m0s = line.cdp_midpoints
    if mid_count:
        mid = len(m0s) // 2
        m0s = m0s[mid:mid + mid_count]
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          storage=storage)
        eng.set_traveltime(w.model, lower, upper, w.apm, 0.0)
        eng.set_window(tau)
        if fp64:
            eng.set_precision(fp64=True)
        for _ in range(2):
            _, st = eng.linear_search(m0s, gran or w.granularity, kernel)
    return st


def _case_oct_pipeline(stage):
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("oct-de")
    mid = len(line.cdp_midpoints) // 2
    m0s = line.cdp_midpoints[mid:mid + 1]
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          storage="fp16")
        eng.set_traveltime("oct", lower, upper, w.apm, 0.0)
        eng.set_window(tau)
        eng.set_oct_half_offsets([0.0, 500.0, 1000.0])
        gens = 20 if stage == "de" else 2
        for _ in range(2):
            de, st = eng.differential_evolution(m0s, w.population, gens, w.de_f, w.de_cr, seed=7)
        if stage == "sf":
            for _ in range(2):
                _, st = eng.stretch_free(m0s, np.ascontiguousarray(de[:, 2:]), 10)
    return st


def _case_cmp_sf():
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("cmp-production", 300)
    m0s = line.cdp_midpoints
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("cmp", lower, upper)
        eng.set_window(tau)
        ls, _ = eng.linear_search(m0s, w.granularity, "tuned")
        prior = np.ascontiguousarray(ls[:, 2:3])
        for _ in range(2):
            _, st = eng.stretch_free(m0s, prior, 10)
    return st


def _case_zocrs_de():
    from highperformanceseismicstacking_gb300 import capi
    w, line, lower, upper, tau = make_workload("zocrs-de")
    mid = len(line.cdp_midpoints) // 2
    m0s = line.cdp_midpoints[mid:mid + 16]
    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime("zocrs", lower, upper, w.apm)
        eng.set_window(tau)
        for _ in range(2):
            _, st = eng.differential_evolution(m0s, w.population, w.generations, w.de_f,
                                               w.de_cr, seed=7)
    return st


# Small cases for ncu captures (the profiles' commands): each runs its kernel
# once as a warm-up and once more; the tuned linear search with a fixed shape
# (HPSS_LS_VARIANT) has one launch of its kernel per call.
PROFILE_CASES = {
    # ls_tuned2_kernel: 300 CMPs of the CMP production line (1.44e10 evals)
    "cmp": lambda: _case_ls("cmp-production", 300, 0),
    # ls_tuned2_kernel (16-bit rows): the same with BF16 amplitude storage
    "cmpbf16": lambda: _case_ls("cmp-production", 300, 0, storage="bf16"),
    # ls_plain_kernel: the plain baseline on the same 300 CMPs
    "cmpplain": lambda: _case_ls("cmp-production", 300, 0, kernel="plain"),
    # ls_f64_kernel: every step in FP64, one ZO-CRS midpoint, 5 x 5 x 5 candidates
    "zocrsf64": lambda: _case_ls("zocrs-ls", None, 1, gran=[5, 5, 5], kernel="plain",
                                 fp64=True),
    # ls_tuned2_kernel: 4 midpoints of the ZO-CRS line, 21 x 21 x 41 candidates
    "zocrs": lambda: _case_ls("zocrs-ls", None, 4),
    # ls_tuned2_kernel (16-bit rows): the same with BF16 amplitude storage
    "zocrsbf16": lambda: _case_ls("zocrs-ls", None, 4, storage="bf16"),
    # ls_oct_kernel: 4 midpoints of the OCT DE line, 11 x 5 candidates
    "octls": lambda: _case_ls("oct-de", None, 4, gran=[11, 5]),
    # de_kernel: OCT DE over h0 0 / 500 / 1000 m, FP16 storage, 1 midpoint,
    # population 48, 20 generations
    "octde": lambda: _case_oct_pipeline("de"),
    # sf_block_kernel: the OCT stretch-free stack after a 2-generation DE, 3 h0, FP16
    "octsf": lambda: _case_oct_pipeline("sf"),
    # sf_block_kernel: CMP stretch-free (21 n, window 7) on 300 CMPs of the
    # production line over the tuned search's velocities
    "cmpsf": _case_cmp_sf,
    # de_kernel: ZO-CRS DE, 16 midpoints, population 32, 60 generations
    "zocrsde": _case_zocrs_de,
}


def time_call(eng, stream, d_m0, n_m0, gran, d_out, kernel, reps=1):
    """One untimed call (autotuning, first-launch costs), then `reps` calls
    timed with CUDA events on the engine's stream; ms per call."""
    import torch
    eng.linear_search_device(d_m0.data_ptr(), n_m0, gran, d_out.data_ptr(), kernel)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        eng.linear_search_device(d_m0.data_ptr(), n_m0, gran, d_out.data_ptr(), kernel)
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def storage_side(eng, line, stream, d_m0, n_m0, gran, evals, fp32_out, reps=1):
    """Tuned kernel with the amplitudes stored as BF16 / FP16 (re-uploaded on
    the same engine): throughput and the fraction of samples whose chosen
    parameters differ from the FP32-storage run.  Leaves the engine with FP32
    storage."""
    import torch
    out = {}
    d_out = torch.empty(fp32_out.shape, dtype=torch.float32, device=d_m0.device)
    for st in ("bf16", "fp16"):
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          storage=st)
        ms = time_call(eng, stream, d_m0, n_m0, gran, d_out, "tuned", reps)
        got = d_out.cpu().numpy()
        changed = float(np.mean(np.any(got[:, 2:] != fp32_out[:, 2:], axis=1)))
        out[st] = {"value": evals / (ms / 1e3), "ms": ms,
                   "chosen_parameters_changed_vs_fp32": changed}
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    return out


def per_midpoint_side(eng, stream, d_m0, gran, S, counts, P, batched_out, n_calls):
    """One midpoint per call, as the reference's ComputeAlgorithm interface
    computes them (computeSemblanceAndParametersForMidpoint,
    common/include/semblance/algorithm/ComputeAlgorithm.hpp:29-100): n_calls
    consecutive device calls of one midpoint each, tuned (its candidates split
    into ranges so that one midpoint fills the GPU) and plain; evals/s over
    the calls and whether the tuned blocks equal the batched call's."""
    import torch
    n = min(n_calls, d_m0.numel())
    d_out = torch.empty((n, 2 + eng.np, S), dtype=torch.float32, device=d_m0.device)
    evals = float(np.sum(np.asarray(counts[:n], np.float64))) * S * P
    res = {"calls": n}
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    for kernel in ("tuned", "plain"):
        st = eng.linear_search_device(d_m0.data_ptr(), 1, gran, d_out.data_ptr(), kernel,
                                      stats=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for i in range(n):
            eng.linear_search_device(d_m0.data_ptr() + 4 * i, 1, gran, d_out[i].data_ptr(),
                                     kernel)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        res[kernel] = {"value": evals / (ms / 1e3), "ms_per_call": ms / n}
        if kernel == "tuned":
            res[kernel]["candidate_parts"] = int(st["candidate_parts"])
            res[kernel]["identical_to_batched"] = bool(
                np.array_equal(d_out.cpu().numpy(), batched_out[:n]))
    res["speedup_tuned_vs_plain"] = res["tuned"]["value"] / res["plain"]["value"]
    return res


# ----------------------------------------------------------------- reference arm

def run_reference(args, world, rank):
    if rank != 0:
        return
    from oracle import oracle
    w, line, lower, upper, tau = make_workload(args.workload, args.n_cmp)
    params = oracle.build_grid(w.model, lower, upper, w.granularity)
    m0s = line.cdp_midpoints
    nthreads = oracle.max_threads()
    S = line.samples_per_trace
    rng = np.random.default_rng(0)

    def one_step(m0):
        sel = np.nonzero(oracle.select(w.model, line.midpoints, line.halfoffsets, m0, w.apm,
                                       w.h0, S, float(line.dt)))[0].astype(np.uint32)
        t = time.perf_counter()
        sem, stk, _ = oracle.ls_eval(w.model, line.samples, line.midpoints, line.halfoffsets,
                                     sel, m0, float(line.dt), tau, params, w.apm, w.h0,
                                     nthreads=nthreads)
        oracle.ls_result(w.model, sem, stk, params)
        return time.perf_counter() - t, float(sel.size) * S * params.shape[0]

    picks = rng.choice(len(m0s), size=args.warmup + args.steps, replace=True)
    for i in range(args.warmup):
        one_step(m0s[picks[i]])
    tot_t = tot_e = 0.0
    for i in range(args.steps):
        dt_, ev = one_step(m0s[picks[args.warmup + i]])
        tot_t += dt_
        tot_e += ev
    v = tot_e / tot_t
    sample = f"{args.steps} steps of one CMP gather each ({tot_e / args.steps:.3g} evals/step)"
    out = {"metric": METRIC, "value": v, "unit": UNIT, "impl": "reference",
           "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": 1e3 * tot_t / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": w.name, "cmps": int(len(m0s)), "fold": 60,
                      "samples": S, "candidates": int(params.shape[0]),
                      "window": 2 * tau + 1, "parallelism": "host threads"},
           "cpu_baseline": {"value": v, "unit": UNIT, "cores": nthreads, "kind": "port",
                            "sample": sample},
           "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
           "note": "reference CPU path is its OpenCL build on a host OpenCL device (absent); "
                   "timed here: the oracle's C restatement of the reference kernels"}
    # the reference's CUDA build on the same GPU, beside: its own kernels,
    # compiled from its sources (oracle/_ref), replayed per midpoint on the
    # midpoints of the engine's side measurements (no engine code runs here)
    if not args.no_reference_cuda:
        try:
            from oracle import ref_timing
            out["reference_cuda"] = ref_timing.reference_cuda()
        except Exception as e:  # no GPU, fatbins absent: reported, not fatal
            out["reference_cuda"] = {"unavailable": f"{type(e).__name__}: {e}"}
    print(json.dumps(out))


# ----------------------------------------------------------------- our arm

def cpu_baseline(w, line, lower, upper, tau, seconds):
    from oracle import oracle
    params = oracle.build_grid(w.model, lower, upper, w.granularity)
    nthreads = oracle.max_threads()
    S = line.samples_per_trace
    tot_t = tot_e = 0.0
    n = 0
    for m0 in line.cdp_midpoints[::37]:
        sel = np.nonzero(oracle.select(w.model, line.midpoints, line.halfoffsets, m0, w.apm,
                                       w.h0, S, float(line.dt)))[0].astype(np.uint32)
        t = time.perf_counter()
        oracle.ls_eval(w.model, line.samples, line.midpoints, line.halfoffsets, sel, m0,
                       float(line.dt), tau, params, w.apm, w.h0, nthreads=nthreads)
        tot_t += time.perf_counter() - t
        tot_e += float(sel.size) * S * params.shape[0]
        n += 1
        if tot_t >= seconds:
            break
    return {"value": tot_e / tot_t, "unit": UNIT, "cores": nthreads, "kind": "port",
            "sample": f"{n} CMP gathers of the same line ({tot_e:.3g} evals, {tot_t:.1f} s)"}


def main():
    args = parse()
    world, rank, local = dist_env()
    if args.profile_case:
        st = PROFILE_CASES[args.profile_case]()
        print(json.dumps({"profile_case": args.profile_case, "kernel_ms": st["kernel_ms"],
                          "evals": st["evals"], "not_used": st["not_used"],
                          "kernel_variant": st["kernel_variant"]}))
        return
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    import torch
    from highperformanceseismicstacking_gb300 import capi

    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    w, line, lower, upper, tau = make_workload(args.workload, args.n_cmp)
    S = line.samples_per_trace
    # Weak scaling: the job is a line of `world` segments of the workload's
    # size; rank r owns segment r (its CMPs shifted past the previous
    # segments), so the work per GPU stays fixed as ranks are added and no
    # data crosses ranks (midpoints are independent units).  This is the
    # shard plan of that line (sharding.shard_plan): a CMP gather selects
    # only its own traces (selection radius 0), so rank r's shard is exactly
    # segment r, with no halo traces.
    if world > 1 and rank > 0:
        shift = np.float32(rank * (float(line.cdp_midpoints[-1] - line.cdp_midpoints[0]) + 1000.0))
        line.midpoints = (line.midpoints + shift).astype(np.float32)
        line.cdp_midpoints = (line.cdp_midpoints + shift).astype(np.float32)
    all_m0 = line.cdp_midpoints
    m0s = all_m0
    P = int(np.prod(w.granularity))

    eng = capi.Engine(local)
    eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
    eng.set_traveltime(w.model, lower, upper, w.apm, w.h0)
    eng.set_window(tau)
    counts = eng.select_traces(m0s)
    evals = evals_per_step(counts, S, P)

    dev = torch.device("cuda", local)
    d_m0 = torch.from_numpy(np.ascontiguousarray(m0s)).to(dev)
    d_out = torch.empty((len(m0s), 2 + eng.np, S), dtype=torch.float32, device=dev)
    stream = torch.cuda.ExternalStream(eng.stream, device=dev)

    def barrier():
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()

    def run(kernel):
        eng.linear_search_device(d_m0.data_ptr(), len(m0s), w.granularity, d_out.data_ptr(),
                                 kernel)

    # per timed step: trace selection, the work-queue order of the midpoints
    # and the semblance kernel (the candidate grid and chunk bounds were built
    # by the warm-up calls and are reused; the batched call is not split into
    # candidate ranges, so no merge)
    launches_per_step = 3
    # ---- tuned, device resident
    for _ in range(args.warmup):
        run("tuned")
    barrier()
    clocks = ClockSampler(local)
    clocks.start()
    time.sleep(0.3)
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps + 1)]
    barrier()
    ev[0].record(stream)
    for i in range(args.steps):
        run("tuned")
        ev[i + 1].record(stream)
    barrier()
    clk = clocks.stop()
    step_ms = [ev[i].elapsed_time(ev[i + 1]) for i in range(args.steps)]
    total_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([total_ms], device=dev)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        total_ms = float(t.item())
        e = torch.tensor([evals], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(e)
        evals_all = float(e.item())
    else:
        evals_all = evals
    value = evals_all * args.steps / (total_ms / 1e3)
    # kernel-only duration of the semblance launch (stats path, one extra call)
    st = eng.linear_search_device(d_m0.data_ptr(), len(m0s), w.granularity, d_out.data_ptr(),
                                  "tuned", stats=True)
    kernel_ms = st["kernel_ms"]
    variant = st.get("kernel_variant")
    near_ties = st.get("near_ties", 0.0)
    tuned_out = d_out.cpu().numpy()

    # ---- plain kernel, same line
    run("plain")
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.plain_steps):
        run("plain")
    e1.record(stream)
    torch.cuda.synchronize()
    plain_ms = e0.elapsed_time(e1) / args.plain_steps
    plain_value = evals / (plain_ms / 1e3)
    plain_out = d_out.cpu().numpy()
    agreement = compare_outputs(tuned_out, plain_out)

    # ---- tuned kernel with the stack summed in the reference's order
    run("tuned_exact")
    torch.cuda.synchronize()
    e0.record(stream)
    for _ in range(args.plain_steps):
        run("tuned_exact")
    e1.record(stream)
    torch.cuda.synchronize()
    exact_ms = e0.elapsed_time(e1) / args.plain_steps
    exact_same = bool(np.array_equal(d_out.cpu().numpy(), plain_out))

    # ---- one midpoint per call (the reference's per-midpoint interface)
    per_mid = None
    if args.per_midpoint_calls > 0:
        per_mid = per_midpoint_side(eng, stream, d_m0, w.granularity, S, counts, P, tuned_out,
                                    args.per_midpoint_calls)

    # ---- 16-bit amplitude storage (tuned kernel), same line
    storage = None
    if not args.no_storage_side:
        storage = storage_side(eng, line, stream, d_m0, len(m0s), w.granularity, evals,
                               tuned_out, reps=args.plain_steps)

    # ---- end to end through the C ABI with host buffers
    pinned = torch.empty(line.samples.shape, dtype=torch.float32, pin_memory=True)
    pinned.numpy()[:] = line.samples
    host_samples = pinned.numpy()
    h2d = host_samples.nbytes + 2 * line.midpoints.nbytes + m0s.nbytes
    d2h = len(m0s) * (2 + eng.np) * S * 4
    eng2 = capi.Engine(local)
    # results land in a page-locked host block, as a caller streaming lines would hold
    res = torch.empty((len(m0s), 2 + eng.np, S), dtype=torch.float32, pin_memory=True).numpy()
    e2e_t, e2e_dev = [], []
    for i in range(args.e2e_steps + 1):
        barrier()
        t0 = time.perf_counter()
        # one call: the line is uploaded in trace ranges while the midpoints
        # whose traces have arrived are searched (hpss_linear_search_line)
        eng2.set_traveltime(w.model, lower, upper, w.apm, w.h0)
        eng2.set_window(tau)
        _, st_line = eng2.linear_search_line(host_samples, line.midpoints, line.halfoffsets,
                                             float(line.dt), m0s, w.granularity, "tuned",
                                             out=res)
        t1 = time.perf_counter()
        if i > 0:
            e2e_t.append(t1 - t0)
            # device span of the call: from its first group's launch sequence
            # (after the midpoints' copy) to its last group's end
            e2e_dev.append(st_line["kernel_ms"])
    e2e_max = max(e2e_t)
    if world > 1:
        t = torch.tensor([e2e_max], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        e2e_max = float(t.item())
    e2e_value = evals_all / (sum(e2e_t) / len(e2e_t)) if world == 1 else evals_all / e2e_max
    e2e_same = bool(np.array_equal(res, tuned_out))
    eng2.close()

    if rank != 0:
        eng.close()
        if world > 1:
            torch.distributed.barrier()
            torch.distributed.destroy_process_group()
        return

    # ---- roofline of the dominant kernel (tuned semblance kernel)
    peaks = measured_peaks()
    props = torch.cuda.get_device_properties(dev)
    sms = props.multi_processor_count
    fmax = float(peaks.get("sm_max_mhz", 2070.0)) * 1e6
    wsz = 2 * tau + 1
    t_model = {"cmp": 2, "zocrs": 5, "oct": 40}[w.model]
    instr_per_eval = 3 * wsz + t_model
    instr_per_launch = instr_per_eval * evals
    peak_instr = sms * 128 * fmax
    achieved = instr_per_launch / (kernel_ms / 1e3)
    n_sel = float(np.sum(counts))
    alg_bytes = n_sel * S * 4 + n_sel * 8 + len(m0s) * (2 + eng.np) * S * 4
    traffic, traffic_note = profile_traffic(f"ls_tuned_{w.name}")
    roof = {"bound": "fp32", "achieved": achieved / 1e12, "peak": peak_instr / 1e12,
            "unit": "Tinstr/s", "frac": achieved / peak_instr,
            "traffic": traffic,
            "instr_per_eval": instr_per_eval,
            "peak_source": "SMs x 128 FP32 lanes x measured max SM clock (MEASURED_PEAKS.json)",
            "kernel_ms": kernel_ms,
            "hbm": {"achieved": alg_bytes / (kernel_ms / 1e3) / 1e9,
                    "peak": float(peaks.get("hbm_gbs", 6800.0)), "unit": "GB/s",
                    "frac": alg_bytes / (kernel_ms / 1e3) / 1e9 / float(peaks.get("hbm_gbs", 6800.0)),
                    "bytes_per_launch": alg_bytes}}
    if traffic_note:
        roof["traffic_note"] = traffic_note

    # the CPU baseline and the single-GPU side measurements run with one GPU
    # only: with N ranks the other GPUs would wait for rank 0 meanwhile
    one = world == 1
    cpu = None
    if not args.no_cpu_baseline and one:
        cpu = cpu_baseline(w, line, lower, upper, tau, args.cpu_seconds)
    su_io = None
    if not args.no_io_side and one:
        su_io = su_io_side(line, d_out, len(m0s), 2 + eng.np, S)
    del pinned, host_samples
    zocrs = None
    if args.zocrs_cmps > 0 and args.workload != "zocrs-ls" and one:
        zocrs = zocrs_side_measure(args.zocrs_cmps, local)
    de = (de_side_measure(args.de_cmps, local, args.zocrs_de_cmps)
          if args.de_cmps > 0 and one else None)
    oct_ls = oct_ls_side(args.oct_cmps, local) if args.oct_cmps > 0 and one else None
    sf = sf_side(args.sf_cmps, local) if args.sf_cmps > 0 and one else None
    c5 = c5_side_measure(args.c5_cmps, local) if args.c5_cmps > 0 and one else None
    fp64 = fp64_agreement_side(args.fp64_cmps, local) if args.fp64_cmps > 0 and one else None
    whole = None if (args.no_whole_lines or not one) else whole_workloads_side(local)
    # every kernel against its roofline (FP32-pipe instructions; HBM view of
    # the algorithmic bytes where the line is read)
    rooflines = {f"ls_tuned ({w.name})": roof}
    if zocrs:
        rooflines["ls_tuned (zocrs-ls)"] = zocrs["tuned"].get("roofline")
    if oct_ls:
        rooflines["ls_oct (oct-de line, 55 candidates)"] = oct_ls["tuned"]["roofline"]
    if de:
        for k, v in de.items():
            rooflines[f"de ({k})"] = v["roofline"]
    if sf:
        rooflines["sf (cmp-production)"] = sf["roofline"]
    if c5:
        for st_ in ("fp16", "fp32"):
            if st_ in c5:
                rooflines[f"de (oct-de, 3 h0, {st_})"] = c5[st_]["de"]["roofline"]
                rooflines[f"sf (oct-de, 3 h0, {st_})"] = c5[st_]["stretch_free"]["roofline"]
    if whole:
        rooflines["de (zocrs-de, whole line)"] = whole["zocrs_de_whole_line"]["roofline"]
        rooflines["ls_tuned (zocrs-ls, whole line)"] = whole["zocrs_ls_whole_line"]["roofline"]

    out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
           "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": total_ms / args.steps, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
           "config": {"workload": w.name, "model": w.model, "algorithm": w.algorithm,
                      "cmps": int(len(all_m0)) * world, "cmps_per_gpu": int(len(all_m0)),
                      "fold": int(np.max(counts)) if len(counts) else 0,
                      "samples": S, "candidates": P, "window": wsz,
                      "evals_per_step": evals_all, "storage": "fp32", "kernel": "tuned",
                      "kernel_variant": variant,
                      "l2": "inputs exceed L2 (line %.0f MB > 129 MB); no flush" %
                            (line.samples.nbytes / 1e6),
                      "parallelism": f"line segments x{world} (one per GPU, {len(all_m0)} CMPs each)"},
           "plain": {"value": plain_value, "ms_per_step": plain_ms,
                     "speedup_tuned_vs_plain": value / plain_value,
                     "tuned_vs_plain": agreement},
           "storage_modes": storage,
           "per_midpoint_calls": per_mid,
           "near_ties": {"samples": near_ties, "of": int(len(m0s)) * S,
                         "rel_tolerance": 1e-4},
           "tuned_exact": {"value": evals / (exact_ms / 1e3), "ms_per_step": exact_ms,
                           "identical_to_plain": exact_same},
           "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(h2d),
                   "d2h_bytes_per_step": int(d2h), "s_per_step": sum(e2e_t) / len(e2e_t),
                   "device_span_ms": sum(e2e_dev) / len(e2e_dev),
                   "matches_device_result": e2e_same},
           "gpu_launches": launches_per_step * args.steps,
           "roofline": roof,
           "cpu_baseline": cpu,
           "zocrs_linear_search": zocrs,
           "oct_linear_search": oct_ls,
           "differential_evolution": de,
           "stretch_free": sf,
           "oct_de_stretch_free_pipeline": c5,
           "fp64_agreement": fp64,
           "whole_workloads": whole,
           "su_io": su_io,
           "rooflines": rooflines,
           "clocks": clk,
           "step_ms": step_ms}
    print(json.dumps(out))
    eng.close()
    if world > 1:
        torch.distributed.barrier()
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
