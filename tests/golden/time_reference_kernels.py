#!/usr/bin/env python3
"""Time the reference's own CUDA kernels (fatbins built from the reference
sources by oracle/build_ref.py) on the bench line: CMP production line, 401
velocities, window 7.  Per midpoint the reference's launch sequence
(computeSemblancesForCommonMidPoint + selectBestSemblancesForCommonMidPoint,
CudaLinearSearchAlgorithm.cu:35-163) is timed with CUDA events; trace
selection and packing are excluded, as in the reference's own
total_kernel_exec_time.  Prints one JSON line.

    python tests/golden/time_reference_kernels.py [n_midpoints]
"""
from __future__ import annotations

import ctypes as C
import json
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from highperformanceseismicstacking_gb300 import synthetic  # noqa: E402
from highperformanceseismicstacking_gb300.su import tau_index  # noqa: E402
from oracle import ref_runner  # noqa: E402


def main(n_mid: int = 20):
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
                      "workload": "cmp-production", "midpoints": n_mid, "evals": evals,
                      "kernel_ms": total_ms, "value": evals / (total_ms / 1e3),
                      "unit": "evals/s"}))


if __name__ == "__main__":
    main(int(sys.argv[1]) if len(sys.argv) > 1 else 20)
