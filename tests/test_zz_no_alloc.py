"""The allocation-free linear search (hpss_linear_search_noalloc).

Callers that may not allocate device memory -- a plug-in living inside another
framework's memory pool, or a service with a fixed device-memory budget --
pass their own device buffers; the library's scratch is a fixed __device__
array.  This test (collected last on purpose) calls the entry point through
the C ABI twice in a row and checks both results against the allocating entry
point's (hpss_linear_search) -- same kernels, so the tolerance is equality,
stricter than the parity tolerances of tests/parity.py -- and reads the
kernels' device error word back with hpss_noalloc_device_error after each.
It allocates its own buffers with torch; the entry point allocates nothing.
It passes alone in a fresh process and after the other tests.
"""
import ctypes as C

import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import capi, synthetic

pytestmark = pytest.mark.gpu


def _device_line(torch, line, stride):
    n, S = line.samples.shape
    padded = np.zeros((n, stride), np.float32)
    padded[:, :S] = line.samples
    dev = torch.device("cuda", 0)
    return (torch.from_numpy(padded).to(dev), torch.from_numpy(line.midpoints).to(dev),
            torch.from_numpy(line.halfoffsets).to(dev))


@pytest.mark.parametrize("model", ["cmp", "zocrs"])
def test_noalloc_matches_allocating_entry_point_twice(model):
    torch = pytest.importorskip("torch")
    lib = capi.lib()
    if model == "cmp":
        w = synthetic.WORKLOADS["cmp-small"]
        line = synthetic.cmp_line(n_cmp=6, halfoffsets=list(range(25, 1176, 50)), ns=500,
                                  dt_us=4000, n_reflectors=4, n_multiples=0, f=25.0, snr=10.0,
                                  seed=71)
        lower, upper, gran, apm = w.lower, w.upper, w.granularity, 0.0
    else:
        line = synthetic.structured_line(n_cmp=16, fold_range=(6, 10), h_max=1000, ns=300,
                                         dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=72)
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, gran, apm = [1414.2136, -a, -b], [6324.5553, a, b], [7, 5, 5], 125.0
    tau = 2
    dt = float(line.dt)
    m0s = np.ascontiguousarray(line.cdp_midpoints[::2])
    np_ = capi.N_PARAMS[model]
    S = line.samples_per_trace

    with capi.Engine(0) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, dt)
        eng.set_traveltime(model, lower, upper, apm)
        eng.set_window(tau)
        want, st = eng.linear_search(m0s, gran, "tuned")
    assert st["device_error"] == 0

    stride = (S + 7) // 8 * 8
    d_smp, d_mid, d_h = _device_line(torch, line, stride)
    d_m0 = torch.from_numpy(m0s).cuda()
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    g = np.asarray(gran, np.uint32)
    for call in range(2):
        d_out = torch.full((m0s.size, 2 + np_, S), -7.0, dtype=torch.float32, device="cuda")
        rc = lib.hpss_linear_search_noalloc(
            capi.MODELS[model], C.c_void_p(d_smp.data_ptr()), stride,
            C.c_void_p(d_mid.data_ptr()), C.c_void_p(d_h.data_ptr()), line.samples.shape[0], S,
            C.c_float(dt), tau, lo.ctypes.data_as(C.POINTER(C.c_float)),
            hi.ctypes.data_as(C.POINTER(C.c_float)), g.ctypes.data_as(C.POINTER(C.c_uint32)),
            C.c_float(apm), C.c_void_p(d_m0.data_ptr()), m0s.size, C.c_void_p(d_out.data_ptr()),
            None)
        assert rc == 0, lib.hpss_last_error(None)
        # the kernels' error word (cleared by every call) reads back as 0
        word = C.c_uint32(0xffffffff)
        assert lib.hpss_noalloc_device_error(None, C.byref(word)) == 0
        assert word.value == 0, f"call {call}: device error word {word.value}"
        torch.cuda.synchronize()
        got = d_out.cpu().numpy()
        assert np.array_equal(got, want), f"call {call}"


def test_noalloc_rejects_sizes_beyond_its_scratch():
    lib = capi.lib()
    lo = np.asarray([1000.0], np.float32)
    hi = np.asarray([5000.0], np.float32)
    g = np.asarray([70000], np.uint32)       # > 65536 candidates
    dummy = C.c_void_p(256)
    rc = lib.hpss_linear_search_noalloc(0, dummy, 8, dummy, dummy, 1, 8, C.c_float(0.004), 1,
                                        lo.ctypes.data_as(C.POINTER(C.c_float)),
                                        hi.ctypes.data_as(C.POINTER(C.c_float)),
                                        g.ctypes.data_as(C.POINTER(C.c_uint32)), C.c_float(0.0),
                                        dummy, 1, dummy, None)
    assert rc == -1
    assert b"limits" in lib.hpss_last_error(None)
