"""The bounds-checked build (-DHPSS_CHECKED) and the staging-timeout path.

The checked build recomputes, inside the tuned kernel, every window position
of a trace taken on the branch without range tests and checks it against the
staged span, and checks every shared-memory window index of the other traces
(device error word bit HPSS_DEVERR_SMEM_BOUNDS).  It runs the CMP, ZO-CRS and
window-at-the-trace-edge cases here and must report no error and produce the
default build's results bit for bit.

The timeout drill (checked builds only, HPSS_STAGE_DRILL=<bytes>) arms the
staging barrier with bytes no copy delivers, so every bounded wait runs out:
the kernel must return with HPSS_DEVERR_TIMEOUT set (HPSS_ERR_TIMEOUT from
the synchronous call, the word from hpss_noalloc_device_error for the
allocation-free search), and the context must stay usable (the next call
without the drill gives the right results).
"""
import ctypes as C
import os

import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import build, capi, synthetic

pytestmark = pytest.mark.gpu

TIMEOUT = 4  # HPSS_DEVERR_TIMEOUT


@pytest.fixture(scope="module")
def checked_lib():
    path = build.build_engine(extra_flags=["-DHPSS_CHECKED"], flavour="checked")
    return capi.load_library(path)


def _cases():
    a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
    cmp_line = synthetic.cmp_line(n_cmp=6, halfoffsets=list(range(25, 1176, 50)), ns=500,
                                  dt_us=4000, n_reflectors=4, n_multiples=0, f=25.0, snr=10.0,
                                  seed=301)
    prod_slice = synthetic.cmp_line(n_cmp=3, halfoffsets=list(range(0, 2951, 50)), ns=2000,
                                    dt_us=2000, n_reflectors=12, n_multiples=3, f=25.0,
                                    snr=10.0, seed=302)
    zl = synthetic.structured_line(n_cmp=16, fold_range=(6, 12), h_max=1000, ns=300,
                                   dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=303)
    # short traces, long offsets, wide window: most windows touch a trace end
    edge = synthetic.cmp_line(n_cmp=4, halfoffsets=list(range(0, 3001, 100)), ns=64,
                              dt_us=4000, n_reflectors=2, n_multiples=0, f=25.0, snr=4.0,
                              seed=304)
    return {
        "cmp-small": (cmp_line, "cmp", [1000.0], [5040.0], [101], 2, 0.0),
        "cmp-production-slice-w7": (prod_slice, "cmp", [1000.0], [6012.5], [401], 3, 0.0),
        "zocrs": (zl, "zocrs", [1414.2136, -a, -b], [6324.5553, a, b], [9, 7, 7], 2, 125.0),
        "window-edge-w15": (edge, "cmp", [1000.0], [5040.0], [64], 7, 0.0),
        "zocrs-window-edge-w11": (zl, "zocrs", [1414.2136, -a, -b], [6324.5553, a, b],
                                  [5, 5, 5], 5, 125.0),
    }


def _search(lib, line, model, lower, upper, gran, tau, apm, kernel):
    with capi.Engine(0, library=lib) as eng:
        eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt))
        eng.set_traveltime(model, lower, upper, apm)
        eng.set_window(tau)
        return eng.linear_search(line.cdp_midpoints, gran, kernel)


@pytest.mark.parametrize("case", list(_cases()))
@pytest.mark.parametrize("kernel", ["tuned", "tuned_exact"])
def test_checked_build_reports_no_error_and_same_results(checked_lib, case, kernel):
    line, model, lower, upper, gran, tau, apm = _cases()[case]
    got, st = _search(checked_lib, line, model, lower, upper, gran, tau, apm, kernel)
    assert st["device_error"] == 0
    assert st["kernel_variant"] >= 0  # the tuned pair kernel ran
    want, st2 = _search(capi.lib(), line, model, lower, upper, gran, tau, apm, kernel)
    assert st2["device_error"] == 0
    assert np.array_equal(got, want)


@pytest.mark.parametrize("storage", ["bf16", "fp16"])
@pytest.mark.parametrize("case", ["cmp-production-slice-w7", "zocrs", "window-edge-w15"])
def test_checked_build_16bit_bulk_staging(checked_lib, case, storage):
    """16-bit rows staged by bulk copies and widened in shared memory, in the
    checked build: every window inside its staged span, no error, and the
    default build's results bit for bit."""
    line, model, lower, upper, gran, tau, apm = _cases()[case]
    outs = []
    for lib in (checked_lib, capi.lib()):
        with capi.Engine(0, library=lib) as eng:
            eng.upload_gather(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                              storage=storage)
            eng.set_traveltime(model, lower, upper, apm)
            eng.set_window(tau)
            got, st = eng.linear_search(line.cdp_midpoints, gran, "tuned")
            assert st["device_error"] == 0
            assert st["kernel_variant"] >= 0
            outs.append(got)
    assert np.array_equal(outs[0], outs[1])


@pytest.mark.parametrize("storage", ["fp32", "fp16"])
@pytest.mark.parametrize("model", ["cmp", "zocrs"])
def test_checked_build_staged_de_windows_stay_in_their_spans(checked_lib, model, storage):
    """Differential evolution with staged spans in the checked build, FP32
    and 16-bit rows: every window read from shared memory lies inside its
    trace's staged span, and every pair of traces taken on the path without
    range tests has all its windows inside the trace (no
    HPSS_DEVERR_SMEM_BOUNDS); the results equal the default build's."""
    zl = synthetic.structured_line(n_cmp=16, fold_range=(6, 12), h_max=1000, ns=300,
                                   dt_us=4000, n_reflectors=4, f=20.0, snr=5.0, seed=305)
    if model == "cmp":
        lower, upper, apm = [1000.0], [5040.0], 0.0
    else:
        a, b = synthetic.zocrs_bounds(1414.2136, 2000.0, 90.0, 0.05)
        lower, upper, apm = [1414.2136, -a, -b], [6324.5553, a, b], 125.0
    outs = []
    for lib in (checked_lib, capi.lib()):
        with capi.Engine(0, library=lib) as eng:
            eng.upload_gather(zl.samples, zl.midpoints, zl.halfoffsets, float(zl.dt),
                              storage=storage)
            eng.set_traveltime(model, lower, upper, apm)
            eng.set_window(3)
            got, st = eng.differential_evolution(zl.cdp_midpoints[4:12], 32, 20, 0.5, 0.9,
                                                 seed=3)
            assert st["device_error"] == 0
            outs.append(got)
    assert np.array_equal(outs[0], outs[1])


def test_staging_timeout_is_reported_and_context_survives(checked_lib, monkeypatch):
    line, model, lower, upper, gran, tau, apm = _cases()["cmp-small"]
    want, _ = _search(checked_lib, line, model, lower, upper, gran, tau, apm, "tuned")
    monkeypatch.setenv("HPSS_STAGE_DRILL", "16")
    with pytest.raises(capi.HpssError) as ei:
        _search(checked_lib, line, model, lower, upper, gran, tau, apm, "tuned")
    assert ei.value.code == -7  # HPSS_ERR_TIMEOUT
    monkeypatch.delenv("HPSS_STAGE_DRILL")
    again, st = _search(checked_lib, line, model, lower, upper, gran, tau, apm, "tuned")
    assert st["device_error"] == 0
    assert np.array_equal(again, want)


def test_noalloc_device_error_word_reports_the_timeout(checked_lib, monkeypatch):
    torch = pytest.importorskip("torch")
    line, model, lower, upper, gran, tau, apm = _cases()["cmp-small"]
    want, _ = _search(checked_lib, line, model, lower, upper, gran, tau, apm, "tuned")
    n, S = line.samples.shape
    stride = (S + 7) // 8 * 8
    padded = np.zeros((n, stride), np.float32)
    padded[:, :S] = line.samples
    d_smp = torch.from_numpy(padded).cuda()
    d_mid = torch.from_numpy(line.midpoints).cuda()
    d_h = torch.from_numpy(line.halfoffsets).cuda()
    m0s = line.cdp_midpoints
    d_m0 = torch.from_numpy(m0s).cuda()
    lo = np.asarray(lower, np.float32)
    hi = np.asarray(upper, np.float32)
    g = np.asarray(gran, np.uint32)

    def call():
        d_out = torch.zeros((m0s.size, 3, S), dtype=torch.float32, device="cuda")
        rc = checked_lib.hpss_linear_search_noalloc(
            0, C.c_void_p(d_smp.data_ptr()), stride, C.c_void_p(d_mid.data_ptr()),
            C.c_void_p(d_h.data_ptr()), n, S, C.c_float(float(line.dt)), tau,
            lo.ctypes.data_as(C.POINTER(C.c_float)), hi.ctypes.data_as(C.POINTER(C.c_float)),
            g.ctypes.data_as(C.POINTER(C.c_uint32)), C.c_float(apm),
            C.c_void_p(d_m0.data_ptr()), m0s.size, C.c_void_p(d_out.data_ptr()), None)
        assert rc == 0, checked_lib.hpss_last_error(None)
        word = C.c_uint32(0xffffffff)
        assert checked_lib.hpss_noalloc_device_error(None, C.byref(word)) == 0
        return d_out.cpu().numpy(), word.value

    out, word = call()
    assert word == 0
    assert np.array_equal(out, want)
    monkeypatch.setenv("HPSS_STAGE_DRILL", "16")
    _, word = call()
    assert word & TIMEOUT
    monkeypatch.delenv("HPSS_STAGE_DRILL")
    out, word = call()
    assert word == 0          # the word is cleared by every call
    assert np.array_equal(out, want)
