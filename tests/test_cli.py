"""The C++ CLI programs (reference flags, SU input/output, exit codes).

CPU: flag parsing and error exits (no device needed).
GPU: a full single_host_linear_search run on an SU file, result files checked
against the engine's own results, then single_host_stretch_free on the
velocity file it wrote, and single_host_de.
"""
import glob
import os
import subprocess
from pathlib import Path

import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import build, capi, su, synthetic

BIN = Path(build.PKG) / "bin"


def _run(exe, *args, timeout=300):
    r = subprocess.run([str(BIN / exe), *map(str, args)], capture_output=True, text=True,
                       timeout=timeout)
    return r.returncode, r.stdout + r.stderr


@pytest.fixture(scope="module", autouse=True)
def _host_built():
    from highperformanceseismicstacking_gb300 import host_build
    host_build.build_host()


def test_missing_required_flags_print_help_and_exit_0():
    rc, out = _run("single_host_linear_search", "--aph", "1000")
    assert rc == 0
    assert "is required but missing" in out
    assert "--granularity" in out and "--lower-bounds" in out


def test_unknown_flag_is_invalid_argument():
    rc, out = _run("single_host_de", "--bogus", "1")
    assert rc == 0 and "unrecognised option" in out


def _has_gpu():
    import ctypes
    n = ctypes.c_int(0)
    return capi.lib().hpss_device_count(ctypes.byref(n)) == 0 and n.value > 0


@pytest.mark.skipif(_has_gpu(), reason="checks the no-device exit code")
def test_no_device_exits_enodev(tmp_path):
    line = synthetic.cmp_line(n_cmp=1, halfoffsets=[25], ns=16, dt_us=4000, n_reflectors=1,
                              n_multiples=0, f=25.0, snr=10.0, seed=1)
    p = tmp_path / "x.su"
    su.write_su(str(p), line.headers, line.samples)
    rc, out = _run("single_host_linear_search", "--aph", 1000, "--apm", 0, "--azimuth", 0,
                   "--tau", 0.01, "--input", p, "--output", tmp_path, "--lower-bounds", 1000,
                   "--upper-bounds", 5000, "--granularity", 10, "--traveltime", "cmp")
    assert rc == (256 - 19) % 256  # -ENODEV as an exit status
    assert "No CUDA devices" in out


def _results(outdir):
    d = glob.glob(str(outdir / "*/"))
    assert len(d) == 1, d
    return Path(d[0])


@pytest.mark.gpu
def test_linear_search_cli_matches_engine_and_feeds_stretch_free(tmp_path):
    line = synthetic.cmp_line(n_cmp=4, halfoffsets=list(range(25, 1176, 50)), ns=400,
                              dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0,
                              seed=81)
    inp = tmp_path / "line.su"
    su.write_su(str(inp), line.headers, line.samples)
    out1 = tmp_path / "ls"
    out1.mkdir()
    rc, log = _run("single_host_linear_search", "--aph", 2000, "--apm", 0, "--azimuth", 0,
                   "--tau", 0.010, "--input", inp, "--output", out1, "--lower-bounds", 1000,
                   "--upper-bounds", 5040, "--granularity", 101, "--traveltime", "cmp",
                   "--verbose", 1)
    assert rc == 0, log
    res = _results(out1)
    names = sorted(os.path.basename(p) for p in glob.glob(str(res / "*")))
    for f in ["coherence.su", "stack.su", "velocity.su", "gather.txt", "traveltime.txt",
              "efficiency.csv", "interpolations_per_sec.csv", "selected_traces.csv",
              "total_kernel_exec_time.csv", "total_selection_kernel_exec_time.csv"]:
        assert f in names, names
    hdr, coh = su.read_su(str(res / "coherence.su"))
    _, vel = su.read_su(str(res / "velocity.su"))
    # one trace per CDP in map order, including the reference's midpoint-0 CDP
    assert coh.shape == (5, 400)
    assert np.all(coh[0] == 0)
    g = su.read_gather(str(inp), aph=2000, apm=0, tau=0.010)
    with capi.Engine(0) as eng:
        eng.upload_gather(g.samples, g.midpoints, g.halfoffsets, float(g.dt))
        eng.set_traveltime("cmp", [1000.0], [5040.0])
        eng.set_window(g.tau_index)
        want, _ = eng.linear_search(line.cdp_midpoints, [101], "tuned")
    assert np.array_equal(coh[1:], want[:, 0])
    assert np.array_equal(vel[1:], want[:, 2])
    # stretch-free on the velocity file the CLI wrote
    out2 = tmp_path / "sf"
    out2.mkdir()
    rc, log = _run("single_host_stretch_free", "--aph", 2000, "--apm", 0, "--azimuth", 0,
                   "--tau", 0.010, "--input", inp, "--output", out2, "--lower-bounds", 1000,
                   "--upper-bounds", 5040, "--traveltime", "cmp", "--stack-datafiles",
                   res / "velocity.su")
    assert rc == 0, log
    res2 = _results(out2)
    _, n = su.read_su(str(res2 / "n.su"))
    assert n.shape == (5, 400)
    assert np.all(np.abs(n[1:]) <= 10)


@pytest.mark.gpu
def test_de_cli_runs_with_seed(tmp_path):
    line = synthetic.cmp_line(n_cmp=2, halfoffsets=list(range(25, 1176, 50)), ns=200,
                              dt_us=4000, n_reflectors=2, n_multiples=0, f=25.0, snr=10.0,
                              seed=82)
    inp = tmp_path / "line.su"
    su.write_su(str(inp), line.headers, line.samples)
    outs = []
    for k in range(2):
        o = tmp_path / f"de{k}"
        o.mkdir()
        rc, log = _run("single_host_de", "--aph", 2000, "--apm", 0, "--azimuth", 0, "--tau",
                       0.010, "--input", inp, "--output", o, "--lower-bounds", 1000,
                       "--upper-bounds", 5000, "--traveltime", "cmp", "--generations", 8,
                       "--population-size", 16, "--seed", 5, "--de-f", 0.5, "--de-cr", 0.9)
        assert rc == 0, log
        _, v = su.read_su(str(_results(o) / "velocity.su"))
        outs.append(v)
    assert np.array_equal(outs[0], outs[1])
    assert np.all((outs[0][1:] >= 1000) & (outs[0][1:] <= 5000))


@pytest.mark.gpu
def test_linear_search_cli_engine_options(tmp_path):
    """--grid-mode inclusive, --precision fp16 and --kernel tuned-exact reach
    the engine: results equal an engine configured the same way."""
    line = synthetic.cmp_line(n_cmp=3, halfoffsets=list(range(25, 1176, 50)), ns=300,
                              dt_us=4000, n_reflectors=3, n_multiples=0, f=25.0, snr=10.0,
                              seed=83)
    inp = tmp_path / "line.su"
    su.write_su(str(inp), line.headers, line.samples)
    out = tmp_path / "ls"
    out.mkdir()
    rc, log = _run("single_host_linear_search", "--aph", 2000, "--apm", 0, "--azimuth", 0,
                   "--tau", 0.010, "--input", inp, "--output", out, "--lower-bounds", 1000,
                   "--upper-bounds", 5000, "--granularity", 41, "--traveltime", "cmp",
                   "--grid-mode", "inclusive", "--precision", "fp16", "--kernel", "tuned-exact")
    assert rc == 0, log
    res = _results(out)
    _, coh = su.read_su(str(res / "coherence.su"))
    _, stk = su.read_su(str(res / "stack.su"))
    _, vel = su.read_su(str(res / "velocity.su"))
    g = su.read_gather(str(inp), aph=2000, apm=0, tau=0.010)
    with capi.Engine(0) as eng:
        eng.upload_gather(g.samples, g.midpoints, g.halfoffsets, float(g.dt), storage="fp16")
        eng.set_traveltime("cmp", [1000.0], [5000.0])
        eng.set_window(g.tau_index)
        eng.set_grid_mode("inclusive")
        want, _ = eng.linear_search(line.cdp_midpoints, [41], "tuned_exact")
    assert np.array_equal(coh[1:], want[:, 0])
    assert np.array_equal(stk[1:], want[:, 1])
    assert np.array_equal(vel[1:], want[:, 2])
    rc, log = _run("single_host_linear_search", "--aph", 2000, "--apm", 0, "--azimuth", 0,
                   "--tau", 0.010, "--input", inp, "--output", out, "--lower-bounds", 1000,
                   "--upper-bounds", 5000, "--granularity", 41, "--traveltime", "cmp",
                   "--grid-mode", "sideways")
    assert "--grid-mode must be reference or inclusive" in log
