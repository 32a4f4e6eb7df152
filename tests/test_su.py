"""SU files and the reference's gather semantics (CPU only)."""
import numpy as np

from highperformanceseismicstacking_gb300 import su, synthetic


def test_header_is_240_bytes_and_round_trips(tmp_path):
    line = synthetic.cmp_line(n_cmp=3, halfoffsets=[25, 75, 125], ns=64, dt_us=4000,
                              n_reflectors=2, n_multiples=0, f=25.0, snr=10.0, seed=1)
    p = tmp_path / "a.su"
    su.write_su(str(p), line.headers, line.samples)
    assert p.stat().st_size == line.samples.shape[0] * (240 + 4 * 64)
    hdr, smp = su.read_su(str(p))
    assert np.array_equal(smp, line.samples)
    assert np.array_equal(hdr["gy"], line.headers["gy"])


def test_geometry_is_exact_and_sorted(tmp_path):
    line = synthetic.cmp_line(n_cmp=4, halfoffsets=[25, 75, 125, 175], ns=32, dt_us=2000,
                              n_reflectors=1, n_multiples=0, f=25.0, snr=10.0, seed=2)
    order = np.random.default_rng(0).permutation(line.samples.shape[0])
    p = tmp_path / "b.su"
    su.write_su(str(p), line.headers[order], line.samples[order])
    g = su.read_gather(str(p), aph=1000.0, apm=0.0, tau=0.005)
    assert np.array_equal(g.midpoints, np.sort(line.midpoints))
    key = np.lexsort((line.halfoffsets, line.midpoints))
    assert np.array_equal(g.halfoffsets, line.halfoffsets[key])
    assert np.array_equal(g.samples, line.samples[key])
    assert g.dt == np.float32(np.float32(2000) * np.float32(1e-6))
    assert g.tau_index == int(np.float32(0.005) / g.dt) == 2
    assert g.window_size == 5


def test_reference_filters_and_eof_cdp(tmp_path):
    line = synthetic.cmp_line(n_cmp=2, halfoffsets=[25, 1500], ns=16, dt_us=4000,
                              n_reflectors=1, n_multiples=0, f=25.0, snr=10.0, seed=3)
    p = tmp_path / "c.su"
    su.write_su(str(p), line.headers, line.samples)
    g = su.read_gather(str(p), aph=1000.0, apm=0.0, tau=0.0)
    # |h| > aph dropped, but the CDP entries exist
    assert g.trace_count == 2
    # the reference's read loop adds a CDP at midpoint 0 after the last trace
    assert list(g.cdps.keys()) == [0.0, 1000.0, 1025.0]
    g2 = su.read_gather(str(p), aph=1000.0, apm=0.0, tau=0.0, emulate_eof_cdp=False)
    assert list(g2.cdps.keys()) == [1000.0, 1025.0]
    # CDP header: offset 0, sx = gx = (sx+gx)>>1, sy = gy = (sy+gy)>>1
    info = g.cdps[1000.0].info
    assert int(info["offset"]) == 0 and int(info["sy"]) == int(info["gy"]) == 1000


def test_nonpositive_midpoints_dropped(tmp_path):
    hdr = np.zeros(3, su.SU_HEADER_DTYPE)
    hdr["scalco"] = 1
    hdr["ns"] = 8
    hdr["dt"] = 4000
    hdr["sy"] = [-10, -50, 90]
    hdr["gy"] = [10, 40, 110]
    smp = np.ones((3, 8), np.float32)
    p = tmp_path / "d.su"
    su.write_su(str(p), hdr, smp)
    g = su.read_gather(str(p), aph=1000.0, apm=0.0, tau=0.0)
    # m = 0 and m = -5 are below FLT_MIN (Gather.cpp:32, Trace.cpp:41-43)
    assert g.midpoints.tolist() == [100.0]


def test_scalco_negative_divides():
    hdr = np.zeros(1, su.SU_HEADER_DTYPE)
    hdr["scalco"] = -10
    hdr["sy"] = 1000
    hdr["gy"] = 3000
    m, h = su.midpoint_halfoffset(hdr, np.float32(0))
    assert m[0] == np.float32(200.0) and h[0] == np.float32(100.0)


def _cdp_result_case(tmp_path):
    line = synthetic.cmp_line(n_cmp=7, halfoffsets=[25, 75, 125], ns=40, dt_us=4000,
                              n_reflectors=1, n_multiples=0, f=25.0, snr=10.0, seed=4)
    p = tmp_path / "line.su"
    su.write_su(str(p), line.headers, line.samples)
    g = su.read_gather(str(p), aph=1000.0, apm=0.0, tau=0.008, emulate_eof_cdp=False)
    cdps = list(g.cdps.values())
    headers = np.stack([c.info for c in cdps]).astype(su.SU_HEADER_DTYPE)
    slab = np.random.default_rng(0).standard_normal((len(cdps), 3, 40)).astype(np.float32)
    return headers, slab


def test_batched_result_writer_matches_per_cdp_writer(tmp_path):
    """hpss_write_result_files (one image per file, one write) produces the
    bytes of the reference's per-CDP Dumper::dumpResult loop: per CDP its
    header, then the row's samples."""
    from highperformanceseismicstacking_gb300 import capi
    headers, slab = _cdp_result_case(tmp_path)
    paths = [str(tmp_path / f"r{r}.su") for r in range(3)]
    capi.write_result_files(slab, headers, paths)
    for r in range(3):
        ref = tmp_path / f"ref{r}.su"
        su.write_su(str(ref), headers, slab[:, r, :])
        assert (tmp_path / f"r{r}.su").read_bytes() == ref.read_bytes()
    # a None path skips its row
    capi.write_result_files(slab, headers, [None, str(tmp_path / "only1.su"), None])
    assert (tmp_path / "only1.su").read_bytes() == (tmp_path / "ref1.su").read_bytes()
