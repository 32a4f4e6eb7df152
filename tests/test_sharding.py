"""Midpoint sharding across ranks (CPU, gloo, world size 2).

Each rank computes its contiguous midpoint shard with the oracle (standing in
for its GPU), reading only its own traces and the halo within the model's
selection radius (sharding.shard_plan); gathering the shards in rank order
must reproduce the single-process result exactly, every midpoint exactly
once, with no collective on the data path besides the final gather.  Covered:
CMP (no halo), ZO-CRS (halo = apm) and OCT (halo = apm + sqrt(hmax^2 + h0^2),
derived in sharding.py) lines split at interior CMPs.
"""
import os
import socket

import numpy as np
import pytest

from highperformanceseismicstacking_gb300 import sharding


def test_shards_cover_every_midpoint_once():
    for n in [0, 1, 7, 2000]:
        for world in [1, 2, 3, 8]:
            seen = []
            for r in range(world):
                a, b = sharding.shard_midpoints(np.arange(n), world, r)
                seen.extend(range(a, b))
                assert b - a in (n // world, n // world + 1)
            assert seen == list(range(n))


def test_halo_range_covers_aperture():
    mid = np.repeat(np.arange(1000.0, 2000.0, 25.0, dtype=np.float32), 3)
    a, b = sharding.halo_trace_range(mid, 1200.0, 1400.0, 100.0)
    sel = mid[a:b]
    assert sel.min() >= 1100.0 and sel.max() <= 1500.0
    assert np.sum((mid >= 1100.0) & (mid <= 1500.0)) == b - a


def test_selection_radius_bounds_the_oct_displacement():
    """|mh - m0| <= sqrt(h^2 + h0^2) for any slope, t0 and velocity (the
    bound behind the OCT halo), checked on the oracle's FP64 displaced
    midpoint through its selection: a trace farther than the radius from m0
    is never selected."""
    from oracle import oracle
    rng = np.random.default_rng(5)
    for h0 in (0.0, 500.0, 1000.0):
        n = 400
        mid = np.sort(rng.uniform(0, 20000, n)).astype(np.float32)
        hoff = rng.uniform(-3000, 3000, n).astype(np.float32)
        m0, apm = 10000.0, 200.0
        cands = oracle.oct_selection_candidates([1200.0, -3e-2], [5000.0, 3e-2])
        sel = oracle.select("oct", mid, hoff, m0, apm, h0, 200, 0.004, cands)
        r = sharding.selection_radius("oct", apm, float(np.max(np.abs(hoff))), [h0])
        assert np.all(np.abs(mid[sel] - m0) <= r)
        # per trace the tighter bound apm + sqrt(h^2 + h0^2) holds too
        assert np.all(np.abs(mid[sel] - m0) <= apm + np.sqrt(hoff[sel] ** 2 + h0 ** 2) * 1.001 + 1)


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _line(model):
    from highperformanceseismicstacking_gb300 import synthetic
    if model == "cmp":
        return synthetic.cmp_line(n_cmp=5, halfoffsets=[25, 75, 125, 175, 225], ns=120,
                                  dt_us=4000, n_reflectors=2, n_multiples=0, f=25.0, snr=10.0,
                                  seed=91)
    if model == "zocrs":
        return synthetic.structured_line(n_cmp=11, fold_range=(3, 6), h_max=500, ns=100,
                                         dt_us=4000, n_reflectors=2, f=20.0, snr=8.0, seed=92)
    # OCT: a line longer than its halo (40 + sqrt(250^2 + 200^2) ~ 360 m)
    return synthetic.structured_line(n_cmp=40, fold_range=(3, 5), h_max=250, ns=100,
                                     dt_us=4000, n_reflectors=2, f=20.0, snr=8.0, seed=93)


SPECS = {
    "cmp": dict(model="cmp", lower=[1000.0], upper=[5040.0], granularity=[40], apm=0.0,
                h0=0.0, tau_index=2),
    "zocrs": dict(model="zocrs", lower=[1414.2136, -1e-3, -1e-7],
                  upper=[6324.5553, 1e-3, 1e-7], granularity=[5, 3, 3], apm=60.0, h0=0.0,
                  tau_index=2),
    "oct": dict(model="oct", lower=[1200.0, -1e-3], upper=[5000.0, 1e-3], granularity=[6, 3],
                apm=40.0, h0=200.0, tau_index=2),
}


def oracle_compute(samples, mid, hoff, dt, m0s, spec):
    """The shard driver's compute step on the oracle (the CPU stand-in for a
    rank's GPU): selection on the rank's trace slice, grid, evaluation,
    argmax."""
    from oracle import oracle
    cands = (oracle.oct_selection_candidates(spec["lower"], spec["upper"])
             if spec["model"] == "oct" else None)
    out, _, _ = oracle.linear_search(spec["model"], samples, mid, hoff, m0s, dt,
                                     spec["tau_index"], spec["lower"], spec["upper"],
                                     spec["granularity"], spec["apm"], spec["h0"],
                                     oct_cands=cands, nthreads=1)
    return out


def _worker(rank, world, port, out_dir, model):
    import torch.distributed as dist
    from highperformanceseismicstacking_gb300 import shard_driver
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    line = _line(model)
    part = shard_driver.run_shard(line.samples, line.midpoints, line.halfoffsets,
                                  float(line.dt), line.cdp_midpoints, SPECS[model], world, rank,
                                  oracle_compute)
    # a rank reads its own traces and the halo only
    ta, tb = part["traces"]
    assert tb - ta < line.midpoints.size or world == 1
    parts = [None] * world
    dist.all_gather_object(parts, part)
    if rank == 0:
        np.save(os.path.join(out_dir, "sharded.npy"), shard_driver.assemble(parts))
    dist.barrier()
    dist.destroy_process_group()


@pytest.mark.parametrize("model", ["cmp", "zocrs", "oct"])
def test_two_rank_gloo_sharding_matches_single_process(tmp_path, model):
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path), model), nprocs=2,
                       start_method="spawn")
    got = np.load(tmp_path / "sharded.npy")
    line = _line(model)
    want = oracle_compute(line.samples, line.midpoints, line.halfoffsets, float(line.dt),
                          line.cdp_midpoints, SPECS[model])
    assert got.shape == want.shape
    assert np.array_equal(got, want)


def test_shard_plan_splits_at_interior_cmps():
    line = _line("zocrs")
    r = sharding.selection_radius("zocrs", 60.0)
    plans = [sharding.shard_plan(line.cdp_midpoints, line.midpoints, 2, k, r) for k in range(2)]
    (a0, b0), (ta0, tb0) = plans[0]
    (a1, b1), (ta1, tb1) = plans[1]
    assert (a0, b1) == (0, line.cdp_midpoints.size) and b0 == a1
    # the halos overlap: rank 0 reads past its last midpoint, rank 1 before its first
    assert tb0 > np.searchsorted(line.midpoints, line.cdp_midpoints[b0 - 1], side="right")
    assert ta1 < np.searchsorted(line.midpoints, line.cdp_midpoints[a1], side="left")


def test_driver_arguments_take_negative_exponents():
    """Parameter bounds like -1e-3 are values of --lower / --upper, as the
    module's usage line writes them."""
    from highperformanceseismicstacking_gb300 import shard_driver
    a = shard_driver.parse_args(["--input", "l.su", "--model", "zocrs", "--lower", "1414.2136",
                                 "-1e-3", "-1e-7", "--upper", "6324.5553", "1e-3", "1e-7",
                                 "--granularity", "41", "21", "21", "--apm", "375",
                                 "--tau", "0.010", "--output", "r.npy"])
    assert a.lower == [1414.2136, -1e-3, -1e-7]
    assert a.upper == [6324.5553, 1e-3, 1e-7]
    assert a.granularity == [41, 21, 21]
