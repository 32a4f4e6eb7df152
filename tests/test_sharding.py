"""Midpoint sharding across ranks (CPU, gloo, world size 2).

Each rank computes its contiguous midpoint shard of a small CMP line with the
oracle (standing in for its GPU); gathering the shards in rank order must
reproduce the single-process result exactly, every midpoint exactly once, with
no collective on the data path besides the final gather of this test.
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


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    from highperformanceseismicstacking_gb300 import synthetic
    from oracle import oracle
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    line = synthetic.cmp_line(n_cmp=5, halfoffsets=[25, 75, 125, 175, 225], ns=120,
                              dt_us=4000, n_reflectors=2, n_multiples=0, f=25.0, snr=10.0,
                              seed=91)
    a, b = sharding.shard_midpoints(line.cdp_midpoints, world, rank)
    out, _, _ = oracle.linear_search("cmp", line.samples, line.midpoints, line.halfoffsets,
                                     line.cdp_midpoints[a:b], float(line.dt), 2, [1000.0],
                                     [5040.0], [40], nthreads=1)
    parts = [None] * world
    dist.all_gather_object(parts, out)
    if rank == 0:
        np.save(os.path.join(out_dir, "sharded.npy"), sharding.gather_results(parts))
    dist.barrier()
    dist.destroy_process_group()


def test_two_rank_gloo_sharding_matches_single_process(tmp_path):
    torch = pytest.importorskip("torch")
    import torch.multiprocessing as mp
    from highperformanceseismicstacking_gb300 import synthetic
    from oracle import oracle
    mp.start_processes(_worker, args=(2, _free_port(), str(tmp_path)), nprocs=2,
                       start_method="spawn")
    got = np.load(tmp_path / "sharded.npy")
    line = synthetic.cmp_line(n_cmp=5, halfoffsets=[25, 75, 125, 175, 225], ns=120,
                              dt_us=4000, n_reflectors=2, n_multiples=0, f=25.0, snr=10.0,
                              seed=91)
    want, _, _ = oracle.linear_search("cmp", line.samples, line.midpoints, line.halfoffsets,
                                      line.cdp_midpoints, float(line.dt), 2, [1000.0], [5040.0],
                                      [40], nthreads=1)
    assert np.array_equal(got, want)
