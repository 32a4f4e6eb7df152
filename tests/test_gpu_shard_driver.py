"""The multi-process shard driver end to end on the GPU engine.

Two ranks (gloo for the final gather, one engine each on the same GPU: the
ranks' kernels never wait on one another, there is no collective on the
data path) read an SU line, each searches its contiguous range of CDPs over
the traces within the model's selection radius, and rank 0 gathers the
result blocks.  The gathered result equals one engine call over the whole
line bit for bit.
"""
import os
import socket
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
pytestmark = pytest.mark.gpu

ARGS = {
    "cmp": ["--model", "cmp", "--lower", "1000", "--upper", "5040", "--granularity", "64",
            "--tau", "0.008"],
    "zocrs": ["--model", "zocrs", "--lower", "1414.2136", "-1e-3", "-1e-7",
              "--upper", "6324.5553", "1e-3", "1e-7", "--granularity", "7", "5", "5",
              "--apm", "150", "--tau", "0.008"],
}


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _rank(rank, world, port, argv):
    sys.path.insert(0, str(ROOT))
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from highperformanceseismicstacking_gb300 import shard_driver
    assert shard_driver.main(argv) == 0


@pytest.mark.parametrize("model", ["cmp", "zocrs"])
def test_two_ranks_on_the_gpu_equal_one_call(tmp_path, model):
    import torch.multiprocessing as mp
    from highperformanceseismicstacking_gb300 import capi, su, synthetic
    line = synthetic.structured_line(n_cmp=24, fold_range=(6, 12), h_max=1000, ns=300,
                                     dt_us=4000, n_reflectors=4, f=20.0, snr=6.0, seed=97)
    path = tmp_path / "line.su"
    su.write_su(str(path), line.headers, line.samples)
    out = tmp_path / "sharded.npy"
    argv = ["--input", str(path), "--output", str(out)] + ARGS[model]
    mp.start_processes(_rank, args=(2, _free_port(), argv), nprocs=2, start_method="spawn")
    got = np.load(out)
    # one call over the whole line, on the gather shard_driver.py reads
    a = dict(zip(argv[::2], argv[1::2]))
    apm = float(a.get("--apm", 0.0))
    g = su.read_gather(str(path), aph=1e30, apm=apm, tau=float(a["--tau"]),
                       emulate_eof_cdp=False)
    i = argv.index("--lower")
    j = argv.index("--upper")
    k = argv.index("--granularity")
    n = 1 if model == "cmp" else 3
    lower = [float(v) for v in argv[i + 1:i + 1 + n]]
    upper = [float(v) for v in argv[j + 1:j + 1 + n]]
    gran = [int(v) for v in argv[k + 1:k + 1 + n]]
    with capi.Engine(0) as eng:
        eng.upload_gather(g.samples, g.midpoints, g.halfoffsets, float(g.dt))
        eng.set_traveltime(model, lower, upper, apm)
        eng.set_window(g.tau_index)
        want, _ = eng.linear_search(np.asarray(g.cdp_midpoints(), np.float32), gran, "tuned")
    assert got.shape == want.shape
    assert np.array_equal(got, want)
