"""Multi-process driver over one line: one process per GPU, each taking a
contiguous range of the line's CDP midpoints and the traces within its
selection radius (sharding.shard_plan), running the engine on that slice,
and rank 0 gathering the result blocks in midpoint order.

This replaces the reference's split of a job across GPU threads
(SingleHostRunner.cpp:141-148) and across SPITS tasks
(SpitzJobManager.cpp:17-42) for one node with one process per GPU.  There is
no collective on the data path: every rank reads the line, uploads its own
slice and computes alone; the ranks meet once, for the final gather of host
arrays (torch.distributed gather_object over gloo, or a single process).

    torchrun --nproc-per-node N --master-addr 127.0.0.1 -m \\
        highperformanceseismicstacking_gb300.shard_driver --input line.su \\
        --model zocrs --lower 1414.2136 -1e-3 -1e-7 --upper 6324.5553 1e-3 1e-7 \\
        --granularity 41 21 21 --apm 375 --tau 0.010 --output result.npy
"""
from __future__ import annotations

import argparse
import os
import re
from ctypes import c_int as C_int
from typing import Callable, Dict, Optional, Sequence

import numpy as np

from . import sharding


def engine_compute(device: int) -> Callable:
    """compute(samples, mid, hoff, dt, m0s, spec) on the GPU engine."""
    def compute(samples, mid, hoff, dt, m0s, spec):
        from . import capi
        with capi.Engine(device) as eng:
            eng.upload_gather(samples, mid, hoff, dt, storage=spec.get("storage", "fp32"))
            eng.set_traveltime(spec["model"], spec["lower"], spec["upper"], spec.get("apm", 0.0),
                               spec.get("h0", 0.0))
            eng.set_window(spec["tau_index"])
            if spec.get("h0s"):
                eng.set_oct_half_offsets(spec["h0s"])
            alg = spec.get("algorithm", "linear-search")
            if alg == "linear-search":
                out, _ = eng.linear_search(m0s, spec["granularity"], spec.get("kernel", "tuned"))
            elif alg == "de":
                out, _ = eng.differential_evolution(m0s, spec["population"], spec["generations"],
                                                    spec["F"], spec["CR"], spec["seed"])
            else:
                raise ValueError(f"unknown algorithm {alg}")
            return out
    return compute


def run_shard(samples: np.ndarray, mid: np.ndarray, hoff: np.ndarray, dt: float,
              cdp_m0s: np.ndarray, spec: Dict, world: int, rank: int,
              compute: Callable) -> Dict:
    """This rank's part: its midpoints, the trace slice it reads and the
    result blocks compute() returns for them (h0-major blocks for an OCT
    half-offset list)."""
    radius = sharding.selection_radius(spec["model"], spec.get("apm", 0.0),
                                       float(np.max(np.abs(hoff))) if hoff.size else 0.0,
                                       spec.get("h0s") or [spec.get("h0", 0.0)])
    (ma, mb), (ta, tb) = sharding.shard_plan(cdp_m0s, mid, world, rank, radius)
    part = {"rank": rank, "midpoints": (ma, mb), "traces": (ta, tb), "result": None}
    if mb > ma:
        part["result"] = compute(np.ascontiguousarray(samples[ta:tb]),
                                 np.ascontiguousarray(mid[ta:tb]),
                                 np.ascontiguousarray(hoff[ta:tb]), dt,
                                 np.ascontiguousarray(cdp_m0s[ma:mb]), spec)
    return part


def assemble(parts: Sequence[Dict], n_blocks: int = 1) -> np.ndarray:
    """Rank 0: the result blocks of all ranks in midpoint order.  With an OCT
    half-offset list every part is [n_blocks * n_i][...], h0-major; the
    whole line's result is re-laid out the same way, [n_blocks * n][...]."""
    parts = sorted((p for p in parts if p["result"] is not None),
                   key=lambda p: p["midpoints"][0])
    if not parts:
        return np.zeros((0,))
    if n_blocks == 1:
        return sharding.gather_results([p["result"] for p in parts])
    per = [p["result"].reshape((n_blocks, -1) + p["result"].shape[1:]) for p in parts]
    whole = np.concatenate(per, axis=1)
    return whole.reshape((-1,) + whole.shape[2:])


def parse_args(argv: Optional[Sequence[str]] = None) -> argparse.Namespace:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    # parameter bounds such as -1e-3 are values, not options (argparse alone
    # takes only plain negative numbers, -1 or -0.5, for values)
    ap._negative_number_matcher = re.compile(r"^-(\d+\.?\d*|\.\d+)([eE][-+]?\d+)?$")
    ap.add_argument("--input", required=True, help="SU file of the line")
    ap.add_argument("--model", required=True, choices=["cmp", "zocrs", "oct"])
    ap.add_argument("--algorithm", default="linear-search", choices=["linear-search", "de"])
    ap.add_argument("--lower", type=float, nargs="+", required=True)
    ap.add_argument("--upper", type=float, nargs="+", required=True)
    ap.add_argument("--granularity", type=int, nargs="+")
    ap.add_argument("--apm", type=float, default=0.0)
    ap.add_argument("--aph", type=float, default=1e30)
    ap.add_argument("--tau", type=float, required=True)
    ap.add_argument("--h0", type=float, nargs="+", default=[0.0])
    ap.add_argument("--population", type=int, default=32)
    ap.add_argument("--generations", type=int, default=60)
    ap.add_argument("--de-f", type=float, default=0.5)
    ap.add_argument("--de-cr", type=float, default=0.9)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--storage", default="fp32", choices=["fp32", "bf16", "fp16"])
    ap.add_argument("--output", required=True, help=".npy of the gathered result blocks")
    return ap.parse_args(argv)


def main(argv: Optional[Sequence[str]] = None) -> int:
    a = parse_args(argv)
    from . import su
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    g = su.read_gather(a.input, aph=a.aph, apm=a.apm, tau=a.tau, emulate_eof_cdp=False)
    cdp = np.asarray(g.cdp_midpoints(), np.float32)
    spec = {"model": a.model, "algorithm": a.algorithm, "lower": a.lower, "upper": a.upper,
            "granularity": a.granularity, "apm": a.apm, "h0": a.h0[0],
            "h0s": a.h0 if len(a.h0) > 1 else None, "tau_index": g.tau_index,
            "population": a.population, "generations": a.generations, "F": a.de_f,
            "CR": a.de_cr, "seed": a.seed, "storage": a.storage}
    # one GPU per process; more processes than GPUs share them round-robin
    from . import capi
    n_dev = C_int()
    capi.lib().hpss_device_count(n_dev)
    device = local % max(1, n_dev.value)
    part = run_shard(g.samples, g.midpoints, g.halfoffsets, float(g.dt), cdp, spec, world, rank,
                     engine_compute(device))
    parts = [part]
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
        parts = [None] * world if rank == 0 else None
        dist.gather_object(part, parts, dst=0)
        dist.destroy_process_group()
    if rank == 0:
        out = assemble(parts, len(a.h0) if (a.model == "oct" and len(a.h0) > 1) else 1)
        np.save(a.output, out)
        print(f"{len(cdp)} midpoints on {world} ranks -> {a.output} {out.shape}")
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
