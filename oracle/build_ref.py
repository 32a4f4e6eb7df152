"""Compile the reference's own CUDA kernels, unmodified, from the reference
source tree into GPU fatbins under oracle/_ref/ (git-ignored).

Test infrastructure only: the fatbins are the reference's kernels, loaded by
oracle/ref_runner.py through the CUDA driver API to produce golden outputs on
a GB300.  Flags follow the reference's cuda/Makefile:26 (-O3 --use_fast_math),
with the target fixed to sm_103a.

Only the .cu files of the hot path are compiled; the reference's host code
(boost, SPITS) is not.  Run: python oracle/build_ref.py [reference_root]
(default: $HPSS_REFERENCE_ROOT, else the path in default_root()); where the
tree is absent nothing is built and the prebuilt fatbins are used.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / "_ref"

KERNELS = [
    "cuda/src/semblance/kernel/cmp/linear_search.cu",
    "cuda/src/semblance/kernel/cmp/common.cu",
    "cuda/src/semblance/kernel/zocrs/linear_search.cu",
    "cuda/src/semblance/kernel/zocrs/common.cu",
    "cuda/src/semblance/kernel/oct/linear_search.cu",
    "cuda/src/semblance/kernel/cmp/stretch_free.cu",
    "cuda/src/semblance/kernel/zocrs/stretch_free.cu",
    "cuda/src/semblance/kernel/oct/stretch_free.cu",
    "cuda/src/semblance/kernel/common/stretch_free.cu",
    "cuda/src/semblance/kernel/cmp/differential_evolution.cu",
    "cuda/src/semblance/kernel/zocrs/differential_evolution.cu",
    "cuda/src/semblance/kernel/oct/differential_evolution.cu",
    "cuda/src/semblance/kernel/common/differential_evolution.cu",
]


# Our own wrapper sources compiled against the reference tree (output name).
SHIMS = {
    "ref_de_f05_cr09.cu": "common_differential_evolution_f05cr09.fatbin",
}


def fatbin_name(rel: str, tag: str = "") -> str:
    parts = Path(rel).with_suffix("").parts[-2:]
    return "_".join(parts) + tag + ".fatbin"


def default_root() -> str:
    """The reference source tree: $HPSS_REFERENCE_ROOT, else the checkout
    this recipe was written against."""
    return os.environ.get("HPSS_REFERENCE_ROOT", "/root/reference")


def build(ref_root: str = None) -> list:
    ref = Path(ref_root or default_root())
    if not ref.exists():
        return []
    OUT.mkdir(exist_ok=True)
    nvcc = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
    base = [nvcc, "-fatbin", "-O3", "--use_fast_math",
            "-gencode=arch=compute_103a,code=sm_103a", "-I" + str(ref)]
    jobs = [(ref / rel, OUT / fatbin_name(rel)) for rel in KERNELS]
    jobs += [(HERE / shim, OUT / name) for shim, name in SHIMS.items()]
    todo = [(src, out) for src, out in jobs
            if not out.exists() or out.stat().st_mtime < src.stat().st_mtime]
    with cf.ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for f in [ex.submit(subprocess.run, base + ["-o", str(out), str(src)], check=True)
                  for src, out in todo]:
            f.result()
    return [out for _, out in jobs]


if __name__ == "__main__":
    for p in build(sys.argv[1] if len(sys.argv) > 1 else None):
        print(p)
