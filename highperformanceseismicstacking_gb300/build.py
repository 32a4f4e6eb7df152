"""Build the native parts in-tree: the CUDA engine (libhpss_gb300.so), the C++
host library and CLI, and the oracle's C restatement (test infrastructure).

Everything is compiled with explicit nvcc / g++ / gcc command lines, one
process per translation unit, in parallel.  Output goes under the package's
``lib/`` and ``bin/`` folders and ``oracle/`` (all git-ignored).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
LIB_DIR = PKG / "lib"
BUILD_DIR = ROOT / "_build"
ORACLE_DIR = ROOT / "oracle"

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
# --use_fast_math as the reference's cuda/Makefile:26 (same device arithmetic);
# host code without FMA contraction so x86-64 and aarch64 builds agree.
NVCC_FLAGS = [ARCH, "-lineinfo", "-O3", "--use_fast_math", "-std=c++17",
              "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
              "-Xcompiler", "-ffp-contract=off"]

LIB_NAME = "libhpss_gb300.so"
ORACLE_LIB = "liboracle.so"


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and Path(c).exists():
            return c
    raise RuntimeError("nvcc not found")


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: " + " ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(out: Path, deps) -> bool:
    if not out.exists():
        return True
    t = out.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build_engine(force: bool = False, extra_flags=(), flavour: str = "") -> Path:
    """Compile every csrc/*.cu for sm_103a and link libhpss_gb300.so.

    ``flavour`` names a separate build with ``extra_flags`` (objects in
    _build/<flavour>/, library in lib/<flavour>/), e.g. the bounds-checked
    build ``build_engine(extra_flags=["-DHPSS_CHECKED"], flavour="checked")``;
    the default build is unaffected."""
    bdir = BUILD_DIR / flavour if flavour else BUILD_DIR
    ldir = LIB_DIR / flavour if flavour else LIB_DIR
    bdir.mkdir(parents=True, exist_ok=True)
    ldir.mkdir(parents=True, exist_ok=True)
    sources = sorted(CSRC.glob("*.cu"))
    headers = list(CSRC.glob("*.cuh")) + list(CSRC.glob("*.h")) + list((ROOT / "include").glob("*.h"))
    objs = []
    jobs = []
    for src in sources:
        obj = bdir / (src.stem + ".o")
        objs.append(obj)
        if force or _stale(obj, [src, *headers]):
            jobs.append([nvcc(), *NVCC_FLAGS, *extra_flags, "-c", str(src), "-o", str(obj)])
    with cf.ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        list(ex.map(_run, jobs))
    lib = ldir / LIB_NAME
    if force or jobs or _stale(lib, objs):
        _run([nvcc(), ARCH, "-shared", "-o", str(lib), *map(str, objs), "-lcudart"])
    return lib


def build_oracle(force: bool = False) -> Path:
    """Compile the oracle's C restatement (test infrastructure) to oracle/liboracle.so."""
    src = ORACLE_DIR / "hpss_oracle.c"
    deps = [src, ORACLE_DIR / "hpss_oracle_impl.inc", ORACLE_DIR / "hpss_oracle.h"]
    out = ORACLE_DIR / ORACLE_LIB
    if force or _stale(out, deps):
        _run(["gcc", "-O2", "-ffp-contract=off", "-fopenmp", "-fPIC", "-shared", "-Wall",
              "-o", str(out), str(src), "-lm"])
    return out


def build_all(force: bool = False) -> None:
    with cf.ThreadPoolExecutor(max_workers=2) as ex:
        f1 = ex.submit(build_engine, force)
        f2 = ex.submit(build_oracle, force)
        f1.result()
        f2.result()
    try:
        from . import host_build
        host_build.build_host(force)
    except ImportError:
        pass


if __name__ == "__main__":
    build_all(force="--force" in sys.argv)
    print("built", LIB_DIR / LIB_NAME)
