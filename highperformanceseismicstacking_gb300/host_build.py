"""Build the C++ host side (host/): libhpss_host.so and the three CLI programs
single_host_linear_search, single_host_de and single_host_stretch_free, linked
against the CUDA engine libhpss_gb300.so.  Plain g++ command lines; host code
is compiled without floating-point contraction so x86-64 and aarch64 builds
read SU geometry identically."""
from __future__ import annotations

import concurrent.futures as cf
import subprocess
from pathlib import Path

PKG = Path(__file__).resolve().parent
HOST = PKG / "host"
LIB = PKG / "lib"
BIN = PKG / "bin"
ROOT = PKG.parent
FLAGS = ["-O2", "-std=c++17", "-fPIC", "-Wall", "-ffp-contract=off", "-pthread",
         "-I" + str(ROOT / "include")]
MAINS = {"single_host_linear_search": "main_linear_search.cpp",
         "single_host_de": "main_differential_evolution.cpp",
         "single_host_stretch_free": "main_stretch_free.cpp"}


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("host build failed: " + " ".join(cmd) + "\n" + r.stderr)


def _stale(out: Path, deps) -> bool:
    return not out.exists() or any(Path(d).stat().st_mtime > out.stat().st_mtime for d in deps)


def build_host(force: bool = False) -> Path:
    LIB.mkdir(exist_ok=True)
    BIN.mkdir(exist_ok=True)
    deps = [HOST / "hpss_host.cpp", HOST / "hpss_host.hpp", ROOT / "include" / "hpss.h"]
    lib = LIB / "libhpss_host.so"
    if force or _stale(lib, deps):
        _run(["g++", *FLAGS, "-shared", "-o", str(lib), str(HOST / "hpss_host.cpp"),
              "-L" + str(LIB), "-lhpss_gb300", "-Wl,-rpath,$ORIGIN"])
    jobs = []
    for exe, src in MAINS.items():
        out = BIN / exe
        if force or _stale(out, [HOST / src, lib]):
            jobs.append(["g++", *FLAGS, "-o", str(out), str(HOST / src), "-L" + str(LIB),
                         "-lhpss_host", "-lhpss_gb300", "-Wl,-rpath,$ORIGIN/../lib"])
    with cf.ThreadPoolExecutor(max_workers=3) as ex:
        list(ex.map(_run, jobs))
    return lib


if __name__ == "__main__":
    build_host(force=True)
