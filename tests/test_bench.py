"""bench.py's output contract, on the CPU: the reference arm (the oracle's
restatement of the reference kernels on host threads, since the reference's
CPU path is an OpenCL build with no OpenCL device here) prints one JSON line
with the keys the bench contract names, and the committed ncu summary of the
headline kernel gives the DRAM traffic per launch the GPU arm reports."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))


def test_reference_arm_prints_the_contract_line():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                       timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config",
              "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["value"] > 0 and line["unit"] == "evals/s"
    assert line["cpu_baseline"]["kind"] in ("port", "reference")
    assert line["cpu_baseline"]["cores"] >= 1 and line["cpu_baseline"]["sample"]
    assert line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["config"]["workload"] == "cmp-production"


def test_headline_traffic_from_the_committed_profile():
    import bench
    val, note = bench.profile_traffic("ls_tuned_cmp-production")
    assert val is not None and 5e8 < val < 2e9   # ~1 GB of amplitudes per launch
    assert note and "2000/300" in note


def test_profile_cases_are_listed():
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--help"], capture_output=True,
                       text=True, timeout=120, cwd=ROOT)
    assert r.returncode == 0
    for case in ("cmp", "cmpbf16", "cmpplain", "cmpsf", "octde", "octls", "octsf", "zocrs",
                 "zocrsbf16", "zocrsde", "zocrsf64"):
        assert case in r.stdout, case
