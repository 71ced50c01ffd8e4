"""The entry scripts compile (a syntax error there would only show on the GPU machine)."""
import py_compile
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_entry_scripts_compile():
    for name in ("bench.py", "__graft_entry__.py"):
        py_compile.compile(str(ROOT / name), doraise=True)


def test_reference_arm_runs_whole_gulps():
    """`bench.py --impl reference` on the plain configuration: one JSON line
    whose step is one whole searched gulp of the oracle pipeline, timed (not
    extrapolated), with the CPU named."""
    import json
    import subprocess
    import sys

    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "plain",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 1 and line["value"] > 0
    assert line["e2e"]["value"] == line["value"] and line["e2e"]["h2d_bytes_per_step"] == 0
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and "whole searched gulp" in cb["sample"]
    gulp_s = 16384 * 1.048576e-3  # the plain configuration's gulp of sky
    assert abs(line["ms_per_step"] / 1e3 - gulp_s / line["value"]) < 1e-3 * line["ms_per_step"]
