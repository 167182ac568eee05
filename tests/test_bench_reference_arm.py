"""bench.py's reference arm (the oracle's whole narrow-phase pass on the host
cores) on a small pile: it needs no GPU, prints one JSON line with the
contract's keys, and its time per step is the passes' own wall time."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_small_pile():
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--bodies", "20", "--steps", "2", "--warmup", "1"],
                       capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["value"] > 0 and line["higher_is_better"] is True
    n = line["config"]["ccd_candidates"] + line["config"]["discrete_candidates"]
    # value = candidates / mean pass time
    assert abs(line["value"] * line["ms_per_step"] / 1e3 - n) <= 1e-6 * n
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["value"] == line["value"]
