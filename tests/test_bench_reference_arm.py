"""The benchmark's reference arm (bench.py --impl reference) on the host alone: one JSON line with
the metric, the CPU baseline it timed (the oracle's KineticMcFirstOmp restatement on the host
threads), no host-device copies, and none of the package's native library loaded in the process."""
import json
import os
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]

PROBE = """
import runpy, sys
sys.argv = ["bench.py", "--impl", "reference", "--steps", "1", "--warmup", "0", "--cpu-cmc-attempts", "20000"]
runpy.run_path("bench.py", run_name="__main__")
loaded = [m for m in sys.modules if m.startswith("latticemontecarlo_gb300")]
print("LOADED " + json.dumps(loaded))
"""


def test_reference_arm_line():
    env = dict(os.environ, OMP_NUM_THREADS="4")
    out = subprocess.run([sys.executable, "-c", "import json\n" + PROBE], cwd=ROOT, env=env, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = out.stdout.strip().splitlines()
    d = json.loads(lines[-2])
    assert d["impl"] == "reference" and d["unit"] == "events/s" and d["value"] > 0
    assert d["e2e"] == {"value": d["value"], "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["cpu_baseline"]["value"] == d["value"] and d["cpu_baseline"]["kind"] in ("port", "reference")
    assert d["cmc"]["value"] > 0
    assert json.loads(lines[-1][len("LOADED "):]) == []
