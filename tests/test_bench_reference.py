"""bench.py's reference arm runs the oracle's restatement of the reference's
CPU solver on the host cores (no GPU) and prints one JSON line in the bench
contract's shape."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def test_reference_arm_line():
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True,
                         check=True, timeout=600)
    lines = [ln for ln in res.stdout.splitlines() if ln.strip()]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference"
    assert d["unit"] == "nodes/s" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["metric"].startswith("7x7 sym_fold count")
    cpu = d["cpu_baseline"]
    assert cpu["kind"] == "port" and cpu["cores"] >= 1 and cpu["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": "nodes/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
