"""bench.py's reference arm runs on the host's cores (no GPU): its JSON line carries the keys the
benchmark contract names, and the batched workloads print an `unavailable` line instead."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parent.parent


def _last_json(args):
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), *args], capture_output=True,
                       text=True, timeout=600, cwd=ROOT)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    return json.loads(lines[0])


def test_reference_arm_line_on_the_uv_sphere():
    d = _last_json(["--impl", "reference", "--workload", "uvsphere", "--steps", "1",
                    "--warmup", "1", "--cpu-sample", "2000"])
    assert d["impl"] == "reference" and d["unit"] == "queries/s" and d["value"] > 0
    assert d["higher_is_better"] is True and d["steps"] == 1 and d["warmup"] == 1
    assert d["config"]["workload"].startswith("uv_sphere") and d["config"]["triangles"] == 3968
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["cores"] >= 1 and cb["kind"] in ("port", "reference")
    assert "2000 queries per step" in cb["sample"]
    e2e = d["e2e"]
    assert e2e["value"] == d["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_forest_is_unavailable():
    d = _last_json(["--impl", "reference", "--workload", "forest", "--steps", "1"])
    assert d["impl"] == "reference" and "unavailable" in d
