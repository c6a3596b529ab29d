"""bench.py's reference arm (the reference's CPU algorithm on the host
cores) needs no GPU: on a small workload it prints one JSON line with the
keys the benchmark contract names, its e2e equal to its value with no
host-link bytes."""
import json
import subprocess
import sys

from conftest import ROOT


def test_reference_arm_line(built_lib):
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--workload", "lap256",
                          "--steps", "1", "--cpu-seconds", "0.3"], capture_output=True, text=True, timeout=300,
                         cwd=str(ROOT))
    assert res.returncode == 0, res.stderr
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["higher_is_better"] is True and d["unit"] == "GFLOP/s"
    assert d["value"] > 0 and d["ms_per_step"] > 0 and d["warmup"] >= 3
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"] and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    assert d["config"]["workload"].startswith("lap256")
