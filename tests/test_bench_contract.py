"""bench.py's reference arm on the CPU: one JSON line carrying the keys of the benchmark line, on
the workload name the GPU arm prints for the same arguments."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--samples", "2000", "--mutations", "20000", "--steps", "2", "--warmup", "1", "--cpu-seconds", "1"]


def test_reference_arm_line(lib_built, monkeypatch):
    res = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", *ARGS],
                         capture_output=True, text=True, timeout=600, cwd=ROOT)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [ln for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, res.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
                "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 1 and d["n_gpus"] == 1
    assert d["value"] > 0 and d["higher_is_better"] is True and d["unit"] == "edge*K/s"
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}

    monkeypatch.syspath_prepend(str(ROOT))
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", *ARGS])
    args = bench.parse_args()
    assert d["config"]["workload"] == bench.workload_name(args, bench.workload(args))
    assert len(bench.workload(args)) == 24
