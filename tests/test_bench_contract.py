"""bench.py's reference arm on the CPU: one JSON line carrying the keys of the benchmark line, with
the config the GPU arm prints for the same arguments (same workload, same graph), from a process
that loaded the oracle library and not the product's."""
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
ARGS = ["--samples", "2000", "--mutations", "20000", "--steps", "2", "--warmup", "1"]


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
    assert d["ms_per_step"] > 0
    loaded = d["reference_cpu"]["native_libraries"]
    assert any(x.endswith("liboracle.so") for x in loaded) and not any("libgrgx" in x for x in loaded), loaded
    one = d["reference_cpu"]["one_core"]["edgeK_per_s"]
    assert len(one) == 12 and all(v > 0 for v in one.values())

    monkeypatch.syspath_prepend(str(ROOT))
    import bench

    monkeypatch.setattr(sys, "argv", ["bench.py", *ARGS])
    args = bench.parse_args()
    assert d["config"]["workload"] == bench.workload_name(args, bench.workload(args))
    assert len(bench.workload(args)) == 24
    import grgl_gb300 as gx

    g = gx.window_tree_grg(2000, 20000, seed=42)
    assert d["config"] == bench.workload_config(args, bench.workload(args), bench.graph_stats(g))
