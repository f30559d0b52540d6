"""bench.py's reference arm (the oracle timed on the host cores) prints one
JSON line with the keys the benchmark contract asks for; it runs here, on the
CPU, at a small size."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference", "--n", "4096",
                          "--steps", "1", "--warmup", "0"], capture_output=True, text=True, timeout=600, cwd=REPO)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["e2e"]["d2h_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] in ("port", "reference") and d["cpu_baseline"]["cores"] >= 1
    assert d["config"]["workload"] and d["config"]["n"] == 4096
    # the same config as the GPU arm's line (same keys and values), and the
    # single-threaded figure of the (single-threaded) reference beside it
    sys.path.insert(0, REPO)
    import bench
    assert d["config"] == bench.workload_config(4096, 1)
    one = d["cpu_baseline"]["single_core"]
    assert one["cores"] == 1 and one["value"] > 0
