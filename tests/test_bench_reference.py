"""The reference arm of bench.py on the host CPU: one JSON line with the benchmark contract's
keys, timed on a small synthetic workload (the oracle restatement of the reference path)."""

import json
import subprocess
import sys

from conftest import REPO


def test_reference_arm_json_line():
    out = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--workload", "rhf_nao24",
                          "--steps", "2", "--warmup", "3", "--cpu-sample", "3"],
                         capture_output=True, text=True, timeout=600, cwd=str(REPO))
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [l for l in out.stdout.splitlines() if l.strip().startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in d, k
    assert d["impl"] == "reference" and d["steps"] == 2 and d["warmup"] == 3
    assert d["value"] > 0 and d["higher_is_better"] is False
    assert d["config"]["workload"] == "rhf_nao24"
    cb = d["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == d["value"]
    assert d["e2e"] == {"value": d["value"], "unit": d["unit"], "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
