"""The benchmark's reference arm on the CPU: one JSON line with the keys the benchmark contract
names, the reference's own CPU mesher timed when its harness is built (else the restatement, with
the reason on the line), on a small seeded grid."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    cmd = [sys.executable, "bench.py", "--impl", "reference", "--size", "4x3x4", "--steps", "2", "--warmup", "3"]
    env = {k: v for k, v in os.environ.items() if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK")}
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout[-2000:]
    d = json.loads(lines[0])
    for key in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better",
                "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert key in d, key
    assert d["impl"] == "reference" and d["metric"] == d["unit"] == "chunks/s"
    assert d["steps"] == 2 and d["warmup"] == 3 and d["n_gpus"] == 1 and d["higher_is_better"] is True
    assert d["value"] > 0 and d["ms_per_step"] > 0
    cpu = d["cpu_baseline"]
    assert cpu["value"] == d["value"] and cpu["cores"] >= 1 and cpu["kind"] in ("reference", "port")
    if cpu["kind"] == "port":
        assert cpu.get("why_not_reference"), "a restatement baseline says why the reference was not timed"
    assert d["e2e"] == {"value": d["value"], "unit": "chunks/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
    # a grid smaller than the sample bound: every one of its 48 chunks is timed in each step
    assert d["config"]["sample_chunks_per_step"] == 48
