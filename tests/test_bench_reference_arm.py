"""The reference arm of bench.py on the host: one JSON line with the contract's
keys, the CPU implementation's throughput as `value`, and the reference GPU
kernel reported as unavailable without a GPU (or skipped)."""
import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_json_line(built_lib, oracle):
    env = dict(os.environ, OMP_NUM_THREADS="2")
    out = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
                          "--warmup", "0", "--cpu-seconds", "1", "--skip-ref-gpu"],
                         capture_output=True, text=True, check=True, env=env, timeout=600).stdout
    lines = [l for l in out.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    for k in ("metric", "value", "unit", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "vs_baseline", "dtype", "data", "config", "impl", "cpu_baseline", "e2e"):
        assert k in j, k
    assert j["impl"] == "reference" and j["metric"] == "sDTW GCUPS" and j["unit"] == "GCUPS"
    assert j["value"] > 0 and j["cpu_baseline"]["value"] == j["value"] and j["cpu_baseline"]["kind"] == "port"
    assert j["cpu_baseline"]["cores"] == 2
    assert j["e2e"]["h2d_bytes_per_step"] == 0 and j["e2e"]["d2h_bytes_per_step"] == 0
