"""bench.py's reference arm without a GPU: one JSON line with the contract's
keys, the same config dict as the GPU arm builds for the same arguments,
a CPU baseline describing the run and an e2e block of its own value."""
import json
import os
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line(tmp_path):
    out = subprocess.run([sys.executable, os.path.join(REPO, "bench.py"), "--impl", "reference",
                          "--workload", "nfw1m_ns512", "--steps", "1", "--warmup", "1",
                          "--ref-seconds", "1"], capture_output=True, text=True, check=True,
                         cwd=str(tmp_path), timeout=600).stdout
    lines = [ln for ln in out.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    for k in ("impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
              "higher_is_better", "config", "cpu_baseline", "e2e", "deposits_per_s"):
        assert k in d, k
    assert d["impl"] == "reference" and d["value"] > 0 and d["higher_is_better"] is True
    assert d["e2e"]["value"] == d["value"] and d["e2e"]["h2d_bytes_per_step"] == 0
    assert d["cpu_baseline"]["kind"] == "port" and d["cpu_baseline"]["value"] == d["value"]
    sys.path.insert(0, REPO)
    import bench

    class Args:
        workload, subset, nside = "nfw1m_ns512", 0, 0
    assert d["config"] == bench.bench_config(Args, 1 << 20, 512)
