"""bench.py's reference arm on the host cores: one JSON line with the arm's
metric, unit and direction, its CPU baseline description and an e2e figure
without host-device copies (no GPU involved)."""

import json
import os
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_line():
    p = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "3",
                        "--cpu-spp", "1"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    line = json.loads(p.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference"
    assert (line["metric"], line["unit"], line["higher_is_better"]) == ("Msamples/s", "Msamples/s", True)
    assert line["value"] > 0 and line["steps"] == 1 and line["warmup"] == 3 and line["n_gpus"] == 1
    cb = line["cpu_baseline"]
    assert cb["value"] == line["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1
    e2e = line["e2e"]
    assert (e2e["value"], e2e["unit"], e2e["h2d_bytes_per_step"], e2e["d2h_bytes_per_step"]) == (
        line["value"], line["unit"], 0, 0)
    assert "enclosed box 512x512, 256 spp" in line["config"]["workload"]


def test_reference_arm_under_torchrun_prints_once():
    """Launched like the multi-GPU arm (torchrun, 2 ranks): rank 0 alone runs and
    prints; the other rank exits 0 without work."""
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29731", "bench.py", "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "3", "--cpu-spp", "1"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    assert json.loads(lines[0])["impl"] == "reference"
