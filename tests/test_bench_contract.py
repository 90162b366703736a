"""bench.py's reference arm keeps the one-JSON-line contract, on one process
and under torch.distributed.run, where only rank 0 measures and prints."""
import json
import os
import subprocess
import sys

from tests.conftest import ROOT

KEYS = {"impl", "metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step",
        "higher_is_better", "scaling", "vs_baseline", "dtype", "data", "config", "cpu_baseline", "e2e"}


def json_lines(text):
    return [json.loads(l) for l in text.splitlines() if l.startswith("{")]


def check_line(line, gpus):
    assert KEYS <= set(line), KEYS - set(line)
    assert line["impl"] == "reference" and line["value"] > 0 and line["n_gpus"] == gpus
    assert line["cpu_baseline"]["value"] == line["value"] and line["cpu_baseline"]["cores"] >= 1
    assert line["e2e"]["value"] == line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0


def test_reference_arm_one_process():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1", "--warmup", "1",
                        "--sample-seconds", "0.5"], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    check_line(lines[0], 1)


def test_reference_arm_two_ranks():
    env = dict(os.environ, MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                        "--master-addr", "127.0.0.1", "--master-port", "29617", "bench.py", "--impl", "reference",
                        "--gpus", "2", "--steps", "1", "--warmup", "1", "--sample-seconds", "0.5"],
                       cwd=ROOT, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1  # rank 0 alone prints
    check_line(lines[0], 2)
