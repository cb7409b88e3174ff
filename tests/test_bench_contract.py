"""The bench's JSON line contract, on the arm that needs no GPU: the reference
CPU path (`bench.py --impl reference`), alone and under torchrun with two
ranks (rank 0 alone prints one line; the other rank exits 0 without work)."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
REQUIRED = ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
            "vs_baseline", "dtype", "data", "config")


def _lines(cmd):
    env = dict(os.environ, CUDA_VISIBLE_DEVICES="")
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    return [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]


def _free_port():
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        return str(sk.getsockname()[1])


def _check(line, steps, warmup):
    for k in REQUIRED:
        assert k in line, k
    assert line["impl"] == "reference"
    assert line["steps"] == steps and line["warmup"] == warmup
    assert line["value"] > 0 and line["higher_is_better"] is True
    assert "workload" in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port") and cb["cores"] >= 1 and cb["sample"]
    assert cb["value"] == line["value"] and cb["unit"] == line["unit"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["unit"] == line["unit"]
    assert e2e["h2d_bytes_per_step"] == 0 and e2e["d2h_bytes_per_step"] == 0


def test_reference_arm_line():
    lines = _lines([sys.executable, "bench.py", "--impl", "reference", "--workload", "plain", "--steps", "1",
                    "--warmup", "1"])
    assert len(lines) == 1
    _check(lines[0], 1, 1)
    assert lines[0]["n_gpus"] == 1


def test_reference_arm_under_torchrun_prints_one_line():
    lines = _lines([sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
                    "--master-addr", "127.0.0.1", "--master-port", _free_port(), "bench.py", "--impl", "reference",
                    "--workload", "plain", "--gpus", "2", "--steps", "1", "--warmup", "1"])
    assert len(lines) == 1
    _check(lines[0], 1, 1)
    assert lines[0]["n_gpus"] == 2
