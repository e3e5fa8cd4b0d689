"""The benchmark's reference arm (bench.py --impl reference) on the CPU: one
JSON line with the GPU arm's metric, unit and configuration, "impl":
"reference", a cpu_baseline describing the run, and an e2e entry with no
host-device copies.  Under torch.distributed with two gloo ranks (rendezvous
on 127.0.0.1) rank 0 alone runs and prints; rank 1 exits 0 without work."""
import json
import os
import socket
import subprocess
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _env():
    env = dict(os.environ)
    for k in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "MASTER_ADDR", "MASTER_PORT"):
        env.pop(k, None)
    return env


def _check(line):
    import bench

    assert line["impl"] == "reference"
    assert line["metric"] == bench.METRIC and line["unit"] == "DOFs/s"
    assert line["higher_is_better"] is True and line["config"]["workload"] == bench.config(1)["workload"]
    assert "arm" not in line["config"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] > 0
    assert line["e2e"] == {"value": line["value"], "unit": "DOFs/s", "h2d_bytes_per_step": 0,
                           "d2h_bytes_per_step": 0}


def test_reference_arm_line():
    res = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--steps", "1",
                          "--warmup", "0"], cwd=ROOT, env=_env(), capture_output=True, text=True,
                         timeout=600)
    assert res.returncode == 0, res.stderr
    lines = _lines(res.stdout)
    assert len(lines) == 1
    _check(lines[0])
    assert lines[0]["n_gpus"] == 1


def test_reference_arm_two_ranks():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    res = subprocess.run([sys.executable, "-m", "torch.distributed.run", "--nnodes=1",
                          "--nproc-per-node", "2", "--master-addr", "127.0.0.1", "--master-port",
                          str(port), "bench.py", "--impl", "reference", "--gpus", "2", "--steps",
                          "1", "--warmup", "0"], cwd=ROOT, env=_env(), capture_output=True,
                         text=True, timeout=600)
    assert res.returncode == 0, res.stderr[-2000:]
    lines = _lines(res.stdout)
    assert len(lines) == 1  # rank 0 only
    _check(lines[0])
    assert lines[0]["n_gpus"] == 2
