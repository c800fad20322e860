"""The N > 1 path of bench.py on CPU (torch.distributed with gloo, world_size 2):
the step does not shard, so N GPUs run N independent replicas, timed with a
barrier on both sides and the maximum over ranks; under torchrun the reference
arm runs on rank 0 alone and the other ranks exit 0 without work."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout=300):
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", str(free_port())] + args
    return subprocess.run(cmd, capture_output=True, text=True, timeout=timeout, cwd=ROOT)


def json_lines(out):
    return [json.loads(line) for line in out.splitlines() if line.startswith("{")]


def test_barrier_and_max_over_ranks(tmp_path):
    script = tmp_path / "replica.py"
    script.write_text(
        "import json, sys\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "import bench\n"
        "ws, rank, local = bench.dist_setup()\n"
        "d = bench.Dist(ws, rank, local, False)\n"
        "d.barrier()\n"
        "m = d.max(1.5 * (rank + 1))\n"
        "d.barrier()\n"
        "if rank == 0:\n"
        "    print(json.dumps({'ws': ws, 'max': m}))\n"
        "d.close()\n")
    r = torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    assert json_lines(r.stdout) == [{"ws": 2, "max": 3.0}]


def test_reference_arm_runs_on_rank_zero_only():
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--N", "16", "--steps", "1", "--warmup", "1"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = json_lines(r.stdout)
    assert len(lines) == 1
    line = lines[0]
    assert line["impl"] == "reference" and line["n_gpus"] == 2 and line["value"] > 0
    # the line reports the steps and warm-up it ran, and ms_per_step x steps is its timed time
    assert line["steps"] == 1 and line["warmup"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["e2e"]["h2d_bytes_per_step"] == 0
