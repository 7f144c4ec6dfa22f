"""The multi-rank (replicas) path of bench.py on CPU: two gloo ranks on 127.0.0.1, as a
`torch.distributed.run --nproc-per-node 2` launch starts them. The single-system force path does not shard (replicas only):
every rank runs its own copy and rank 0 reports the slowest rank's time."""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

torch = pytest.importorskip("torch")


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def torchrun(args, timeout=600):
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(free_port()), *args]
    env = dict(os.environ, OMP_NUM_THREADS="2")
    return subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=timeout, env=env)


def test_reduce_max_and_barrier_over_two_gloo_ranks(tmp_path):
    script = tmp_path / "r.py"
    script.write_text(
        "import sys, os\n"
        f"sys.path.insert(0, {ROOT!r})\n"
        "import bench\n"
        "world, rank, local, dist = bench.dist_setup()\n"
        "bench.barrier(dist)\n"
        "m = bench.reduce_max(dist, 10.0 + rank)\n"
        f"open(os.path.join({str(tmp_path)!r}, f'rank{{rank}}.txt'), 'w').write(f'{{rank}} {{world}} {{m}}')\n")
    r = torchrun([str(script)])
    assert r.returncode == 0, r.stderr[-2000:]
    # One file per rank: the ranks' stdout streams interleave.
    got = sorted((tmp_path / f"rank{k}.txt").read_text() for k in range(2))
    assert got == ["0 2 11.0", "1 2 11.0"]


def test_reference_arm_prints_one_line_from_rank_zero():
    r = torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "0", "--ref-steps", "1",
                  "--workload", "plummer16k"])
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(ln) for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["steps"] == 1 and d["warmup"] == 0  # the arm times the requested steps
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] in ("reference", "port")
