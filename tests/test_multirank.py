"""The N>1 path on CPU (gloo, two ranks): the path does not shard, so N GPUs run
N independent replicas; these tests cover the host side of that: process-group
setup from the torchrun environment, the barrier, the max-over-ranks step
time, and the reference arm's rank-0-only line."""
import json
import os
import socket
import subprocess
import sys

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _torchrun(args, timeout=300, attempts=2):
    """Two ranks under torchrun on 127.0.0.1. A launch that fails is retried once on
    a fresh port: the port is picked before torchrun binds it, so another process
    can take it in between; a real failure fails both times."""
    env = dict(os.environ, OMP_NUM_THREADS="2")
    for _ in range(attempts):
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
               "--master-addr", "127.0.0.1", "--master-port", str(_free_port())] + args
        res = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=timeout, env=env)
        if res.returncode == 0:
            break
    return res


def test_replica_barrier_and_max_over_ranks():
    res = _torchrun([os.path.join("tests", "mr_replicas.py")])
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(ln) for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert sorted(d["rank"] for d in lines) == [0, 1]
    assert all(d["world"] == 2 and d["max"] == 20.0 for d in lines)


def test_reference_arm_prints_one_line_from_rank_0(oracle_mod):
    res = _torchrun(["bench.py", "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1",
                     "--qubits", "10", "--layers", "1", "--ref-gates", "3"])
    assert res.returncode == 0, res.stderr[-2000:]
    lines = [json.loads(ln) for ln in res.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = lines[0]
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
