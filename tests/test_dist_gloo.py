"""The N > 1 path of bench.py on CPU: two ranks over gloo.

The operator does not shard across GPUs here (replicas): every rank runs the
whole workload, the job's time is its slowest rank's and its throughput counts
the units of all ranks; replica results must agree bit for bit.  These tests
run the host logic of that path with the gloo backend and the reference arm
under torchrun with two ranks (rank 0 alone runs and prints).
"""
import json
import os
import socket
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, q):
    import numpy as np
    import torch.distributed as dist
    sys.path.insert(0, ROOT)
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import bench
    import pdg_oracle as O
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank,
                            world_size=world)
    try:
        # slowest rank defines the job time
        t = bench.max_over_ranks(1.0 + rank, world)
        # a replica: the same seeded apply on every rank (the oracle on a small grid)
        rng = np.random.default_rng(3)
        P = O.Problem(3, 2, (3, 3, 2), alpha=3.0, K=np.exp(rng.standard_normal(18)))
        y = P.jacobian_apply(rng.uniform(-1, 1, P.ndof))
        sums = bench.gather_checksums(float(np.sum(y)), world)
        q.put((rank, t, sums, bench.job_throughput(world, P.ndof, t)))
    finally:
        dist.destroy_process_group()


def test_replica_host_logic_two_ranks_gloo(oracle):
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.SimpleQueue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    out = sorted(q.get() for _ in range(2))
    for rank, t, sums, rate in out:
        assert t == 2.0                       # max over ranks of 1.0, 2.0
        assert len(sums) == 2 and sums[0] == sums[1]
        assert rate == 2 * 486 / 2.0          # 2 ranks x 486 DoF (18 cells x 27) / slowest time


def test_single_rank_is_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.gather_checksums(2.0, 1) == [2.0]
    assert bench.job_throughput(1, 10, 2.0) == 5.0


def test_reference_arm_under_torchrun_two_ranks(oracle):
    env = dict(os.environ, PYTHONPATH=ROOT)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node",
           "2", "--master-addr", "127.0.0.1", "--master-port", str(_free_port()), "bench.py",
           "--impl", "reference", "--gpus", "2", "--cells", "6", "--steps", "1", "--warmup", "3"]
    r = subprocess.run(cmd, cwd=ROOT, env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1                    # rank 0 alone prints
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["value"] > 0
    assert d["config"]["workload"] == "sipg3d_q2_6^3_f64_apply"
    assert d["e2e"]["h2d_bytes_per_step"] == 0
