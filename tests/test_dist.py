"""Multi-process plumbing of bench.py on CPU (gloo, world size 2): shards are
disjoint and cover every unit, the max/sum reductions and barrier agree on all
ranks, and the reference arm prints exactly one line from rank 0."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, q):
    os.environ.update(RANK=str(rank), WORLD_SIZE=str(world), LOCAL_RANK=str(rank), MASTER_ADDR="127.0.0.1",
                      MASTER_PORT=str(port))
    sys.path.insert(0, os.path.join(REPO, "astrogenesis2.0_gb300"))
    import dist

    d = dist.init(backend="gloo")
    units = list(dist.shard(11, d))
    mx = dist.max_over_ranks(float(rank + 1) * 1.5, d)
    sm = dist.sum_over_ranks(float(len(units)), d)
    dist.barrier(d)
    q.put((rank, units, mx, sm))
    dist.finalize(d)


def test_gloo_world2_shard_and_reductions():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, u0, mx0, sm0), (r1, u1, mx1, sm1) = out
    assert sorted(u0 + u1) == list(range(11)) and not set(u0) & set(u1)
    assert abs(len(u0) - len(u1)) <= 1
    assert mx0 == mx1 == 3.0
    assert sm0 == sm1 == 11.0


def test_single_process_is_not_distributed():
    sys.path.insert(0, os.path.join(REPO, "astrogenesis2.0_gb300"))
    import dist

    env = {k: os.environ.pop(k) for k in ("WORLD_SIZE", "RANK", "LOCAL_RANK") if k in os.environ}
    try:
        d = dist.init()
        assert not d.active and list(dist.shard(5, d)) == list(range(5))
        assert dist.max_over_ranks(2.5, d) == 2.5
    finally:
        os.environ.update(env)


@pytest.mark.skipif(not os.path.exists(os.path.join(REPO, "oracle", "liboracle.so")), reason="oracle not built")
def test_reference_arm_under_torchrun_prints_one_line():
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(_free_port()), os.path.join(REPO, "bench.py"), "--impl", "reference",
           "--workload", "plummer16k", "--steps", "1", "--warmup", "1", "--gpus", "2"]
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [json.loads(x) for x in r.stdout.splitlines() if x.startswith("{")]
    assert len(lines) == 1 and lines[0]["impl"] == "reference" and lines[0]["value"] > 0
