"""The N > 1 host logic of bench.py on CPU ranks (gloo, world size 2): the
whole-job throughput of replicas takes the max of the ranks' times through an
all-reduce, and the reference arm under torchrun runs on rank 0 alone (the other
ranks exit 0 without output).  No GPU is involved."""
import json
import os
import subprocess
import sys

import pytest
import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _worker(rank, world, port, results):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    local = 1.0 + rank  # rank 1 is the slow one
    value, t = bench.replica_value(local, 10, world, dist, "cpu")
    results[rank] = (value, t)
    dist.destroy_process_group()


def test_replica_throughput_takes_max_over_ranks():
    world = 2
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    results = manager.dict()
    procs = [ctx.Process(target=_worker, args=(r, world, 29517, results)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    for r in range(world):
        value, t = results[r]
        assert t == 2.0
        assert value == world * 10 / 2.0


@pytest.mark.timeout(600)
def test_reference_arm_under_torchrun_prints_on_rank0_only():
    env = dict(os.environ)
    env.pop("CUDA_VISIBLE_DEVICES", None)
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", "29519", os.path.join(ROOT, "bench.py"), "--impl", "reference", "--steps", "1",
           "--warmup", "0"]
    r = subprocess.run(cmd, capture_output=True, text=True, cwd=ROOT, env=env, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    out = json.loads(lines[0])
    assert out["impl"] == "reference" and out["n_gpus"] == 2 and out["value"] > 0
    # the reference's own C++ where it builds on this host, else the numpy restatement
    assert out["e2e"]["h2d_bytes_per_step"] == 0 and out["cpu_baseline"]["kind"] in ("reference", "port")
