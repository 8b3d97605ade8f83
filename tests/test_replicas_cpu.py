"""The multi-GPU path is replicas only: each rank solves its own pairs and the
job's throughput is all ranks' pairs over the slowest rank's time.  Checked
with two gloo ranks on the CPU."""
import os
import socket

import pytest

torch = pytest.importorskip("torch")


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _rank(rank, port, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=2)
    import bench
    value, slowest = bench.replica_value(torch, 1000.0 + 500.0 * rank, pairs_per_rank=64, steps=10)
    out[rank] = (value, slowest)
    dist.destroy_process_group()


def test_replicas_report_all_pairs_over_the_slowest_rank():
    mp = torch.multiprocessing.get_context("spawn")
    with mp.Manager() as m:
        out = m.dict()
        port = _free_port()
        procs = [mp.Process(target=_rank, args=(r, port, out)) for r in range(2)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        for r in range(2):
            value, slowest = out[r]
            assert slowest == 1500.0
            assert value == pytest.approx(2 * 64 * 10 / 1.5)


def test_bench_gpus_flag_spawns_the_replicas_itself():
    """`python bench.py --gpus 2` outside torchrun starts two ranks with the
    torchrun environment and prints one line for the two-rank job (checked
    with synthetic per-rank times over gloo)."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--gpus", "2", "--replica-selftest",
                        "--batch", "8", "--steps", "5"], capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0, r.stderr
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["n_gpus"] == 2
    assert line["ms_per_step"] == pytest.approx(200.0 / 5)        # the slower rank: 200 ms
    assert line["value"] == pytest.approx(2 * 8 * 5 / 0.2)


def test_single_process_is_its_own_job():
    import bench
    value, slowest = bench.replica_value(torch, 2000.0, pairs_per_rank=8, steps=5)
    assert slowest == 2000.0 and value == pytest.approx(20.0)
