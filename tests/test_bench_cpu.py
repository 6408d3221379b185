"""bench.py's contract pieces that need no GPU: the max-over-ranks timing and
barrier of the multi-replica path (world size 2 over gloo, on CPU), and the
reference arm's JSON line."""
import json
import os
import socket
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    import torch.distributed as dist

    sys.path.insert(0, REPO)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        bench.barrier(world)
        # each replica's elapsed time; the line reports the slowest
        out[rank] = bench.all_max(world, 1.5 + rank)
        bench.barrier(world)
    finally:
        dist.destroy_process_group()


def test_replicas_report_the_slowest_rank_over_gloo():
    import torch.multiprocessing as mp

    mgr = mp.Manager()
    out = mgr.dict()
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    assert dict(out) == {0: 2.5, 1: 2.5}


def test_single_process_helpers_are_identity():
    sys.path.insert(0, REPO)
    import bench

    bench.barrier(1)
    assert bench.all_max(1, 3.25) == 3.25


def test_reference_arm_prints_one_contract_line():
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "20000", "--steps", "1",
                        "--warmup", "3"], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    j = json.loads(lines[0])
    assert j["impl"] == "reference" and j["unit"] == "iter/s" and j["value"] > 0
    assert j["cpu_baseline"]["kind"] == "port" and j["cpu_baseline"]["cores"] >= 1
    assert j["e2e"] == {"value": j["value"], "unit": "iter/s", "h2d_bytes_per_step": 0,
                        "d2h_bytes_per_step": 0}
    assert j["config"]["workload"] == "c3"


@pytest.mark.parametrize("world", [2])
def test_reference_arm_other_ranks_do_no_work(world):
    env = dict(os.environ, WORLD_SIZE=str(world), RANK="1", LOCAL_RANK="1")
    r = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--n", "2000", "--steps", "1"],
                       cwd=REPO, capture_output=True, text=True, timeout=300, env=env)
    assert r.returncode == 0 and not [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
