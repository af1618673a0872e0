"""Multi-process paths of bench.py on the CPU (gloo, world_size 2, 127.0.0.1).

The workload does not shard (one problem per GPU, no exchange between GPUs), so `bench.py --gpus N` runs N
independent replicas: a gloo barrier around the timed region, the maximum of the ranks' times, and rank 0 alone
prints the line.  These tests run that host logic with two processes and no GPU.
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


def _allmax_worker(rank, port, out_dir):
    os.environ.update({"MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port), "RANK": str(rank),
                       "WORLD_SIZE": "2", "LOCAL_RANK": str(rank)})
    sys.path.insert(0, ROOT)
    import bench
    dist, r, ws, local = bench.dist_init()
    got = bench.allmax(dist, 1.5 + rank)
    dist.barrier()
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump({"rank": r, "ws": ws, "local": local, "max": got}, f)
    dist.destroy_process_group()


def test_allmax_over_two_gloo_ranks(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_allmax_worker, args=(port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    res = [json.load(open(tmp_path / f"rank{r}.json")) for r in range(2)]
    assert [x["rank"] for x in res] == [0, 1]
    assert all(x["ws"] == 2 for x in res)
    assert all(x["max"] == 2.5 for x in res)  # every rank sees the slowest rank's time


@pytest.mark.timeout(900)
def test_reference_arm_under_torchrun_prints_one_line_from_rank0():
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus",
           "2", "--steps", "1", "--warmup", "3"]
    p = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=850)
    assert p.returncode == 0, p.stderr[-2000:]
    lines = [ln for ln in p.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1, p.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["e2e"]["h2d_bytes_per_step"] == 0 and d["cpu_baseline"]["kind"] == "port"
