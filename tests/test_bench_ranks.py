"""bench.py's multi-rank pieces on the host with gloo (world size 2, no GPU):
the max-over-ranks step time every rank agrees on, and the reference arm,
which only rank 0 runs and prints."""
import json
import os
import socket
import subprocess
import sys

import torch.multiprocessing as mp

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out_dir):
    import torch.distributed as dist

    sys.path.insert(0, ROOT)
    import bench

    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms = [1.5, 4.25][rank]
    got = bench.max_over_ranks(ms, world, device="cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"got": got}, f)
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_agrees_on_the_slowest(tmp_path):
    port = _free_port()
    mp.start_processes(_rank, args=(2, port, str(tmp_path)), nprocs=2, start_method="spawn", join=True)
    got = [json.load(open(tmp_path / f"r{r}.json"))["got"] for r in range(2)]
    assert got == [4.25, 4.25]


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", LOCAL_RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "1"], capture_output=True, text=True, timeout=300, cwd=ROOT,
                       env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""
