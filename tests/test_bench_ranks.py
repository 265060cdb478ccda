"""bench.py's multi-process logic on CPU (gloo, world size 2): the timing is
the maximum over ranks, the barrier releases both ranks, the per-rank
replicas add up, and the reference arm runs on rank 0 only.  One GB300 per
process is the GPU layout; the scenes are replicas, with no data-path
collective."""
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


def _rank_main(rank, world, port, out_dir):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank),
                      WORLD_SIZE=str(world), LOCAL_RANK=str(rank))
    sys.path.insert(0, ROOT)
    import bench
    import torch.distributed as dist
    r, w, local = bench.dist_setup(None, "gloo")
    assert (r, w, local) == (rank, world, rank)
    bench.barrier(w)
    t = bench.max_over_ranks(1.5 + rank, w, "cpu")      # rank 1 is the slow one
    total = bench.max_over_ranks(float(rank + 1), w, "cpu")
    with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
        json.dump({"max": t, "total": total}, f)
    dist.destroy_process_group()


def test_max_over_ranks_and_barrier_gloo_world2(tmp_path):
    import torch.multiprocessing as mp
    port = _free_port()
    mp.start_processes(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True,
                       start_method="spawn")
    for r in range(2):
        got = json.load(open(tmp_path / f"r{r}.json"))
        assert got["max"] == 2.5
        assert got["total"] == 2.0


def test_single_process_helpers_are_identity():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.25, 1) == 3.25
    bench.barrier(1)


@pytest.mark.parametrize("rank", ["1"])
def test_reference_arm_is_silent_on_other_ranks(rank):
    env = dict(os.environ, RANK=rank, WORLD_SIZE="2", LOCAL_RANK=rank)
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "config0", "--steps", "1", "--warmup", "0"],
                       env=env, capture_output=True, text=True, timeout=120)
    assert r.returncode == 0
    assert r.stdout.strip() == ""


def test_reference_arm_line_on_rank0():
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference",
                        "--workload", "config0", "--steps", "2", "--warmup", "3"],
                       env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["warmup"] == 3 and line["steps"] == 2
    assert line["value"] > 0 and line["e2e"]["h2d_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port"
