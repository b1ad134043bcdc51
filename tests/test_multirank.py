"""The multi-rank side of the benchmark on CPU (gloo, world size 2): the path does
not shard (a sequence's history carries from frame to frame), so N GPUs run N
independent replicas; the job is timed by its slowest replica (barrier, then the
maximum over ranks of each rank's time) and its throughput is the units of all
ranks over that time.  The reference arm runs on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys
import time
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir, delays):
    import torch.distributed as dist
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    try:
        # each replica reports its own time; every rank learns the slowest one
        own_ms = 10.0 + 5.0 * rank
        slowest = bench.max_over_ranks(own_ms, world)
        # the timed region of a step: barrier, work of uneven length, barrier
        dist.barrier()
        t0 = time.perf_counter()
        time.sleep(delays[rank])
        measured = bench.max_over_ranks((time.perf_counter() - t0) * 1e3, world)
        dist.barrier()
        px = 3840 * 2160
        mpx = bench.job_throughput(px, world, measured / 1e3) / 1e6
        (Path(out_dir) / f"rank{rank}.json").write_text(json.dumps(dict(slowest=slowest, measured=measured, mpx=mpx)))
    finally:
        dist.destroy_process_group()


def test_replicas_are_timed_by_the_slowest_rank(tmp_path):
    import torch.multiprocessing as mp
    delays = [0.05, 0.25]
    mp.start_processes(_rank_main, args=(2, free_port(), str(tmp_path), delays), nprocs=2, join=True,
                       start_method="spawn")
    r = [json.loads((tmp_path / f"rank{i}.json").read_text()) for i in range(2)]
    assert r[0]["slowest"] == r[1]["slowest"] == 15.0
    assert r[0]["measured"] == r[1]["measured"]
    assert 250.0 <= r[0]["measured"] < 1000.0  # the slower rank's 0.25 s, not the faster one's
    # throughput counts both ranks' pixels over the slowest time
    assert r[0]["mpx"] == pytest.approx(2 * 3840 * 2160 / (r[0]["measured"] / 1e3) / 1e6)


def test_single_rank_needs_no_process_group():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.max_over_ranks(3.5, 1) == 3.5
    assert bench.job_throughput(100.0, 1, 2.0) == 50.0
    assert bench.job_throughput(100.0, 4, 2.0) == 200.0


def test_reference_arm_runs_on_rank_zero_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2"], env=env,
                       capture_output=True, text=True, timeout=120, cwd=str(ROOT))
    assert r.returncode == 0, r.stderr
    assert r.stdout.strip() == ""
