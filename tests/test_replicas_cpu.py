"""The N > 1 path of bench.py on the CPU: replicas only (one independent prover per GPU, no
data-path collective), so the only cross-rank step is the max-over-ranks time of the timed
region. Two gloo ranks run the same aggregation the GPU ranks run over NCCL; the reference arm
runs on rank 0 alone and the other ranks exit without work."""
import os
import socket
import subprocess
import sys
from pathlib import Path

import torch.multiprocessing as mp

ROOT = Path(__file__).resolve().parent.parent


def _free_port() -> int:
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank: int, world: int, port: int, times, out):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    sys.path.insert(0, str(ROOT))
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        dist.barrier()
        out[rank] = bench.replica_throughput(dist, times[rank], steps=5, world=world)
        dist.barrier()
    finally:
        dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    port = _free_port()
    times = [100.0, 150.0]  # ms of the timed region on each rank
    with mp.get_context("spawn").Manager() as m:  # no fork from this multi-threaded process
        out = m.dict()
        mp.start_processes(_rank, args=(2, port, times, out), nprocs=2, start_method="spawn")
        res = dict(out)
    # every rank sees the slowest rank's time; the value counts both ranks' units
    for r in (0, 1):
        max_ms, value = res[r]
        assert max_ms == 150.0
        assert abs(value - 2 * 5 / 0.150) < 1e-9


def test_single_process_is_its_own_maximum():
    sys.path.insert(0, str(ROOT))
    import bench
    assert bench.replica_throughput(None, 200.0, steps=4, world=1) == (200.0, 20.0)


def test_reference_arm_runs_on_rank_zero_only():
    # under torchrun every rank starts bench.py; ranks other than 0 exit 0 without work or output
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1", MASTER_ADDR="127.0.0.1")
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--impl", "reference", "--gpus", "2",
                        "--steps", "1", "--warmup", "0"], capture_output=True, text=True, env=env, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    assert r.stdout.strip() == ""


def test_gpus_flag_launches_ranks_and_rank0_reports():
    # `bench.py --gpus 2` outside a launcher starts two ranks itself (torch.distributed.run); with
    # --impl reference rank 0 alone times the CPU arm, on every host core although the launcher
    # sets OMP_NUM_THREADS=1, and prints the one JSON line; rank 1 exits 0 without work
    import json
    env = {k: v for k, v in os.environ.items() if k not in ("WORLD_SIZE", "RANK", "LOCAL_RANK")}
    r = subprocess.run([sys.executable, str(ROOT / "bench.py"), "--gpus", "2", "--impl", "reference", "--n-cols", "2",
                        "--log-rows", "6", "--steps", "2", "--warmup", "1"], cwd=ROOT, env=env, capture_output=True,
                       text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1
    res = json.loads(lines[0])
    assert res["impl"] == "reference" and res["unit"] == "commit steps/s" and res["steps"] == 2
    assert res["cpu_baseline"]["cores"] == (os.cpu_count() or 1)
