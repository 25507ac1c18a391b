"""The multi-replica path of bench.py on CPU: two gloo ranks aggregate their
timings as the torchrun launch on N GPUs does (max over ranks, every rank's
frames counted), and the reference arm runs on rank 0 only."""
import json
import os
import subprocess
import sys
from pathlib import Path

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

REPO = Path(__file__).resolve().parents[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sys.path.insert(0, str(REPO))
    import bench

    elapsed, e2e, value, e2e_value = bench.aggregate_ranks(10.0 + rank, 20.0 + 3 * rank, steps=50,
                                                           world=world, device="cpu")
    bench.barrier(world)
    out[rank] = (elapsed, e2e, value, e2e_value)
    dist.destroy_process_group()


def test_two_replicas_take_the_slowest_rank():
    world = 2
    port = 29500 + os.getpid() % 1000
    with mp.Manager() as m:
        out = m.dict()
        mp.spawn(_rank, args=(world, port, out), nprocs=world, join=True)
        res = dict(out)
    frames = 50 * 4 * world
    for rank in range(world):
        elapsed, e2e, value, e2e_value = res[rank]
        assert elapsed == 11.0 and e2e == 23.0
        assert value == pytest.approx(frames / 11.0e-3)
        assert e2e_value == pytest.approx(frames / 23.0e-3)


def test_reference_arm_rank0_only():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2", LOCAL_RANK="1")
    proc = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "2",
                           "--warmup", "3"], env=env, capture_output=True, text=True, timeout=120)
    assert proc.returncode == 0 and proc.stdout.strip() == ""
    env = dict(os.environ, RANK="0", WORLD_SIZE="1", LOCAL_RANK="0")
    proc = subprocess.run([sys.executable, str(REPO / "bench.py"), "--impl", "reference", "--steps", "2",
                           "--warmup", "3"], env=env, capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    line = json.loads(proc.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["value"] > 0 and line["cpu_baseline"]["kind"] == "port"
    assert line["e2e"]["h2d_bytes_per_step"] == 0
