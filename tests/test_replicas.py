"""The multi-GPU path of bench.py is replicas only (each rank runs the whole
step on its own GPU, no data-path collective): its reduction of the step time
(maximum over ranks) and of the job throughput, run as two gloo ranks on CPU;
and the reference arm, which rank 0 alone runs."""
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    ms, value = bench.replica_throughput(1.0 + rank, 1000, world, "cpu")
    out[rank] = (ms, value)
    dist.barrier()
    dist.destroy_process_group()


def test_replica_throughput_two_gloo_ranks():
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.spawn(_rank, args=(world, _free_port(), out), nprocs=world, join=True)
    for r in range(world):
        ms, value = out[r]
        assert ms == 2.0  # the slowest rank's step time
        assert value == pytest.approx(world * 1000 / 2.0e-3)


def test_reference_arm_nonzero_rank_exits_without_work():
    env = dict(os.environ, RANK="1", WORLD_SIZE="2")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference"], env=env,
                       capture_output=True, text=True, timeout=120)
    assert r.returncode == 0 and r.stdout.strip() == ""


def test_reference_arm_runs_the_steps_it_is_given():
    """Rank 0 of the reference arm runs exactly the warm-up and timed steps asked,
    each on the full mesh, and prints one JSON line in the GPU arm's metric."""
    import json
    env = dict(os.environ, RANK="0", WORLD_SIZE="1")
    r = subprocess.run([sys.executable, os.path.join(ROOT, "bench.py"), "--impl", "reference", "--n", "6",
                        "--steps", "3", "--warmup", "2"], env=env, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    line = json.loads(r.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["steps"] == 3 and line["warmup"] == 2
    assert line["unit"] == "tets/s" and line["value"] > 0 and line["config"]["tets"] == 6 * 6 ** 3
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"
