"""bench.py's multi-rank path on CPU: two gloo ranks (one per GPU in a real run).

Each rank reports its own time; the whole-job value is every rank's updates
over the slowest rank's time, and only rank 0 prints the reference arm.
"""
import os
import socket

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

import bench  # noqa: E402


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        slowest = bench.max_over_ranks(1.5 + rank, world)  # rank 1 is the slow one
        gups = bench.whole_job_gups(world, 1e9, 4, slowest)
        out.put((rank, slowest, gups))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_take_the_slowest_time():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    assert [r[1] for r in res] == [2.5, 2.5]
    # 2 ranks x 4 steps x 1e9 updates over 2.5 s
    assert res[0][2] == pytest.approx(3.2)


def test_single_rank_is_identity():
    assert bench.max_over_ranks(3.25, 1) == 3.25


def test_reference_arm_only_on_rank_zero():
    class Args:
        steps, warmup = 1, 0

    assert bench.run_reference(Args(), rank=1, world=2) == 0


def test_reference_arm_prints_the_contract_line():
    """``bench.py --impl reference`` (the oracle on the host cores, small
    workload here) prints one JSON line with the keys the contract asks for."""
    import json
    import subprocess
    import sys

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, "bench.py", "--impl", "reference", "--workload", "c2",
                          "--steps", "2", "--warmup", "1"], cwd=root, capture_output=True,
                         text=True, timeout=600)
    assert out.returncode == 0, out.stderr[-2000:]
    line = json.loads(out.stdout.strip().splitlines()[-1])
    assert line["impl"] == "reference" and line["unit"] == "GUPS" and line["value"] > 0
    assert line["higher_is_better"] is True and "workload" in line["config"]
    assert line["steps"] == 2 and line["warmup"] == 1  # the counts it ran
    # the same config the GPU arm reports for this workload on one GPU
    bench.N, bench.ANGLES, bench.DET = bench.WORKLOADS["c2"]
    try:
        assert line["config"] == bench.config({"parallelism": "single GPU"})
    finally:
        bench.N, bench.ANGLES, bench.DET = bench.WORKLOADS["headline"]
    cb = line["cpu_baseline"]
    assert cb["kind"] == "port" and cb["cores"] >= 1 and cb["value"] == line["value"] and cb["sample"]
    e2e = line["e2e"]
    assert e2e["value"] == line["value"] and e2e["h2d_bytes_per_step"] == 0
    assert e2e["d2h_bytes_per_step"] == 0
