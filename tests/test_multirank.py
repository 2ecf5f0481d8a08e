"""Host logic of the multi-GPU replicas path on the CPU: gloo ranks at world
size 2.  Rays are independent, so every rank traces its own rays on its own
copy of the scene with no collective on the data path; the only exchange is
the maximum of the per-rank times, and the reference arm runs on rank 0 alone."""
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


def _rank_main(rank, world, port, times, q):
    import torch.distributed as dist
    sys.path.insert(0, REPO)
    import bench
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    slowest = bench.max_over_ranks(times[rank], dist, "cpu")
    # weak scaling: each rank's rays differ (seeded by rank), the rate counts all ranks
    rays = bench.workload("soup", 0.0001, rank)[2]
    rate = bench.job_rate(rays.shape[0], world, slowest)
    q.put((rank, slowest, rate, float(rays["org_x"][0])))
    dist.barrier()
    dist.destroy_process_group()


def test_max_over_ranks_and_job_rate_gloo():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    times = [0.25, 0.5]
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, times, q)) for r in range(2)]
    for p in procs:
        p.start()
    out = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(60)
        assert p.exitcode == 0
    assert [o[1] for o in out] == [0.5, 0.5]
    assert out[0][2] == out[1][2] == pytest.approx(2 * 1600 / 0.5 / 1e6)
    assert out[0][3] != out[1][3]  # each rank traces its own rays


def test_max_over_ranks_without_group():
    sys.path.insert(0, REPO)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.job_rate(16_000_000, 4, 0.02) == pytest.approx(3200.0)


def test_reference_arm_prints_on_rank_zero_only():
    """`bench.py --impl reference` under torchrun at world size 2: rank 0 times
    the reference path on the host (the reference library where it is built, else
    the oracle port scaled by the measured reference/port ratio) and prints one
    JSON line, rank 1 exits 0 without work."""
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes", "1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(REPO, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--scale", "0.001", "--steps", "1", "--warmup", "0",
           "--cpu-seconds", "0.2"]
    env = dict(os.environ, OMP_NUM_THREADS="1")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, env=env, cwd=REPO)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["value"] > 0
    cb = line["cpu_baseline"]
    assert cb["kind"] in ("reference", "port")
    if cb["kind"] == "port":
        assert cb["port_measured"] > 0 and cb["value"] == pytest.approx(cb["port_measured"] * cb["scaled_by_ref_over_port"])
    assert line["e2e"]["h2d_bytes_per_step"] == 0
