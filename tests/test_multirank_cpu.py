"""The bench's multi-GPU path is replicas only: each rank advances its own box and
the ranks exchange nothing but a barrier and the maximum of their timed
intervals.  These tests run that host logic as two gloo ranks on the CPU: the
job's time is the slowest rank's, the job's rate counts every rank's cells, and
under torchrun the reference arm runs (and prints) on rank 0 alone."""
import json
import os
import socket
import subprocess
import sys

import pytest

torch = pytest.importorskip("torch")
import torch.distributed as dist  # noqa: E402
import torch.multiprocessing as mp  # noqa: E402

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world))
    sys.path.insert(0, ROOT)
    import bench
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        # rank r "took" 1 + r seconds; the job took the slowest rank's time
        t = bench.max_over_ranks(1.0 + rank, dist, "cpu")
        dist.barrier()
        rate = bench.whole_job_rate(1000, world, 3, 10, t)
        out.put((rank, t, rate))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_agree_on_the_slowest_time():
    world = 2
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_rank_main, args=(r, world, port, q)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    got = sorted(q.get(timeout=10) for _ in range(world))
    for rank, t, rate in got:
        assert t == 2.0  # max over ranks
        assert rate == pytest.approx(world * 1000 * 3 * 10 / 2.0 / 1e6)


def test_single_process_time_is_its_own():
    sys.path.insert(0, ROOT)
    import bench
    assert bench.max_over_ranks(3.5) == 3.5
    assert bench.whole_job_rate(16_777_216, 1, 3, 30, 0.339) == pytest.approx(16_777_216 * 90 / 0.339 / 1e6)


def test_reference_arm_runs_on_rank_zero_only():
    """Under torchrun with two ranks, rank 1 exits without work or output and rank
    0 prints the reference line (a small CPU sample keeps the test short)."""
    if not os.path.exists(os.path.join(ROOT, "oracle", "_build")):
        pytest.skip("the oracle is not built")
    port = _free_port()
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.join(ROOT, "bench.py"),
           "--impl", "reference", "--gpus", "2", "--steps", "1", "--warmup", "1", "--cpu-n", "16"]
    r = subprocess.run(cmd, cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    line = json.loads(lines[0])
    assert line["impl"] == "reference" and line["n_gpus"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["cpu_baseline"]["kind"] == "port"


def test_roofline_block_follows_the_stage_path_in_use():
    """The roofline names the RK stage the autotuner chose and takes that stage's
    DRAM traffic from its own committed ncu summary."""
    sys.path.insert(0, ROOT)
    import bench
    assert bench.stage_path(False, False, False) == "three_kernel"
    assert bench.stage_path(False, True, True) == "cell_flux"
    assert bench.stage_path(True, True, False) == "march"
    assert bench.stage_path(True, False, False) == "tile"
    k3, s3 = bench.STAGE_PATHS["three_kernel"]
    km, sm = bench.STAGE_PATHS["march"]
    t3, tm = bench.stage_traffic(s3, 256), bench.stage_traffic(sm, 256)
    assert t3 == 8 * bench.stage_traffic(s3, 128) and tm == 8 * bench.stage_traffic(sm, 128)
    n = 256 ** 3
    # B per cell-update: three kernels (shared geometry tables on the uniform box) vs one marching kernel
    assert 450 < t3 / n < 700 and 250 < tm / n < 320
    assert bench.stage_traffic(s3, 64) is None and bench.stage_traffic(None, 256) is None
