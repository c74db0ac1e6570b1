"""The N > 1 path of bench.py on CPU: two gloo ranks (one process each, as
torchrun launches them) run independent replicas -- each its own seeded
point cloud -- and the job's time is the slowest rank's (one MAX all-reduce
of a scalar after the timed region); the reference arm does its work on rank
0 only.  No data-path collective exists to test: replicas share nothing."""
import os
import socket

import numpy as np
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
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        r, w, local = bench.dist_env()
        pts, scale = bench.workload(4096, r)
        # a rank's "timed region": its own seconds, then the job's
        mine = 1.0 + 0.5 * r
        slowest = bench.max_over_ranks(mine, w, device="cpu")
        rate = bench.job_rate(10, w, slowest)
        # the reference arm: rank 0 works, the others return at once
        class A:  # the arguments run_reference reads before its rank check
            n = 4096
        skipped = bench.run_reference(A()) is None if r != 0 else None
        out.put((r, w, local, float(pts[0, 0]), float(pts.sum()), scale, slowest, rate, skipped))
    finally:
        dist.destroy_process_group()


def test_two_replicas_over_gloo():
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
    (r0, w0, l0, a0, s0, sc0, t0, rate0, _), (r1, w1, l1, a1, s1, sc1, t1, rate1, skip1) = res
    assert (r0, r1, w0, w1, l0, l1) == (0, 1, 2, 2, 0, 1)
    # replicas: different seeded clouds of the same size and kernel scale
    assert a0 != a1 and s0 != s1 and sc0 == sc1
    p0, _ = bench.workload(4096, 0)
    assert float(p0[0, 0]) == a0  # seeded: the same cloud in every run
    # the slowest rank's time, seen by both; whole-job rate over both ranks' steps
    assert t0 == t1 == 1.5
    assert rate0 == rate1 == pytest.approx(20 / 1.5)
    assert skip1 is True


def test_single_rank_needs_no_process_group():
    assert bench.max_over_ranks(2.5, 1) == 2.5
    assert bench.job_rate(20, 1, 4.0) == 5.0
    assert not np.array_equal(bench.workload(64, 0)[0], bench.workload(64, 1)[0])
