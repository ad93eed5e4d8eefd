"""The multi-GPU form of the benchmark is replicas only: one process per GPU,
each integrating its own independent replicas, no collective on the data
path.  Its host logic (process group, per-rank workloads, max over ranks,
whole-job rate, end-of-run gather) runs here as two gloo ranks on the CPU."""
import os
import socket

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def rank_main(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist

    r, n, local = bench.dist_env()
    bench.init_ranks(n, local, backend="gloo")
    w = bench.rank_workload("sc_sweep256", r)
    spins = sum(int(x.L[0]) * int(x.L[1]) * int(x.L[2]) for x in w.replicas)
    t = 1.0 + 0.5 * r                      # this rank's timed seconds
    slowest = bench.max_over_ranks(t, n)
    bench.barrier(n)
    gathered = bench.gather_scalars([float(r), 10.0 + r], n)
    rate = bench.job_rate(spins, n, 100, slowest)
    out.put((r, w.seed, spins, slowest, rate, gathered))
    dist.destroy_process_group()


def test_two_gloo_ranks_run_distinct_replicas_and_agree_on_the_job_rate():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = free_port()
    procs = [ctx.Process(target=rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    (r0, seed0, n0, t0, rate0, g0), (r1, seed1, n1, t1, rate1, g1) = res
    assert seed0 != seed1                   # independent replicas per rank
    assert n0 == n1                         # same size per rank: weak scaling
    assert t0 == t1 == 1.5                  # the slowest rank's time
    assert rate0 == rate1 == 2 * n0 * 100 / 1.5
    assert g0 == g1 == [[0.0, 10.0], [1.0, 11.0]]


def test_reference_arm_runs_on_rank_zero_only():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    args = bench.parse(["--impl", "reference"])
    assert bench.run_reference(args, rank=1, world=2) == 0
