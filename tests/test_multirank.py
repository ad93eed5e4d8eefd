"""The multi-GPU form of the benchmark: one process per GPU and no
collective on the data path.  A replica list (temperature or field sweep)
is split over the ranks, balanced by spin count; a single-replica workload
runs as an independent copy per rank.  The host logic (process group,
per-rank workloads, max over ranks, whole-job rate, end-of-run gather) runs
here as two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _bench():
    import sys

    sys.path.insert(0, ROOT)
    import bench

    return bench


@pytest.mark.parametrize("world", [1, 2, 3, 4, 8])
def test_split_replicas_covers_the_list_once_and_balances_spins(world):
    bench = _bench()
    w = bench.WORKLOADS["sc_sweep256"]()
    spins = [int(np.prod(r.L)) * w.model.nb for r in w.replicas]
    parts = bench.split_replicas(spins, world)
    assert len(parts) == world
    flat = [i for p in parts for i in p]
    assert sorted(flat) == list(range(len(spins)))          # every replica, once
    assert all(p == sorted(p) and p for p in parts)          # ascending, none empty
    totals = [sum(spins[i] for i in p) for p in parts]
    assert max(totals) - min(totals) <= max(spins)            # within one replica of balanced


def test_split_replicas_edge_cases():
    bench = _bench()
    assert bench.split_replicas([5, 5, 5], 1) == [[0, 1, 2]]
    assert bench.split_replicas([7], 2) == [[0], []]          # more ranks than replicas: an empty rank
    assert bench.split_replicas([], 2) == [[], []]
    with pytest.raises(ValueError):
        bench.split_replicas([1], 0)


def rank_main(rank, world, port, out):
    import sys

    sys.path.insert(0, ROOT)
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), RANK=str(rank), WORLD_SIZE=str(world),
                      LOCAL_RANK=str(rank))
    import bench
    import torch.distributed as dist

    r, n, local = bench.dist_env()
    bench.init_ranks(n, local, backend="gloo")
    w = bench.rank_workload("sc_sweep256", r, n)
    spins = sum(int(np.prod(x.L)) for x in w.replicas)
    copy = bench.rank_workload("bcc64_3shell", r, n)         # a single replica: one copy per rank
    t = 1.0 + 0.5 * r                      # this rank's timed seconds
    slowest = bench.max_over_ranks(t, n)
    total = int(bench.sum_over_ranks(float(spins), n))
    bench.barrier(n)
    gathered = bench.gather_scalars([float(i) for i in w.replica_ids], n)
    rate = bench.job_rate(total, 100, slowest)
    out.put((r, w.seed, copy.seed, spins, total, slowest, rate, gathered))
    dist.destroy_process_group()


def test_two_gloo_ranks_split_the_replica_list_and_agree_on_the_job_rate():
    import torch.multiprocessing as mp

    bench = _bench()
    full = bench.WORKLOADS["sc_sweep256"]()
    all_spins = sum(full.spins_per_replica)
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
    (r0, seed0, cseed0, n0, tot0, t0, rate0, g0), (r1, seed1, cseed1, n1, tot1, t1, rate1, g1) = res
    assert seed0 == seed1                   # one job, split: the same seed
    assert cseed0 != cseed1                 # single-replica copies: independent seeds
    assert n0 + n1 == tot0 == tot1 == all_spins
    assert abs(n0 - n1) <= max(full.spins_per_replica)
    assert t0 == t1 == 1.5                  # the slowest rank's time
    assert rate0 == rate1 == all_spins * 100 / 1.5
    assert g0 == g1
    ids = [int(i) for part in g0 for i in part]
    assert sorted(ids) == list(range(len(full.replicas)))   # disjoint, and together the full list


def test_reference_arm_runs_on_rank_zero_only():
    bench = _bench()
    args = bench.parse(["--impl", "reference"])
    assert bench.run_reference(args, rank=1, world=2) == 0


def test_reference_arm_prints_the_contract_line():
    """`bench.py --impl reference` on the CPU: one JSON line with the arm's
    metric, a cpu_baseline describing the run and an e2e object with no
    host-device traffic (a small workload, so the test takes a second)."""
    import json
    import subprocess
    import sys
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    out = subprocess.run([sys.executable, os.path.join(root, "bench.py"), "--impl", "reference", "--workload", "sc32",
                          "--steps", "3", "--warmup", "3"], capture_output=True, text=True, timeout=600, cwd=root)
    assert out.returncode == 0, out.stderr[-2000:]
    lines = [ln for ln in out.stdout.splitlines() if ln.startswith("{")]
    assert len(lines) == 1
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["unit"] == "spin-steps/s" and d["higher_is_better"] is True
    assert d["value"] > 0 and d["steps"] == 3 and d["warmup"] == 3 and d["n_gpus"] == 1
    assert d["config"]["workload"] == "sc32" and d["config"]["spins"] == 32768
    cb = d["cpu_baseline"]
    assert cb["value"] == d["value"] and cb["kind"] in ("port", "reference") and cb["cores"] >= 1 and cb["sample"]
    assert d["e2e"] == {"value": d["value"], "unit": "spin-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}
