"""The N > 1 path of bench.py on CPU: two gloo ranks, each solving its own
shard of load scenarios with the oracle, combined by the same reductions the
GPU run uses (converged solves summed, time the maximum over ranks)."""
import json
import os
import socket
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

N_PER_RANK = 6


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _rank_main(rank, world, port, out_dir):
    import time

    import torch.distributed as dist

    import bench
    import oracle

    dist.init_process_group("gloo", init_method=f"tcp://127.0.0.1:{port}", rank=rank, world_size=world)
    og = oracle.Grid(os.path.join(ROOT, "tests", "golden", "c2_base.cdf"))
    base = dict(Pload=og.Pload.copy(), Qload=og.Qload.copy(), Pg=og.Pg.copy())
    seed = bench.shard_seed(bench.BASE_SEED + 7, rank)
    Pl, Ql, Pg = bench.scenarios(np, base, N_PER_RANK, seed)
    t0 = time.perf_counter()
    conv = 0
    for i in range(N_PER_RANK):
        og.set_bus(Pload=Pl[i], Qload=Ql[i], Pg=Pg[i])
        conv += og.solve(1e-8, 100, True)["converged"]
    dt = time.perf_counter() - t0
    total = bench.sum_over_ranks(conv, dist, 0)
    slowest = bench.max_over_ranks(dt, dist, 0)
    with open(os.path.join(out_dir, f"rank{rank}.json"), "w") as f:
        json.dump(dict(conv=conv, dt=dt, total=total, slowest=slowest, first_load=float(Pl[0].sum())), f)
    dist.barrier()
    dist.destroy_process_group()


def test_two_gloo_ranks_shard_scenarios(tmp_path, oracle):
    mp = pytest.importorskip("torch.multiprocessing")
    pytest.importorskip("torch.distributed")
    port = _free_port()
    mp.spawn(_rank_main, args=(2, port, str(tmp_path)), nprocs=2, join=True)
    r = [json.load(open(tmp_path / f"rank{k}.json")) for k in range(2)]
    # each rank drew its own scenarios
    assert r[0]["first_load"] != r[1]["first_load"]
    # the job's converged count is the sum over ranks, its time the slowest rank
    for k in range(2):
        assert r[k]["total"] == r[0]["conv"] + r[1]["conv"]
        assert r[k]["slowest"] == max(r[0]["dt"], r[1]["dt"])
    assert r[0]["total"] >= 2 * N_PER_RANK - 2
