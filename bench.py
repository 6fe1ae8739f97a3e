#!/usr/bin/env python3
"""Benchmark: converged Newton-Raphson power-flow solves per second on one GB300.

Workload c2 (default): the seeded synthetic 118-bus meshed grid (1 slack, 53 PV,
64 PQ, 177 lines + 9 transformers), 32,768 load scenarios (per-bus load x
lognormal(sigma 0.1), generator P x U(0.9, 1.1)), reactive limits on, flat start,
tolerance 1e-8 p.u., no_max_iter 100.  A step solves all 32,768 scenarios.  About
one scenario in 1,100 never converges (Newton oscillates or PV/PQ-cycles) and
runs all 100 iterations on a few SMs at the end of the step; four batches of
the same scenarios are kept in flight, one stream each, steps going round them,
so that one step's tail runs beside the next steps' bulk.
  value    batched, FP32 LU + FP64 mismatch/test/update, inputs resident in
           device memory; one graph launch per step, CUDA events on the batch
           streams; counts converged scenarios only (config.serial_solves_per_s:
           one batch, step after step)
  e2e      the same through the public API with host arrays: host->device copy
           of every scenario's loads and generation, the solve, device->host
           copy of |V|, theta, P, Q, iterations and status, every step
           (four in flight: step k is launched before step k-3's results are
           read back; c5: two)
  config   also reports the plain FP64 form (one scenario per gbpf_solve, the
           oracle-matching path) and batched FP64 on the same scenarios
Other workloads: c2-plain (one FP64 solve of the grid per step), c3 (the
15,104-bus grid, one FP64 solve per step), c4 (4,096 instances of 14..472-bus
grids, batched FP32), c5 (the learned warm start on the 1,888-bus grid: 50,000
training solves, the 5664 -> 3 x 512 -> 3776 network trained for 120 epochs on
the GPU, then a step = batched FP32 Newton from the predicted start, flat-start
fallback, over 8,192 held-out scenarios; two batches in flight).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2]
  python bench.py --impl reference     the CPU restatement of the reference
                                       path (oracle/) on every host core
Multi-GPU (torch.distributed.run, one process per GPU): scenarios are sharded
over ranks (weak scaling: every rank solves its own 32,768), no collective in
the data path; a single grid does not shard, so c2-plain/c3 run replicas.
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "experience-of-using-gpu-in-power-flow-computation_gb300"
BASE_SEED = 20261203
METRIC = "converged PF solves/s on 1 GB300 @ mismatch<=1e-8 pu"
UNIT = "solves/s"
N_SCEN = 4096           # c4 instances (and the default c2 CPU sample size)
N_SCEN_C2 = 32768       # c2 scenarios per step
IN_FLIGHT = 4           # c2/c4: batches of the same scenarios in flight, one stream each
L2_BYTES = 129 * 1024 * 1024


def args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbpf", choices=["gbpf", "reference"])
    p.add_argument("--workload", default="c2", choices=["c2", "c2-plain", "c2-dense", "c3", "c4", "c5", "c5-dense"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--scenarios", type=int, default=0,
                   help="scenarios per step (c2: default 32768, c4: 4096; c5: held-out, default 8192); smaller cases "
                        "for profiler captures")
    p.add_argument("--train", type=int, default=0, help="c5 training solves (default 50000)")
    p.add_argument("--no-autotune", action="store_true",
                   help="batched workloads: keep the default launch plan instead of the autotuner's")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def write_grid(g):
    d = tempfile.mkdtemp(prefix="gbpf_bench_")
    path = os.path.join(d, "grid.cdfx" if g.nB > 9999 else "grid.cdf")
    g.write_cdf(path)
    return path


def scenarios(np, base, n, seed):
    """Per-bus load x lognormal(sigma 0.1), generation x U(0.9, 1.1)."""
    rng = np.random.default_rng(seed)
    nb = len(base["Pload"])
    lf = np.exp(rng.normal(-0.005, 0.1, (n, nb)))
    gf = rng.uniform(0.9, 1.1, (n, nb))
    return base["Pload"] * lf, base["Qload"] * lf, base["Pg"] * gf


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.device, self.proc, self.out = device, None, None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
            time.sleep(0.5)
        except Exception:
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.3)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        if not self.proc or not self.out:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.out.flush()
        rows = []
        with open(self.out.name) as f:
            for line in f:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9 and parts[1].isdigit():
                    rows.append(parts)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"], "samples": 0}
        sm = [int(r[1]) for r in rows]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({n for r in rows for n, v in zip(names, r[5:9]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": reasons,
                "samples": len(rows)}


def peak_hbm():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        return json.load(open(p))["hbm_gbs"], "measured"
    return 6800.0, "fallback"


# ---------------------------------------------------------------------- CPU
def _oracle():
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    oracle.lib()
    return oracle


def _oracle_shard(task):
    """Worker: solve scenarios [lo, hi) of the `total` drawn with `seed` with
    the oracle; returns the converged count."""
    cdf, lo, hi, seed, lim, nreps, total = task
    import numpy as np

    oracle = _oracle()
    og = oracle.Grid(cdf)
    base = dict(Pload=og.Pload.copy(), Qload=og.Qload.copy(), Pg=og.Pg.copy())
    Pl, Ql, Pg = scenarios(np, base, total, seed)
    conv = 0
    for _ in range(nreps):
        for i in range(lo, hi):
            og.set_bus(Pload=Pl[i], Qload=Ql[i], Pg=Pg[i])
            conv += og.solve(1e-8, 100, bool(lim))["converged"]
    return conv


def cpu_baseline_scenarios(cdf, lim, seed, total, target_s=12.0):
    """The oracle on one host core over a bounded sample of the scenarios
    (about target_s seconds: the per-scenario time comes from runs of 64 and
    256 scenarios, so that a call's fixed cost -- loading the grid -- does not
    count as solving)."""
    _oracle_shard((cdf, 0, 8, seed, lim, 1, total))
    t0 = time.perf_counter()
    _oracle_shard((cdf, 0, 64, seed, lim, 1, total))
    t64 = time.perf_counter() - t0
    t0 = time.perf_counter()
    _oracle_shard((cdf, 0, 256, seed, lim, 1, total))
    t256 = time.perf_counter() - t0
    per = max((t256 - t64) / 192, t256 / 256 / 4, 1e-7)
    n = max(64, min(total, int(target_s / per)))
    t0 = time.perf_counter()
    conv = _oracle_shard((cdf, 0, n, seed, lim, 1, total))
    dt = time.perf_counter() - t0
    return {"value": conv / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {n} of the {total} scenarios, {conv} converged, {dt:.1f} s single-threaded "
                      f"oracle (oracle/pf_oracle.c via ctypes)"}


def cpu_baseline_repeat(cdf, lim, target_s=12.0):
    oracle = _oracle()
    if not os.path.exists(oracle.CLI_PATH):
        oracle.build()
    probe = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", "2"],
                                      capture_output=True, text=True, check=True).stdout)
    reps = max(2, int(target_s / max(probe["solve_s"], 1e-6)))
    r = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", str(reps)],
                                  capture_output=True, text=True, check=True).stdout)
    return {"value": 1.0 / r["solve_s"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{reps} solves of the grid ({r['iterations']} iterations each), "
                      f"{reps * r['solve_s']:.1f} s single-threaded oracle/pforacle"}


def run_reference(a):
    """--impl reference: the reference path restated in C (oracle/) on every
    host core, the same scenarios and metric.  The reference's own executables
    need MKL (absent here, and not available for the Arm host) or cuSPARSE
    calls removed from CUDA 12+, so the restatement stands in for them."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp
    import numpy as np

    gb = importlib.import_module(PKG)
    lim = 1
    if a.workload in ("c2", "c4"):
        g = gb.generate(2, BASE_SEED + 2)
        desc = (f"118-bus synthetic, {a.scenarios or (N_SCEN_C2 if a.workload == 'c2' else N_SCEN)} load "
                f"scenarios, limits on")
    elif a.workload == "c3":
        g, lim, desc = gb.generate(3, BASE_SEED + 3, tiles=128), 1, "15104-bus synthetic, limits on"
    else:
        g, desc = gb.generate(2, BASE_SEED + 2), "118-bus synthetic, limits on"
    cdf = write_grid(g)
    cores = os.cpu_count() or 1
    steps = min(a.steps, 5)
    warm = min(a.warmup, 3)
    if a.workload in ("c2", "c4"):
        total = a.scenarios or (N_SCEN_C2 if a.workload == "c2" else N_SCEN)
        per = (total + cores - 1) // cores
        tasks = [(cdf, i * per, min(total, (i + 1) * per), BASE_SEED + 7, lim, 1, total) for i in range(cores)]
        tasks = [t for t in tasks if t[1] < t[2]]
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(tasks)) as pool:
            for _ in range(warm):
                pool.map(_oracle_shard, tasks)
            t0 = time.perf_counter()
            conv = 0
            for _ in range(steps):
                conv += sum(pool.map(_oracle_shard, tasks))
            dt = time.perf_counter() - t0
        value = conv / dt
        sample = f"each step: all {total} scenarios over {len(tasks)} processes (one per core)"
    else:
        oracle = _oracle()
        probe = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", "2"],
                                          capture_output=True, text=True, check=True).stdout)
        reps = max(1, int(1.0 / max(probe["solve_s"], 1e-6)))
        def step():
            ps = [subprocess.Popen([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", str(reps)],
                                   stdout=subprocess.PIPE, text=True) for _ in range(cores)]
            for p in ps:
                p.communicate()
        for _ in range(warm):
            step()
        t0 = time.perf_counter()
        for _ in range(steps):
            step()
        dt = time.perf_counter() - t0
        value = steps * cores * reps / dt
        sample = f"each step: {cores} processes x {reps} solves of the grid"
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": steps, "warmup": warm,
            "ms_per_step": 1e3 * dt / steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": a.workload, "grid": desc, "nB": g.nB, "tolerance": 1e-8, "lim_inj_reat": lim},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


# ------------------------------------------------------------- multi-rank
def shard_seed(seed, rank):
    """Weak scaling: every rank solves its own scenarios, drawn with this seed
    (instances are independent, so the data path has no collective)."""
    return seed + 1000 * rank


def _reduce(x, dist, device, op):
    if not dist:
        return x
    import torch

    on_gpu = dist.get_backend() == "nccl"
    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{device}" if on_gpu else "cpu")
    dist.all_reduce(t, op=op)
    return float(t.item())


_PINNED = []  # the page-locked tensors behind pinned() views, kept alive


def pinned(a=None, shape=None, dtype=None):
    """A numpy view of page-locked host memory (a torch pinned tensor): a copy
    of array a, or an empty array of shape/dtype.  The end-to-end steps read
    inputs from and write results to such memory, so that the host<->device
    copies run at the DMA rate whatever the host's own memory traffic."""
    import numpy as np
    import torch
    if a is not None:
        a = np.ascontiguousarray(a)
        shape, dtype = a.shape, a.dtype
    t = torch.empty(shape, dtype=torch.from_numpy(np.zeros(0, dtype)).dtype, pin_memory=True)
    _PINNED.append(t)
    v = t.numpy()
    if a is not None:
        v[...] = a
    return v


def pinned_results(n, nb):
    """Result arrays of Batch.results(out=...) in pinned memory."""
    import numpy as np
    d = {k: pinned(shape=(n,), dtype=np.int32) for k in ("iterations", "status", "n_events")}
    d["final_mismatch"] = pinned(shape=(n,), dtype=np.float64)
    for k in ("V", "theta", "Pcalc", "Qcalc"):
        d[k] = pinned(shape=(nb,), dtype=np.float64)
    return d


def max_over_ranks(x, dist, device):
    """Step time of the job: the slowest rank."""
    return _reduce(x, dist, device, dist.ReduceOp.MAX) if dist else x


def sum_over_ranks(x, dist, device):
    """Converged solves of the job: all ranks."""
    return _reduce(x, dist, device, dist.ReduceOp.SUM) if dist else x


# ---------------------------------------------------------------------- GPU


def launches_per_solve(plan):
    """Kernels of one batch graph launch: the block kernel, the warp kernel and
    the hand-off launch, each when the plan uses it."""
    warp = plan["warp_instances"] > 0
    return int(plan["block_instances"] > 0) + int(warp) + int(warp and plan["handoff_it"] > 0)


def bench_batch(a, gb, np, rank, dev, world, dist):
    N_SCEN = a.scenarios or (globals()["N_SCEN"] if a.workload == "c4" else N_SCEN_C2)
    if a.workload == "c4":
        sizes = [14, 30, 57, 118, 236, 472]
        grids = [gb.generate(4, BASE_SEED + 4 + 1000 * i, nbus=nb) for i, nb in enumerate(sizes)]
        rng = np.random.default_rng(shard_seed(BASE_SEED + 4, rank))
        gi = rng.integers(0, len(grids), N_SCEN).astype(np.int32)
        cols = {k: [] for k in ("Pload", "Qload", "Pg")}
        for t in gi:
            b = grids[t].buses()
            lf = np.exp(rng.normal(-0.005, 0.1, grids[t].nB))
            cols["Pload"].append(b["Pload"] * lf)
            cols["Qload"].append(b["Qload"] * lf)
            cols["Pg"].append(b["Pg"] * rng.uniform(0.9, 1.1, grids[t].nB))
        Pl, Ql, Pg = (np.concatenate(cols[k]) for k in ("Pload", "Qload", "Pg"))
        desc = "4096 instances of 14/30/57/118/236/472-bus synthetic grids, load x lognormal(0.1), Pg x U(0.9,1.1)"
        cdf = None
    else:
        g0 = gb.generate(2, BASE_SEED + 2)
        cdf = write_grid(g0)
        grids = [gb.read_grid(cdf)]
        base = grids[0].buses()
        Pl, Ql, Pg = scenarios(np, base, N_SCEN, shard_seed(BASE_SEED + 7, rank))
        Pl, Ql, Pg = Pl.ravel(), Ql.ravel(), Pg.ravel()
        gi = np.zeros(N_SCEN, np.int32)
        desc = f"118-bus synthetic meshed grid (1 slack/53 PV/64 PQ, 186 branches), {N_SCEN} load scenarios"
    opts = dict(tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    fast = gb.Batch(grids, device=dev, precision=gb.PREC_FP32_IR, **opts)
    fast.set_instances(gi, Pload=Pl, Qload=Ql, Pg=Pg)
    fast.solve()
    # launch plan: the autotuner's coordinate search on these instances (setup,
    # outside the timed region), or the default plan with --no-autotune
    tune = None
    if not a.no_autotune:
        plan, ms0, ms1 = fast.autotune(repeats=3)
        tune = {"plan": plan, "ms_default_plan": ms0, "ms_chosen_plan": ms1}
    fast.solve()
    r = fast.results(state=False)
    conv = int((r["status"] == 0).sum())
    assert np.all(r["final_mismatch"][r["status"] == 0] <= 1e-8)
    # more batches of the same scenarios and plan, IN_FLIGHT in all, each on
    # its own stream: one step's hand-off tail (the few scenarios that run all
    # no_max_iter iterations on a few SMs) runs beside the next steps' bulk
    pl = fast.plan()
    ring = [fast]
    for _ in range(IN_FLIGHT - 1):
        twin = gb.Batch(grids, device=dev, precision=gb.PREC_FP32_IR, **opts)
        twin.set_instances(gi, Pload=Pl, Qload=Ql, Pg=Pg)
        twin.set_plan(**{k: pl[k] for k in ("warp_mode", "warps_per_block", "handoff_it", "resume_group",
                                            "warp_group", "narrow", "lu1", "warp_lu1", "flat_shared", "rotate",
                                            "gstate", "warp_gstate")})
        twin.solve()
        assert np.array_equal(twin.results(state=False)["status"], r["status"])
        ring.append(twin)
    pair = ring
    # the autotuner times one batch at a time; in flight, where one step's
    # tail overlaps the next steps, the hand-off iteration is chosen again
    # with the ring itself (setup, outside the timed region)
    handoff_trials = {}
    if not a.no_autotune and len(pair) > 1 and pl["warp_instances"]:
        keys = ("warp_mode", "warps_per_block", "handoff_it", "resume_group", "warp_group", "narrow", "lu1",
                "warp_lu1", "flat_shared", "rotate", "gstate", "warp_gstate")
        for ho in dict.fromkeys([pl["handoff_it"], 0, 24]):
            for b in pair:
                b.set_plan(**{**{k: pl[k] for k in keys}, "handoff_it": ho})
                b.solve()
            gb.time_pipelined(pair, 2 * len(pair))
            handoff_trials[ho] = gb.time_pipelined(pair, 4 * len(pair)) / (4 * len(pair))
        best = min(handoff_trials, key=handoff_trials.get)
        for b in pair:
            b.set_plan(**{**{k: pl[k] for k in keys}, "handoff_it": best})
            b.solve()
        r = fast.results(state=False)
        conv = int((r["status"] == 0).sum())
        assert np.all(r["final_mismatch"][r["status"] == 0] <= 1e-8)
        assert np.array_equal(pair[-1].results(state=False)["status"], r["status"])
    # device-resident: CUDA events on the batch streams; every step is a full
    # solve of all scenarios, steps go round the batches
    gb.time_pipelined(pair, max(3, a.warmup))
    fast.time(max(3, a.warmup))
    if dist:
        dist.barrier()
    with Clocks(dev) as clk:
        ms = gb.time_pipelined(pair, a.steps)
    if dist:
        dist.barrier()
    ms_serial = fast.time(a.steps)
    t_dev = max_over_ranks(ms / 1e3, dist, dev)
    total_conv = sum_over_ranks(conv, dist, dev)
    value = total_conv * a.steps / t_dev
    serial = total_conv * a.steps / max_over_ranks(ms_serial / 1e3, dist, dev)
    # end to end: host arrays through the API every step (inputs up, solve,
    # results down into host arrays), round the same batches: step i's inputs
    # go up and its solve is launched before step i-(IN_FLIGHT-1)'s results are
    # read back
    nb = len(Pl)
    kf = len(pair)
    hPl, hQl, hPg = pinned(Pl), pinned(Ql), pinned(Pg)
    outs = [pinned_results(N_SCEN, nb) for _ in range(kf)]

    def e2e_steps(k):
        for i in range(k):
            b = pair[i % kf]
            b.set_instances(gi, Pload=hPl, Qload=hQl, Pg=hPg)
            b.launch()
            if i >= kf - 1:
                j = (i - kf + 1) % kf
                outs[j] = pair[j].results(state=True, out=outs[j])
        for i in range(max(0, k - kf + 1), k):
            j = i % kf
            outs[j] = pair[j].results(state=True, out=outs[j])

    e2e_steps(max(3, a.warmup))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps(a.steps)
    t_e2e = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e = total_conv * a.steps / t_e2e
    res = outs[(a.steps - 1) % kf]
    assert np.array_equal(res["iterations"], r["iterations"])
    # the plain FP64 form (one scenario per gbpf_solve) and batched FP64, same scenarios
    plain = None
    if cdf is not None:
        s = gb.Solver(grids[0], device=dev, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1, metodo=0)
        base = grids[0].buses()
        n_plain = 256
        Pl2, Ql2, Pg2 = Pl.reshape(N_SCEN, -1), Ql.reshape(N_SCEN, -1), Pg.reshape(N_SCEN, -1)
        nconv = 0
        t0 = time.perf_counter()
        for i in range(n_plain):
            s.set_start(Pliq=Pg2[i] - Pl2[i], Qliq=base["Qg"] - Ql2[i])
            nconv += s.solve(full=False)["converged"]
        plain = nconv / (time.perf_counter() - t0)
    slow = gb.Batch(grids, device=dev, precision=gb.PREC_FP64, **opts)
    slow.set_instances(gi, Pload=Pl, Qload=Ql, Pg=Pg)
    if not a.no_autotune:
        slow.autotune(repeats=2)
    slow.solve()
    rs = slow.results(state=False)
    ms64 = slow.time(max(3, a.steps // 4)) / max(3, a.steps // 4)
    batched64 = int((rs["status"] == 0).sum()) / (ms64 / 1e3)
    info = fast.info()
    peak, src = peak_hbm()
    # algorithmic bytes of one batch launch: inputs (V0, theta0, Pliq, Qliq, Qload),
    # outputs (V, theta, P, Q) and per-instance results; topology blobs counted once
    bytes_launch = nb * 8 * 5 + nb * 8 * 4 + N_SCEN * (4 * 3 + 8)
    # the dominant kernel's own time per launch: CUDA events recorded inside
    # the graph around each kernel, on the stream it runs on
    kt = fast.kernel_times(max(3, a.steps // 4))
    pl_k = fast.plan()
    main_kernel = (f"k_nr_warp<float, {pl_k['warp_state_global']}>" if info["warp_instances"] else
                   f"k_nr_block<float, {pl_k['block_state_global']}>")
    t_launch = (kt["warp"] if info["warp_instances"] else kt["block"]) / 1e3
    achieved = bytes_launch / t_launch / 1e9
    # DRAM traffic of one k_nr_warp<float, level> launch of the 32,768 c2
    # scenarios (ncu dram__bytes_read.sum + dram__bytes_write.sum, one-pass
    # captures of full-size runs with the hand-off at iteration 12), by state
    # placement level and warps per block, scaled by instances; null for a
    # plan shape not captured
    measured = {(0, 8): 201.7e6, (3, 4): 264.4e6, (3, 6): 243.6e6, (3, 8): 233.2e6, (3, 9): 243.8e6,
                (3, 10): 264.3e6, (3, 12): 218.5e6}
    pl_now = fast.plan()
    key = (pl_now["warp_state_global"], pl_now["warps_per_block_used"])
    traffic = measured[key] * N_SCEN / 32768 if a.workload == "c2" and key in measured else None
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "grid": desc, "instances_per_gpu": N_SCEN, "tolerance": 1e-8,
                   "no_max_iter": 100, "lim_inj_reat": 1,
                   "form": "batched, FP32 LU + FP64 mismatch/test/update, flat start (the learned start: workload c5)",
                   "converged_per_step": int(total_conv), "mean_iterations": float(np.mean(r["iterations"])),
                   "max_iterations": int(np.max(r["iterations"])),
                   "plain_fp64_solves_per_s": plain, "batched_fp64_solves_per_s": batched64,
                   "speedup_vs_plain_fp64": (value / plain) if plain else None,
                   "in_flight": f"{IN_FLIGHT} batches of the same scenarios, one stream each, steps going round "
                                "them; each step a full solve of every scenario",
                   "serial_solves_per_s": serial,
                   "l2": (f"inputs+outputs {nb * 8 * 9 / 2**20:.0f} MiB > L2 (129 MB)" if nb * 72 > L2_BYTES else
                          f"inputs+outputs {nb * 8 * 9 / 2**20:.1f} MiB < L2; no flush"),
                   "batch": info, "plan": fast.plan(), "autotune": tune,
                   "in_flight_handoff_ms_per_step": handoff_trials or None,
                   "parallelism": f"scenarios sharded x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nb * 8 * 3,
                "d2h_bytes_per_step": nb * 8 * 4 + N_SCEN * 20,
                "note": "per step: the caller's Pload, Qload, Pg arrays (pinned host memory) up as they are "
                        "(packed into Pliq, Qliq, "
                        "Qload on the device; the start is the grid's own, kept on the device), V, theta, Pcalc, "
                        f"Qcalc and the per-instance results down into the caller's arrays; {IN_FLIGHT} batches in "
                        f"flight (step k is launched before step k-{IN_FLIGHT - 1}'s results are read)"},
        "roofline": {"bound": "hbm", "kernel": main_kernel, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src_note(src),
                     "traffic": traffic / 1e9 if traffic else None, "traffic_unit": "GB per launch",
                     "algorithmic_bytes_per_launch": bytes_launch,
                     "kernel_ms_per_launch": kt,
                     "note": "dependent-latency bound (ncu: issue ~25 % of active cycles, FP64 pipe ~33 %, stalls "
                             "on L2 loads of the placed state and on shared memory); the working set stays in L2 "
                             "and DRAM traffic is the inputs and outputs once; the step's remaining time is the "
                             "hand-off launch of the few instances that run all 100 iterations"},
        "clocks": clk.summary(),
        "gpu_launches": a.steps * launches_per_solve(fast.plan()),
    }
    if rank == 0 and not a.no_cpu_baseline and cdf is not None:
        line["cpu_baseline"] = cpu_baseline_scenarios(cdf, 1, BASE_SEED + 7, N_SCEN)
    return line


C5_TRAIN, C5_TEST = 50000, 8192


def c5_scenarios(np, base, n, seed):
    """Per-bus load x U(0.7, 1.3) (P and Q together), generator P x U(0.85, 1.15)."""
    rng = np.random.default_rng(seed)
    nb = len(base["Pload"])
    lf = rng.uniform(0.7, 1.3, (n, nb))
    gf = rng.uniform(0.85, 1.15, (n, nb))
    return base["Pload"] * lf, base["Qload"] * lf, base["Pg"] * gf


def train_flops_per_step(nb, width, B, k_metric):
    """Multiply-add FLOPs of the tensor-core GEMMs of one training step."""
    kin, out = 3 * nb, 2 * nb
    fwd = kin * width + 2 * width * width + width * out + kin * out
    metric = 2 * out * k_metric
    dh = out * width + 2 * width * width
    dw = width * kin + 2 * width * width + out * width + out * kin
    return 2.0 * B * (fwd + metric + dh + dw)


def bench_c5(a, gb, np, rank, dev, world, dist):
    C5_TRAIN = a.train or globals()["C5_TRAIN"]
    C5_TEST = a.scenarios or globals()["C5_TEST"]
    grid = gb.generate(3, BASE_SEED + 5, tiles=16)
    nB, base = grid.nB, grid.buses()
    opts = dict(tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    # training set: solutions of the plain Newton method (batched FP64, flat start)
    Pl, Ql, Pg = c5_scenarios(np, base, C5_TRAIN, shard_seed(BASE_SEED + 5, rank))
    gen = gb.Batch([grid], device=dev, precision=gb.PREC_FP64, **opts)
    t0 = time.perf_counter()
    gen.set_instances(np.zeros(C5_TRAIN, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    gen.solve()
    r = gen.results()
    t_gen = time.perf_counter() - t0
    ok = r["status"] == 0
    V, th = r["V"].reshape(-1, nB)[ok], r["theta"].reshape(-1, nB)[ok]
    X = gb.warm_features(Pg[ok] - Pl[ok], base["Qg"] - Ql[ok], np.tile(base["V0"], (int(ok.sum()), 1)))
    Y = gb.warm_targets(V, th)
    gen.close()
    del r, Pl, Ql, Pg
    # batch 1024 at lr 2e-3, 120 epochs: against batch 256 at 1e-3 for 60
    # epochs, 3.5x the tensor-core rate (146 vs 42 TFLOP/s), 6.1 vs 10.8 s,
    # lower loss and fewer iterations from the predicted start (3.13 vs 3.27)
    width, batch, epochs, lam, lr0 = 512, 1024, 120, 1.0, 2e-3
    m = gb.MLP(3 * nB, 2 * nB, width=width, n_layers=3, skip=True, seed=BASE_SEED + 5, device=dev)
    m.set_data(X, Y)
    plain = gb.Solver(grid, device=dev, metodo=0, **opts)
    A = gb.warm_loss_metric(plain, V.mean(0), th.mean(0), m.norm()["out_scale"])
    m.set_loss_metric(A, lam)
    loss, train_ms = m.train(epochs, batch=batch, lr=lr0, lr_final=1e-5, seed=BASE_SEED + 5)
    steps_per_epoch = len(X) // batch
    train_tflops = train_flops_per_step(nB, width, batch, (A.shape[1] + 7) // 8 * 8) * steps_per_epoch * epochs / (
        train_ms / 1e3) / 1e12
    del X, Y, V, th
    # held-out scenarios
    Pt, Qt, Gt = c5_scenarios(np, base, C5_TEST, shard_seed(BASE_SEED + 12, rank))
    gi = np.zeros(C5_TEST, np.int32)
    inputs = dict(Pload=Pt.ravel(), Qload=Qt.ravel(), Pg=Gt.ravel())
    ref = gb.Batch([grid], device=dev, precision=gb.PREC_FP64, **opts)
    ref.set_instances(gi, **inputs)
    ref.solve()
    r64 = ref.results()
    ms64 = ref.time(3) / 3
    w64 = ref.solve_warm(m)
    r64w = ref.results(state=False)
    fast = gb.Batch([grid], device=dev, precision=gb.PREC_FP32_IR, **opts)
    fast.set_instances(gi, **inputs)
    fast.solve()
    r32 = fast.results(state=False)
    ms32 = fast.time(3) / 3
    # a second batch of the same scenarios, for two warm-started solves in
    # flight (the timed steps and the end-to-end steps)
    twin = gb.Batch([grid], device=dev, precision=gb.PREC_FP32_IR, **opts)
    twin.set_instances(gi, **inputs)
    for _ in range(max(3, a.warmup)):
        w = fast.solve_warm(m)
    gb.time_warm_pipelined([fast, twin], m, max(3, a.warmup))
    # one solve at a time: the phases of a step and the serial rate
    t_serial = 0.0
    phases = dict(network=0.0, start_choice=0.0, newton=0.0)
    for _ in range(a.steps):
        w = fast.solve_warm(m)
        t_serial += w["ms"]
        for k in phases:
            phases[k] += w["phases_ms"][k] / a.steps
    if dist:
        dist.barrier()
    with Clocks(dev) as clk:
        t_steps = gb.time_warm_pipelined([fast, twin], m, a.steps)
    if dist:
        dist.barrier()
    w = fast.solve_warm(m)
    rw = fast.results()
    kind = w["start_kind"]
    conv = int((rw["status"] == 0).sum())
    t_dev = max_over_ranks(t_steps / 1e3, dist, dev)
    value = sum_over_ranks(conv, dist, dev) * a.steps / t_dev
    both = (r64["status"] == 0) & (rw["status"] == 0)
    sel = np.repeat(both, nB)
    err_v = float(np.max(np.abs(rw["V"][sel] - r64["V"][sel]))) if both.any() else None
    err_t = float(np.max(np.abs(rw["theta"][sel] - r64["theta"][sel]))) if both.any() else None
    assert np.all(rw["final_mismatch"][rw["status"] == 0] <= 1e-8)
    it_w = rw["iterations"] + np.where(kind == 2, w["warm_iterations"], 0)
    # end to end through the public API with host buffers, double-buffered
    # as in c2: step k's inputs go up and its warm-started solve is launched
    # before step k-1's results are read back (two batches, one network)
    pair = [fast, twin]
    hinputs = {k: pinned(v) for k, v in inputs.items()}
    outs = [pinned_results(C5_TEST, C5_TEST * nB) for _ in range(2)]

    def e2e_steps(k):
        for i in range(k):
            b = pair[i % 2]
            b.set_instances(gi, **hinputs)
            b.solve_warm_launch(m)
            if i >= 1:
                j = (i - 1) % 2
                pair[j].solve_warm_wait()
                outs[j] = pair[j].results(state=True, out=outs[j])
        j = (k - 1) % 2
        pair[j].solve_warm_wait()
        outs[j] = pair[j].results(state=True, out=outs[j])

    e2e_steps(max(3, a.warmup))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps(a.steps)
    t_e2e = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e = sum_over_ranks(conv, dist, dev) * a.steps / t_e2e
    res = outs[(a.steps - 1) % 2]
    assert np.array_equal(res["status"], rw["status"]) and np.array_equal(res["V"], rw["V"])
    twin.close()
    # the plain FP64 form: one held-out scenario per gbpf_solve
    n_plain, nconv = 64, 0
    t0 = time.perf_counter()
    for i in range(n_plain):
        plain.set_start(Pliq=Gt[i] - Pt[i], Qliq=base["Qg"] - Qt[i])
        nconv += plain.solve(full=False)["converged"]
    plain_rate = nconv / (time.perf_counter() - t0)
    peak, src = peak_hbm()
    nb_tot = C5_TEST * nB
    bytes_launch = nb_tot * 8 * 5 + nb_tot * 8 * 4 + C5_TEST * 20
    achieved = bytes_launch / (phases["newton"] / 1e3) / 1e9
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if src == "measured" else {}
    tpeak = peaks.get("bf16_tflops_sustained", 1700.0)
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": t_dev * 1e3 / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "c5", "grid": "1888-bus (16 tied 118-bus copies), limits off",
                   "instances_per_gpu": C5_TEST, "tolerance": 1e-8, "no_max_iter": 30,
                   "form": "batched, FP32 LU + FP64 mismatch/test/update, learned warm start with flat-start "
                           "fallback (network inference, start choice and Newton inside the timed region)",
                   "network": f"{3 * nB} -> 3 x {width} GELU -> {2 * nB} + linear skip, bf16 weights, fp32 "
                              f"accumulation; loss |e A|^2 + {lam} |e|^2 (A = S J0^T); Adam lr {lr0:g} cosine to "
                              f"1e-5, {epochs} epochs, batch {batch}",
                   "train_solves": C5_TRAIN, "train_converged": int(ok.sum()),
                   "train_generation_s": t_gen, "train_s": train_ms / 1e3,
                   "train_loss_first_last": [float(loss[0]), float(loss[-1])],
                   "converged_per_step": conv,
                   "in_flight": "2 batches of the same scenarios, one stream each, steps alternating; each step a "
                                "full warm-started solve of every scenario",
                   "serial_solves_per_s": sum_over_ranks(conv, dist, dev) * a.steps
                                          / max_over_ranks(t_serial / 1e3, dist, dev),
                   "phases_ms": {k: round(v, 4) for k, v in phases.items()},
                   "plan": fast.plan(),
                   "mean_iterations_flat_fp32": float(r32["iterations"].mean()),
                   "mean_iterations_warm_fp32": float(it_w.mean()),
                   "mean_iterations_flat_fp64": float(r64["iterations"].mean()),
                   "mean_iterations_warm_fp64": float((r64w["iterations"] + np.where(
                       w64["start_kind"] == 2, w64["warm_iterations"], 0)).mean()),
                   "start_kind_counts": {"flat_chosen": int((kind == 0).sum()), "predicted": int((kind == 1).sum()),
                                         "fallback": int((kind == 2).sum())},
                   "fallback_rate": float((kind == 2).mean()),
                   "max_abs_err_vs_fp64": {"V": err_v, "theta": err_t},
                   "plain_fp64_solves_per_s": plain_rate,
                   "batched_fp64_flat_solves_per_s": int((r64["status"] == 0).sum()) / (ms64 / 1e3),
                   "batched_fp32_flat_solves_per_s": int((r32["status"] == 0).sum()) / (ms32 / 1e3),
                   "speedup_vs_plain_fp64": value / plain_rate if plain_rate else None,
                   "l2": f"per-step inputs {nb_tot * 8 * 9 / 2**20:.0f} MiB > L2",
                   "parallelism": f"scenarios sharded x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nb_tot * 8 * 3,
                "d2h_bytes_per_step": nb_tot * 8 * 4 + C5_TEST * 20},
        "roofline": {"bound": "hbm", "kernel": f"k_nr_block<float, {fast.plan()['block_state_global']}> (one "
                                               "persistent launch per step; achieved over its phase of the step)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_source": peak_src_note(src),
                     # ncu dram__bytes_read.sum + dram__bytes_write.sum of the
                     # level-3 launch on 2,048 flat-start scenarios (4.89 GB),
                     # scaled by scenarios and by iterations a scenario
                     "traffic": 4.889e9 * C5_TEST / 2048 * float(it_w.mean()) / 4.86 / 1e9,
                     "traffic_unit": "GB per launch (scaled from a 2,048-scenario capture)",
                     "note": "dependent-load latency bound: ~200 MB of per-block factors and state exceed the L2, "
                             "so lines go to DRAM and back at ~5 % of its bandwidth; the misses' latency is the "
                             "main stall"},
        "roofline_training": {"bound": "tensor", "kernel": "k_gemm (tcgen05 bf16, all training GEMMs)",
                              "achieved": train_tflops, "peak": tpeak, "unit": "TFLOP/s",
                              "frac": train_tflops / tpeak,
                              "peak_source": "MEASURED_PEAKS.json bf16_tflops_sustained" if peaks else "fallback"},
        "clocks": clk.summary(),
        # features, 4 network layers, start choice, queue order, Newton (restarts included)
        "gpu_launches": a.steps * (1 + 4 + 1 + 1 + 1),
    }
    if rank == 0 and not a.no_cpu_baseline:
        cdf = write_grid(grid)
        line["cpu_baseline"] = cpu_baseline_c5(cdf, Pt, Qt, Gt)
    return line


def cpu_baseline_c5(cdf, Pt, Qt, Gt, target_s=12.0):
    """The oracle (flat start) on one host core over a bounded sample of the
    held-out scenarios."""
    oracle = _oracle()
    og = oracle.Grid(cdf)
    conv, n = 0, 0
    t0 = time.perf_counter()
    while n < len(Pt) and time.perf_counter() - t0 < target_s:
        og.set_bus(Pload=Pt[n], Qload=Qt[n], Pg=Gt[n])
        conv += og.solve(1e-8, 30, False)["converged"]
        n += 1
    dt = time.perf_counter() - t0
    return {"value": conv / dt, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"first {n} of the {len(Pt)} held-out scenarios, {conv} converged, {dt:.1f} s single-threaded "
                      f"oracle (oracle/pf_oracle.c via ctypes), flat start"}


def peak_src_note(src):
    return f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else "fallback 6.8 TB/s"


def bench_single(a, gb, np, rank, dev, world, dist):
    dense = a.workload.endswith("-dense")
    lim = 1
    if a.workload == "c3":
        g, desc = gb.generate(3, BASE_SEED + 3, tiles=128), "15104-bus (128 tied 118-bus copies), limits on"
    elif a.workload == "c5-dense":
        g, desc, lim = gb.generate(3, BASE_SEED + 5, tiles=16), "1888-bus (16 tied 118-bus copies), limits off", 0
    else:
        g, desc = gb.generate(2, BASE_SEED + 2), "118-bus meshed (1 slack/53 PV/64 PQ, 186 branches), limits on"
    cdf = write_grid(g)
    grid = gb.read_grid(cdf)
    s = gb.Solver(grid, device=dev, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=1 if dense else 0)
    first = s.solve(full=False)
    assert first["converged"] and first["final_mismatch"] <= 1e-8, first
    info = s.info()
    b = grid.buses()
    V0, th0, Pliq, Qliq = b["V0"], b["theta0"], b["Pg"] - b["Pload"], b["Qg"] - b["Qload"]
    s.time(max(3, a.warmup))
    if dist:
        dist.barrier()
    with Clocks(dev) as clk:
        ms = s.time(a.steps)
    t_dev = max_over_ranks(ms / 1e3, dist, dev)
    value = world * a.steps / t_dev
    for _ in range(max(3, a.warmup)):
        s.set_start(V0, th0, Pliq, Qliq)
        s.solve(full=False)
        s.state()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        s.set_start(V0, th0, Pliq, Qliq)
        r = s.solve(full=False)
        s.state()
    t_e2e = max_over_ranks(time.perf_counter() - t0, dist, dev)
    # config 3 also runs the FP32-LU form of the same solver (FP32 factor and
    # substitutions, FP64 fill, mismatch, test and update): solves/s and its
    # |V|, theta error against the FP64 solution
    fp32 = None
    if a.workload == "c3":
        s32 = gb.Solver(grid, device=dev, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=0,
                        precision=gb.PREC_FP32_IR)
        r32 = s32.solve()
        r64 = s.solve()
        s32.time(max(3, a.warmup))
        ms32 = s32.time(a.steps)
        fp32 = {"solves_per_s": a.steps / (ms32 / 1e3), "ms_per_solve": ms32 / a.steps,
                "iterations": r32["iterations"], "final_mismatch": r32["final_mismatch"],
                "max_abs_err_V": float(np.max(np.abs(r32["V"] - r64["V"]))),
                "max_abs_err_theta": float(np.max(np.abs(r32["theta"] - r64["theta"]))),
                "same_switch_events": [e[1:] for e in r32["events"]] == [e[1:] for e in r64["events"]],
                "phases": s32.profile(5)}
    peak, src = peak_hbm()
    if dense:
        # metodo = denso: per Newton iteration the N x N FP64 matrix is written
        # by the fill and read and written once by the LU's panel sweep (lower
        # bound on its traffic); the LU does 2/3 N^3 + 2 N^2 flops
        N = 2 * (grid.nB - 1)
        it = max(1, first["iterations"])
        t_it = t_dev / a.steps / it
        achieved = 3 * N * N * 8 / t_it / 1e9
        top, prof = "dense fill + LU + solves", {"matrix_order": N, "iterations": first["iterations"],
                                                 "ms_per_iteration": 1e3 * t_it,
                                                 "lu_fp64_gflops": (2 / 3 * N ** 3 + 2 * N * N) / t_it / 1e9,
                                                 "phases": s.profile(5)}
    else:
        prof = s.profile(10)
        top = max(prof, key=lambda k: prof[k]["ms"])
        achieved = prof[top]["bytes"] / (prof[top]["ms"] * 1e-3) / 1e9
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "grid": desc, "nB": grid.nB, "tolerance": 1e-8, "lim_inj_reat": lim,
                   "form": ("metodo = denso: dense FP64 Jacobian and LU with partial pivoting, one solve per step"
                            if dense else "plain FP64, one solve per step"), "iterations": first["iterations"],
                   "solver": info, "parallelism": f"replicas x{world}", "fp32_lu": fp32,
                   "l2": "working set fits in L2; no flush"},
        "e2e": {"value": world * a.steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * grid.nB * 8,
                "d2h_bytes_per_step": 4 * grid.nB * 8 + 32},
        "roofline": {"bound": "hbm", "kernel_phase": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src_note(src), "traffic": None, "phases": prof},
        "clocks": clk.summary(),
        "gpu_launches": a.steps * (6 + max(1, first["iterations"]) * info["kernels_per_iteration"] + 1),
    }
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_repeat(cdf, lim)
    return line


def main():
    a = args()
    if a.impl == "reference":
        run_reference(a)
        return
    rank, local_rank, world = dist_env()
    import numpy as np

    dist = None
    if world > 1:
        import torch
        import torch.distributed as dist

        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    gb = importlib.import_module(PKG)
    if a.workload in ("c2", "c4"):
        line = bench_batch(a, gb, np, rank, local_rank, world, dist)
    elif a.workload == "c5":
        line = bench_c5(a, gb, np, rank, local_rank, world, dist)
    else:
        line = bench_single(a, gb, np, rank, local_rank, world, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
