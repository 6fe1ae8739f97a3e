#!/usr/bin/env python3
"""Benchmark: converged Newton-Raphson power-flow solves per second on one GB300.

Workloads (seeded synthetic grids of the named shapes, generated in process):
  c2   118-bus meshed grid (1 slack, 53 PV, 64 PQ, 186 branches), reactive
       limits on, tolerance 1e-8 p.u., plain FP64 -- the default
  c1   14-bus ring-plus-chords grid, limits off
  c3   15,104-bus grid (128 tied copies of the 118-bus grid), limits on
A step is one solve of the grid from its flat start.  `value` is solves/s with
the inputs resident in device memory (one CUDA-graph launch per solve, CUDA
events on the solver stream); `e2e` is the same through the public API with
host buffers: host->device copy of the start state and injections, the solve,
device->host copy of |V| and theta, every step.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c2]
  python bench.py --impl reference ...   (the CPU restatement of the reference
                                          path on all host cores)
Multi-GPU: one process per GPU under torch.distributed.run; a single grid does
not shard (the LU has one elimination order), so every rank solves its own
replica and `value` is the sum over ranks ("replicas only").
"""
import argparse
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
PKG = "experience-of-using-gpu-in-power-flow-computation_gb300"
BASE_SEED = 20261203
METRIC = "converged PF solves/s on 1 GB300 @ mismatch<=1e-8 pu"
UNIT = "solves/s"


def args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=200)
    p.add_argument("--warmup", type=int, default=5)
    p.add_argument("--impl", default="gbpf", choices=["gbpf", "reference"])
    p.add_argument("--workload", default="c2", choices=["c1", "c2", "c3"])
    p.add_argument("--no-cpu-baseline", action="store_true")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


def workload(gb, name):
    """(grid, cdf path, limits flag, description)"""
    if name == "c1":
        g, lim, desc = gb.generate(1, BASE_SEED + 1), 0, "14-bus ring+chords, limits off"
    elif name == "c3":
        g, lim, desc = gb.generate(3, BASE_SEED + 3, tiles=128), 1, "15104-bus (128 tied 118-bus copies), limits on"
    else:
        g, lim, desc = gb.generate(2, BASE_SEED + 2), 1, "118-bus meshed (1 slack/53 PV/64 PQ, 186 branches), limits on"
    d = tempfile.mkdtemp(prefix="gbpf_bench_")
    path = os.path.join(d, "grid.cdfx" if g.nB > 9999 else "grid.cdf")
    g.write_cdf(path)
    return gb.read_grid(path), path, lim, desc


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.out = None

    def __enter__(self):
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.out = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.out, stderr=subprocess.DEVNULL)
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
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": int(rows[0][2]), "reasons": sorted(reasons),
                "samples": len(rows)}


def cpu_baseline(cdf, lim, target_s=12.0):
    """The oracle (CPU restatement of the reference path, single thread) on a
    bounded sample of the same workload: repeated solves of the same grid."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if not os.path.exists(oracle.CLI_PATH):
        oracle.build()
    probe = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", "3"],
                                      capture_output=True, text=True, check=True).stdout)
    reps = max(3, int(target_s / max(probe["solve_s"], 1e-6)))
    r = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", str(reps)],
                                  capture_output=True, text=True, check=True).stdout)
    return {"value": 1.0 / r["solve_s"], "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"{reps} repeated solves of the same grid ({r['iterations']} iterations each), "
                      f"{reps * r['solve_s']:.1f} s single-threaded oracle/pforacle"}


def run_reference(a):
    """--impl reference: the reference path restated in C (oracle/) on every
    host core (one single-threaded process per core), same grid and metric.
    The reference's own executables need MKL or a CUDA 10-era library set, so
    the restatement stands in for them."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle

    if not os.path.exists(oracle.CLI_PATH):
        oracle.build()
    gb = importlib.import_module(PKG)
    grid, cdf, lim, desc = workload(gb, a.workload)
    cores = os.cpu_count() or 1
    probe = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", "2"],
                                      capture_output=True, text=True, check=True).stdout)
    reps = max(1, int(1.0 / max(probe["solve_s"], 1e-6)))  # about one second per process per step

    def step():
        t0 = time.perf_counter()
        ps = [subprocess.Popen([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", str(reps)],
                               stdout=subprocess.PIPE, text=True) for _ in range(cores)]
        for p in ps:
            p.communicate()
        return time.perf_counter() - t0

    for _ in range(min(a.warmup, 3)):
        step()
    steps = min(a.steps, 10)
    total = sum(step() for _ in range(steps))
    value = steps * cores * reps / total
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": steps,
            "warmup": min(a.warmup, 3), "ms_per_step": 1e3 * total / steps, "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "impl": "reference",
            "config": {"workload": a.workload, "grid": desc, "nB": grid.nB, "tolerance": 1e-8,
                       "lim_inj_reat": lim},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                             "sample": f"each step: {cores} processes x {reps} solves of the grid"},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


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
    grid, cdf, lim, desc = workload(gb, a.workload)
    s = gb.Solver(grid, device=local_rank, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=0)
    first = s.solve(full=False)
    assert first["converged"] and first["final_mismatch"] <= 1e-8, first
    info = s.info()
    buses = grid.buses()
    V0, th0 = buses["V0"], buses["theta0"]
    Pliq, Qliq = buses["Pg"] - buses["Pload"], buses["Qg"] - buses["Qload"]

    def barrier():
        if dist:
            dist.barrier()

    # device-resident: one graph launch per solve, CUDA events on the solver stream
    s.time(max(3, a.warmup))
    barrier()
    with Clocks(local_rank) as clk:
        ms = s.time(a.steps)
    barrier()
    t_dev = ms / 1e3
    if dist:
        import torch

        t = torch.tensor([t_dev], dtype=torch.float64, device=f"cuda:{local_rank}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        t_dev = float(t.item())
    value = world * a.steps / t_dev

    # end to end through the public API with host buffers
    for _ in range(max(3, a.warmup)):
        s.set_start(V0, th0, Pliq, Qliq)
        s.solve(full=False)
        s.state()
    barrier()
    t0 = time.perf_counter()
    for _ in range(a.steps):
        s.set_start(V0, th0, Pliq, Qliq)
        r = s.solve(full=False)
        st = s.state()
    t_e2e = time.perf_counter() - t0
    assert r["converged"]
    e2e = world * a.steps / t_e2e

    prof = s.profile(20)
    top = max(prof, key=lambda k: prof[k]["ms"])
    peaks_path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(peaks_path):
        peak, peak_src = json.load(open(peaks_path))["hbm_gbs"], "measured"
    else:
        peak, peak_src = 6800.0, "fallback"
    achieved = prof[top]["bytes"] / (prof[top]["ms"] * 1e-3) / 1e9
    # prologue (reset, phasors, injections, [limits], mismatch, test) + one body
    # pass per Newton update + branch flows
    launches_per_solve = 5 + (1 if lim else 0) + max(1, first["iterations"]) * info["kernels_per_iteration"] + 1
    if rank != 0:
        return
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "grid": desc, "nB": grid.nB, "nL": grid.nL, "tolerance": 1e-8,
                   "lim_inj_reat": lim, "form": "plain FP64 sparse, one solve per step",
                   "iterations": first["iterations"], "switch_events": first["n_events"],
                   "l2": "working set of a solve fits in L2; no flush between steps",
                   "solver": info, "parallelism": f"replicas x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * grid.nB * 8,
                "d2h_bytes_per_step": 4 * grid.nB * 8 + 32},
        "roofline": {"bound": "hbm", "kernel_phase": top, "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "peak_source": peak_src, "traffic": None,
                     "phases": prof},
        "clocks": clk.summary(),
        "gpu_launches": launches_per_solve * a.steps,
    }
    if not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(cdf, lim)
    print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
