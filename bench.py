#!/usr/bin/env python3
"""Benchmark: converged Newton-Raphson power-flow solves per second on one GB300.

Default workload c5 -- the headline, "plain FP64 vs batched + learned": the
seeded 1,888-bus grid (16 tied copies of the 118-bus config-2 generator,
tests/golden/c5_base.cdf.gz), reactive limits off, flat start, tolerance 1e-8
p.u.  Set-up, outside the timed region: 50,000 training scenarios (per-bus load
x U(0.7, 1.3), generator P x U(0.85, 1.15)) solved by the batched FP64 Newton
method, and the 3776 -> 3 x 512 -> 3776 network trained on them on the GPU
(tcgen05 GEMMs, 120 epochs).  A step is one warm-started solve of the 8,192
held-out scenarios: network inference, start choice, batched Newton with the
LU in FP32 and mismatch/test/update in FP64, flat-start fallback; two steps in
flight.
  value    converged solves/s, counting only the scenarios whose answer the
           batched FP64 solve of the same scenario confirms (same switch path,
           |V| and theta within 1e-6: config.fp64_check); inputs resident in
           device memory, CUDA events on the batch streams
  e2e      the same through the public API with host arrays: every step the
           host->device copy of every scenario's loads and generation, the
           solve, the device->host copy of |V|, theta, P, Q and the
           per-instance results
  config   the plain FP64 form on the same scenarios (gbpf_solve, one scenario
           per call: the oracle-matching path), batched FP64 and batched FP32
           from the flat start, iterations saved, fallback rate
  roofline the Newton kernel against HBM with the per-iteration algorithmic
           bytes of the path (36 nnzY + 12 nnzJ + 24|36 nnzLU + 112 nB + 32
           dimJ per instance and iteration, FP32|FP64 LU values) and against
           the L2 copy bandwidth measured in the same run
Other workloads: c2 (the 118-bus config-2 grid, limits on, 32,768 load
scenarios per step, batched FP32 LU from the flat start, four batches in
flight), c2-plain (one FP64 solve of the 118-bus grid per step), c2-dense
(metodo = denso), c3 (the 15,104-bus grid, one FP64 solve per step, and its
FP32-LU form), c4 (4,096 instances of 14..472-bus grids), c5-dense.  A
default (c5) run on one GPU also benches c2, c4 and c3 after the headline and
reports them under "secondary_workloads" (--no-secondary skips them).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--workload c5]
  python bench.py --impl reference     the reference path restated in C
                                       (oracle/) on every host core, same
                                       grids, scenarios, steps and warm-up
Every grid is read from a committed file (tests/golden/, written by
make_golden.py / make_bench_grids.py), so both arms solve byte-identical inputs.
Multi-GPU (torch.distributed.run, one process per GPU): scenarios are sharded
over ranks (weak scaling: every rank solves its own draw), no collective in the
data path; a single grid does not shard, so c2-plain/c3 run replicas.
"""
import argparse
import gzip
import importlib
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)
PKG = "experience-of-using-gpu-in-power-flow-computation_gb300"
BASE_SEED = 20261203
METRIC = "converged PF solves/s on 1 GB300 @ mismatch<=1e-8 pu"
UNIT = "solves/s"
N_SCEN = 4096           # c4 instances
N_SCEN_C2 = 32768       # c2 scenarios per step
C5_TRAIN, C5_TEST = 50000, 8192
C4_SIZES = (14, 30, 57, 118, 236, 472)
IN_FLIGHT = 4           # c2/c4: batches of the same scenarios in flight, one stream each
L2_BYTES = 129 * 1024 * 1024
ACC_TOL = 1e-6          # FP32-LU answers: |V|, theta within this of the FP64 solve
WORKLOADS = ["c5", "c2", "c2-plain", "c2-dense", "c3", "c4", "c5-dense"]

# DRAM and L2 (lts__t_bytes) bytes per instance-iteration of the batch Newton
# kernels, from one small-case ncu capture each (one kernel, one launch; the
# command and the raw figures are in the named profiles/ summary).  A bench
# line scales them by the instance-iterations of its own launch.
TRAFFIC = {
    # (workload, kernel family): (dram bytes, lts bytes, per instance-iteration; summary)
    ("c5", "k_nr_block<float"): (1.976263e9 / 4207, 11.962471e9 / 4207,
                                 "profiles/k_nr_block_fp32_level3_c5_1024_bytes.md (level 3, 1,024 scenarios, "
                                 "flat start)"),
    ("c2", "k_nr_warp<float"): (93.784e6 / 65671, 2.964886e9 / 65671,
                                "profiles/k_nr_warp_fp32_level2_c2_16384_bytes.md (level 2, 16,384 scenarios)"),
}


def args():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=20)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gbpf", choices=["gbpf", "reference"])
    p.add_argument("--workload", default="c5", choices=WORKLOADS)
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--scenarios", type=int, default=0,
                   help="scenarios per step (c2: default 32768, c4: 4096; c5: held-out, default 8192); smaller cases "
                        "for profiler captures")
    p.add_argument("--train", type=int, default=0, help="c5 training solves (default 50000)")
    p.add_argument("--no-secondary", action="store_true",
                   help="workload c5: skip the c2, c4 and c3 summaries that follow the headline")
    p.add_argument("--no-autotune", action="store_true",
                   help="batched workloads: keep the default launch plan instead of the autotuner's")
    return p.parse_args()


def dist_env():
    return int(os.environ.get("RANK", 0)), int(os.environ.get("LOCAL_RANK", 0)), int(os.environ.get("WORLD_SIZE", 1))


_UNPACKED = {}


def grid_file(name):
    """Path of a committed grid file (a .gz fixture is unpacked once)."""
    if name in _UNPACKED:
        return _UNPACKED[name]
    src = os.path.join(GOLDEN, name)
    if name.endswith(".gz"):
        d = tempfile.mkdtemp(prefix="gbpf_bench_")
        path = os.path.join(d, name[:-3])
        with gzip.open(src, "rb") as f, open(path, "wb") as o:
            o.write(f.read())
    else:
        path = src
    _UNPACKED[name] = path
    return path


def workload_files(workload):
    """Committed input file(s) of a workload."""
    if workload in ("c2", "c2-plain", "c2-dense"):
        return ["c2_base.cdf"]
    if workload == "c3":
        return ["c3_base.cdfx.gz"]
    if workload == "c4":
        return [f"c4_{nb}.cdf.gz" for nb in C4_SIZES]
    return ["c5_base.cdf.gz"]


# ------------------------------------------------------------ scenario draws
def scenarios(np, base, n, seed):
    """c2: per-bus load x lognormal(sigma 0.1), generation x U(0.9, 1.1)."""
    rng = np.random.default_rng(seed)
    nb = len(base["Pload"])
    lf = np.exp(rng.normal(-0.005, 0.1, (n, nb)))
    gf = rng.uniform(0.9, 1.1, (n, nb))
    return base["Pload"] * lf, base["Qload"] * lf, base["Pg"] * gf


def c4_instances(np, bases, n, seed):
    """c4: grid of each instance drawn uniformly from the six sizes; per-bus
    load x lognormal(sigma 0.1), generation x U(0.9, 1.1).  Returns the grid
    index per instance and the packed Pload, Qload, Pg."""
    rng = np.random.default_rng(seed)
    gi = rng.integers(0, len(bases), n).astype(np.int32)
    cols = {k: [] for k in ("Pload", "Qload", "Pg")}
    for t in gi:
        b = bases[t]
        nb = len(b["Pload"])
        lf = np.exp(rng.normal(-0.005, 0.1, nb))
        cols["Pload"].append(b["Pload"] * lf)
        cols["Qload"].append(b["Qload"] * lf)
        cols["Pg"].append(b["Pg"] * rng.uniform(0.9, 1.1, nb))
    return gi, tuple(np.concatenate(cols[k]) for k in ("Pload", "Qload", "Pg"))


def c5_scenarios(np, base, n, seed):
    """c5: per-bus load x U(0.7, 1.3) (P and Q together), generator P x U(0.85, 1.15)."""
    rng = np.random.default_rng(seed)
    nb = len(base["Pload"])
    lf = rng.uniform(0.7, 1.3, (n, nb))
    gf = rng.uniform(0.85, 1.15, (n, nb))
    return base["Pload"] * lf, base["Qload"] * lf, base["Pg"] * gf


def draw_seed(workload, rank):
    return shard_seed(BASE_SEED + {"c2": 7, "c4": 4, "c5": 12}[workload], rank)


# ---------------------------------------------------------- timing helpers
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


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return dict(hbm=d["hbm_gbs"], bf16=d.get("bf16_tflops_sustained", 1700.0), src="measured")
    return dict(hbm=6800.0, bf16=1700.0, src="fallback")


def peak_src_note(src):
    return f"{src} (MEASURED_PEAKS.json hbm_gbs)" if src == "measured" else "fallback 6.8 TB/s"


def l2_copy_gbs(dev):
    """L2 bandwidth of this GPU, measured here: device copies of 16, 24 and 32
    MiB (working sets of 32-64 MiB stay in the 129 MB L2; smaller copies are
    bound by launch gaps), read + write bytes over CUDA-event time, best of 5
    runs of 50 copies, the fastest size."""
    import torch

    best_gbs = 0.0
    for mib in (16, 24, 32):
        n = mib * 2 ** 20 // 4
        a = torch.ones(n, dtype=torch.float32, device=f"cuda:{dev}")
        b = torch.empty_like(a)
        for _ in range(20):
            b.copy_(a)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        best = float("inf")
        for _ in range(5):
            torch.cuda.synchronize(dev)
            s.record()
            for _ in range(50):
                b.copy_(a)
            e.record()
            e.synchronize()
            best = min(best, s.elapsed_time(e))
        best_gbs = max(best_gbs, 2 * n * 4 * 50 / (best / 1e3) / 1e9)
        del a, b
    return best_gbs


# ------------------------------------------------------ per-iteration bytes
def path_sizes(grid):
    """Sizes of the Newton path of a grid, by the reference's rules: nnzY =
    nB + 2 x (unique branches), dimJ = nB - 1 + nPQ, nnzJ = |H|+|N|+|M|+|L| over
    the Ybus pattern (GPU/esparso.h:481-654 with the initial PQ set), and nnzLU
    = scalar nonzeros of this solver's 2x2 block factor (diagonal blocks and
    both triangles' off-diagonal blocks)."""
    import numpy as np

    a = grid.analyse()
    t = grid.buses()["type"]
    br = grid.branches()
    f, to = br["from_bus"] - 1, br["to_bus"] - 1
    keep = f != to
    pairs = np.unique(np.stack([np.minimum(f, to)[keep], np.maximum(f, to)[keep]], 1), axis=0)
    i = np.concatenate([np.arange(grid.nB), pairs[:, 0], pairs[:, 1]])
    j = np.concatenate([np.arange(grid.nB), pairs[:, 1], pairs[:, 0]])
    ns = (t != 3).astype(np.int64)
    pq = ((t == 0) | (t == 1)).astype(np.int64)
    nnzJ = int(np.sum(ns[i] * ns[j] + ns[i] * pq[j] + pq[i] * ns[j] + pq[i] * pq[j]))
    return dict(nB=grid.nB, nnzY=int(len(i)), nnzJ=nnzJ, dimJ=grid.nB - 1 + int(pq.sum()),
                nnzLU=4 * (a["blocks"] + 2 * a["factor_blocks"]), lu_levels=a["forward_levels"])


def bytes_per_iteration(sz, lu_value_bytes):
    """Algorithmic bytes of one Newton iteration of one instance, each array
    counted once: injections 20 nnzY + 4(nB+1) + 32 nB; mismatch and max
    32 nB + 8 dimJ; Jacobian fill 12 nnzJ + 16 nnzY + 32 nB; numeric LU
    2 (v + 4) nnzLU; both substitutions (v + 4) nnzLU + 16 dimJ; update
    8 dimJ + 16 nB (v = bytes of an LU value: 8 FP64, 4 FP32)."""
    return (36 * sz["nnzY"] + 12 * sz["nnzJ"] + 3 * (lu_value_bytes + 4) * sz["nnzLU"] + 112 * sz["nB"]
            + 32 * sz["dimJ"] + 4)


def chord_bytes_saved(sz, lu_value_bytes):
    """Algorithmic bytes one chord iteration (iteration 0 of a predicted run:
    the shared factor of the Jacobian at the network's mean output) does not
    move: the Jacobian fill and the numeric LU of bytes_per_iteration."""
    return 12 * sz["nnzJ"] + 16 * sz["nnzY"] + 32 * sz["nB"] + 2 * (lu_value_bytes + 4) * sz["nnzLU"]


def roofline(kernel, alg_bytes, kernel_s, inst_iters, pk, l2_gbs, note, workload=None):
    """The roofline object of a bench line: algorithmic bytes of one launch of
    the dominant kernel over its CUDA-event time, against the measured HBM
    peak and the L2 copy bandwidth measured in this run; DRAM and L2 traffic
    scaled from the kernel's small-case ncu capture where one exists."""
    achieved = alg_bytes / kernel_s / 1e9
    tr = next((v for (w, k), v in TRAFFIC.items() if w == workload and kernel.startswith(k)), None)
    out = {"bound": "hbm", "kernel": kernel, "achieved": achieved, "peak": pk["hbm"], "unit": "GB/s",
           "frac": achieved / pk["hbm"], "peak_source": peak_src_note(pk["src"]),
           "traffic": tr[0] * inst_iters / 1e9 if tr else None, "traffic_unit": "GB per launch",
           "algorithmic_bytes_per_launch": alg_bytes, "instance_iterations_per_launch": int(inst_iters),
           "kernel_ms_per_launch": kernel_s * 1e3,
           "l2": {"peak_gbs": l2_gbs, "peak_source": "16-32 MiB device copies measured in this run (fastest)",
                  "l2_frac": achieved / l2_gbs if l2_gbs else None,
                  "lts_bytes_per_launch": tr[1] * inst_iters if tr else None,
                  "lts_frac": (tr[1] * inst_iters / kernel_s / 1e9 / l2_gbs) if tr and l2_gbs else None,
                  "profile": tr[2] if tr else None},
           "note": note}
    return out


# ------------------------------------------------------ FP32 against FP64
def fp64_check(np, b32, r32, b64, r64, offsets):
    """Every FP32-LU answer against the batched FP64 solve of the same
    scenario.  A scenario counts as converged when both converge, their switch
    paths (the ordered bus / PV position / code of every PV<->PQ switch,
    GPU/limiteInjReat.cuh:5-40) are the same, and |V|, theta agree within
    ACC_TOL.  Returns that mask and the line's fp64_check record."""
    ok32, ok64 = r32["status"] == 0, r64["status"] == 0
    starts = offsets[:-1].astype(np.int64)
    eV = np.maximum.reduceat(np.abs(r32["V"] - r64["V"]), starts)
    eT = np.maximum.reduceat(np.abs(r32["theta"] - r64["theta"]), starts)
    e32, n32 = b32.events_all()
    e64, n64 = b64.events_all()
    path = (n32 == n64) & np.all(e32[:, :, 1:] == e64[:, :, 1:], axis=(1, 2))
    when = path & np.all(e32[:, :, 0] == e64[:, :, 0], axis=1)
    both = ok32 & ok64
    same = both & path
    within = same & (eV <= ACC_TOL) & (eT <= ACC_TOL)
    mx = lambda e, m: float(np.max(e[m])) if m.any() else None
    rec = {"compared": int(len(ok32)), "tolerance": ACC_TOL,
           "fp64_converged": int(ok64.sum()), "fp32_converged": int(ok32.sum()),
           "both_converged": int(both.sum()),
           "diverged_switch_path": int((both & ~path).sum()),
           "switch_iteration_differs": int((same & ~when).sum()),
           "beyond_tolerance": int((same & ~((eV <= ACC_TOL) & (eT <= ACC_TOL))).sum()),
           "fp32_only_converged": int((ok32 & ~ok64).sum()),
           "counted": int(within.sum()),
           "max_abs_err_vs_fp64": {"V": mx(eV, within), "theta": mx(eT, within)},
           "max_abs_err_beyond_tolerance": {"V": mx(eV, same & ~within), "theta": mx(eT, same & ~within)},
           "max_abs_err_vs_fp64_diverged_paths": {"V": mx(eV, both & ~path), "theta": mx(eT, both & ~path)}}
    return within, rec


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


# --------------------------------------------------------- reference arm
_REF = {}


def _ref_init(files, inst_grid, Pl, Ql, Pg, offsets, lim, maxit):
    """Pool worker set-up: the oracle's grids and the step's scenarios."""
    oracle = _oracle()
    _REF.update(grids=[oracle.Grid(f) for f in files], inst_grid=inst_grid, Pl=Pl, Ql=Ql, Pg=Pg,
                offsets=offsets, lim=lim, maxit=maxit)


def _ref_solve(span):
    """Pool worker: solve instances [lo, hi) of the sample; converged count."""
    lo, hi = span
    R = _REF
    conv = 0
    for i in range(lo, hi):
        og = R["grids"][R["inst_grid"][i]]
        a, b = R["offsets"][i], R["offsets"][i + 1]
        og.set_bus(Pload=R["Pl"][a:b], Qload=R["Ql"][a:b], Pg=R["Pg"][a:b])
        conv += og.solve(1e-8, R["maxit"], bool(R["lim"]))["converged"]
    return conv


def reference_sample(np, workload, files, rank):
    """The scenarios of a batched workload exactly as the GPU arm draws them
    (the oracle's reader gives the same bus arrays as the product's): grid
    index per instance, packed Pload, Qload, Pg and per-instance offsets."""
    oracle = _oracle()
    ogs = [oracle.Grid(f) for f in files]
    bases = [dict(Pload=o.Pload.copy(), Qload=o.Qload.copy(), Pg=o.Pg.copy()) for o in ogs]
    if workload == "c4":
        gi, (Pl, Ql, Pg) = c4_instances(np, bases, N_SCEN, draw_seed("c4", rank))
    else:
        n = N_SCEN_C2 if workload == "c2" else C5_TEST
        draw = scenarios if workload == "c2" else c5_scenarios
        Pl, Ql, Pg = draw(np, bases[0], n, draw_seed(workload, rank))
        Pl, Ql, Pg = Pl.ravel(), Ql.ravel(), Pg.ravel()
        gi = np.zeros(n, np.int32)
    nbs = np.array([o.nB for o in ogs], np.int64)
    offsets = np.concatenate([[0], np.cumsum(nbs[gi])])
    return gi, Pl, Ql, Pg, offsets


def run_reference(a):
    """--impl reference: the reference path restated in C (oracle/, which the
    tests pin to the reference's own CPU-tree code) on every host core, on the
    same committed grids, the same scenario draws, tolerance, iteration limit
    and the same --steps/--warmup as the GPU arm; each step solves a bounded
    sample of the workload (the first S scenarios, S sized to about a second
    of work on all cores).  The reference's own executables cannot run on the
    Arm GPU host: its GPU tree needs MKL headers and cuSPARSE calls removed
    from CUDA 12+, its CPU tree's sparse solve is MKL PARDISO (no MKL build
    exists for Arm), and its sources are not on that host; so the
    restatement stands in for them (cpu_baseline.kind "port").  Never loads
    the product."""
    rank, _, world = dist_env()
    if rank != 0:
        return
    import multiprocessing as mp

    import numpy as np

    oracle = _oracle()
    files = [grid_file(f) for f in workload_files(a.workload)]
    cores = os.cpu_count() or 1
    warm = a.warmup
    batched = a.workload in ("c2", "c4", "c5")
    if batched:
        lim, maxit = (0, 30) if a.workload == "c5" else (1, 100)
        gi, Pl, Ql, Pg, offsets = reference_sample(np, a.workload, files, rank)
        # probe: one core, the first few instances
        _ref_init(files, gi, Pl, Ql, Pg, offsets, lim, maxit)
        _ref_solve((0, 2))
        t0 = time.perf_counter()
        _ref_solve((0, 6))
        per = (time.perf_counter() - t0) / 6
        S = int(min(len(gi), max(cores, cores * int(max(1, 1.0 / per)))))
        b = offsets[S]
        spans = [(k * S // cores, (k + 1) * S // cores) for k in range(cores)]
        spans = [s for s in spans if s[0] < s[1]]
        ctx = mp.get_context("spawn")
        with ctx.Pool(len(spans), initializer=_ref_init,
                      initargs=(files, gi[:S], Pl[:b], Ql[:b], Pg[:b], offsets[:S + 1], lim, maxit)) as pool:
            for _ in range(warm):
                pool.map(_ref_solve, spans)
            t0 = time.perf_counter()
            conv = 0
            for _ in range(a.steps):
                conv += sum(pool.map(_ref_solve, spans))
            dt = time.perf_counter() - t0
        value = conv / dt
        sample = (f"each step: the first {S} of the {len(gi)} scenarios of the workload's draw over {len(spans)} "
                  f"processes (one per core), flat start, {conv // max(a.steps, 1)} converged per step")
        cfg = {"instances_per_step": S, "instances_of_workload": int(len(gi))}
    else:
        lim = 0 if a.workload == "c5-dense" else 1
        cdf = files[0]
        probe = json.loads(subprocess.run([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", "2"],
                                          capture_output=True, text=True, check=True).stdout)
        reps = max(1, int(1.0 / max(probe["solve_s"], 1e-6)))

        def step():
            ps = [subprocess.Popen([oracle.CLI_PATH, cdf, "--lim", str(lim), "--repeat", str(reps)],
                                   stdout=subprocess.PIPE, text=True) for _ in range(cores)]
            return sum(json.loads(p.communicate()[0])["converged"] for p in ps)

        for _ in range(warm):
            step()
        t0 = time.perf_counter()
        conv = 0
        for _ in range(a.steps):
            conv += step() * reps
        dt = time.perf_counter() - t0
        value = conv / dt
        sample = f"each step: {cores} processes x {reps} solves of the grid"
        cfg = {"solves_per_step": cores * reps}
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": a.gpus, "steps": a.steps, "warmup": warm,
            "ms_per_step": 1e3 * dt / a.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": {"workload": a.workload, "grids": workload_files(a.workload), "tolerance": 1e-8,
                       "lim_inj_reat": lim, "form": "plain FP64 Newton-Raphson, flat start (the reference "
                                                    "path restated in C, oracle/pf_oracle.c)", **cfg},
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


def plain_fp64_rate(gb, grid, dev, Pl, Ql, Pg, n, lim, maxit):
    """The plain FP64 form on the first n scenarios: one gbpf_solve per
    scenario (set the injections, solve, read the state back), wall time."""
    s = gb.Solver(grid, device=dev, tolerancia=1e-8, no_max_iter=maxit, lim_inj_reat=lim, metodo=0)
    base = grid.buses()
    for i in range(min(3, n)):
        s.set_start(Pliq=Pg[i] - Pl[i], Qliq=base["Qg"] - Ql[i])
        s.solve(full=False)
    nconv = 0
    t0 = time.perf_counter()
    for i in range(n):
        s.set_start(Pliq=Pg[i] - Pl[i], Qliq=base["Qg"] - Ql[i])
        nconv += s.solve(full=False)["converged"]
        s.state()
    dt = time.perf_counter() - t0
    info = s.info()
    info["form"] = "persistent" if s.form()["form"] == gb.FORM_PERSISTENT else "graph"
    s.close()
    return nconv / dt, info


PLAN_SET_KEYS = ("warp_mode", "warps_per_block", "handoff_it", "resume_group", "warp_group", "narrow", "lu1",
                 "warp_lu1", "flat_shared", "rotate", "gstate", "warp_gstate")


def bench_batch(a, gb, np, rank, dev, world, dist):
    n_scen = a.scenarios or (N_SCEN if a.workload == "c4" else N_SCEN_C2)
    files = [grid_file(f) for f in workload_files(a.workload)]
    grids = [gb.read_grid(f) for f in files]
    if a.workload == "c4":
        gi, (Pl, Ql, Pg) = c4_instances(np, [g.buses() for g in grids], n_scen, draw_seed("c4", rank))
        desc = (f"{n_scen} instances of 14/30/57/118/236/472-bus synthetic grids, load x lognormal(0.1), "
                "Pg x U(0.9,1.1)")
    else:
        Pl, Ql, Pg = scenarios(np, grids[0].buses(), n_scen, draw_seed("c2", rank))
        Pl, Ql, Pg = Pl.ravel(), Ql.ravel(), Pg.ravel()
        gi = np.zeros(n_scen, np.int32)
        desc = f"118-bus synthetic meshed grid (1 slack/53 PV/64 PQ, 186 branches), {n_scen} load scenarios"
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
    # more batches of the same scenarios and plan, IN_FLIGHT in all, each on
    # its own stream: one step's hand-off tail (the few scenarios that run all
    # no_max_iter iterations on a few SMs) runs beside the next steps' bulk
    pl = fast.plan()
    ring = [fast]
    for _ in range(IN_FLIGHT - 1):
        twin = gb.Batch(grids, device=dev, precision=gb.PREC_FP32_IR, **opts)
        twin.set_instances(gi, Pload=Pl, Qload=Ql, Pg=Pg)
        twin.set_plan(**{k: pl[k] for k in PLAN_SET_KEYS})
        twin.solve()
        ring.append(twin)
    # the autotuner times one batch at a time; in flight, where one step's
    # tail overlaps the next steps, the hand-off iteration is chosen again
    # with the ring itself (setup, outside the timed region)
    handoff_trials = {}
    if not a.no_autotune and len(ring) > 1 and pl["warp_instances"]:
        for ho in dict.fromkeys([pl["handoff_it"], 0, 24]):
            for b in ring:
                b.set_plan(**{**{k: pl[k] for k in PLAN_SET_KEYS}, "handoff_it": ho})
                b.solve()
            gb.time_pipelined(ring, 2 * len(ring))
            handoff_trials[ho] = gb.time_pipelined(ring, 4 * len(ring)) / (4 * len(ring))
        best = min(handoff_trials, key=handoff_trials.get)
        for b in ring:
            b.set_plan(**{**{k: pl[k] for k in PLAN_SET_KEYS}, "handoff_it": best})
            b.solve()
    # the FP32 answers of the timed plan against batched FP64, scenario by
    # scenario: only the confirmed ones count
    r = fast.results(state=True)
    assert np.all(r["final_mismatch"][r["status"] == 0] <= 1e-8)
    for b in ring[1:]:
        assert np.array_equal(b.results(state=False)["status"], r["status"])
    slow = gb.Batch(grids, device=dev, precision=gb.PREC_FP64, **opts)
    slow.set_instances(gi, Pload=Pl, Qload=Ql, Pg=Pg)
    if not a.no_autotune:
        slow.autotune(repeats=2)
    slow.solve()
    rs = slow.results(state=True)
    valid, check = fp64_check(np, fast, r, slow, rs, fast.offsets)
    conv = int(valid.sum())
    ms64 = slow.time(max(3, a.steps // 4)) / max(3, a.steps // 4)
    batched64 = int((rs["status"] == 0).sum()) / (ms64 / 1e3)
    slow.close()
    # device-resident: CUDA events on the batch streams; every step is a full
    # solve of all scenarios, steps go round the batches
    gb.time_pipelined(ring, max(3, a.warmup))
    fast.time(max(3, a.warmup))
    if dist:
        dist.barrier()
    with Clocks(dev) as clk:
        ms = gb.time_pipelined(ring, a.steps)
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
    kf = len(ring)
    hPl, hQl, hPg = pinned(Pl), pinned(Ql), pinned(Pg)
    outs = [pinned_results(n_scen, nb) for _ in range(kf)]

    def e2e_steps(k):
        for i in range(k):
            b = ring[i % kf]
            b.set_instances(gi, Pload=hPl, Qload=hQl, Pg=hPg)
            b.launch()
            if i >= kf - 1:
                j = (i - kf + 1) % kf
                outs[j] = ring[j].results(state=True, out=outs[j])
        for i in range(max(0, k - kf + 1), k):
            j = i % kf
            outs[j] = ring[j].results(state=True, out=outs[j])

    e2e_steps(max(3, a.warmup))
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    e2e_steps(a.steps)
    t_e2e = max_over_ranks(time.perf_counter() - t0, dist, dev)
    e2e = total_conv * a.steps / t_e2e
    res = outs[(a.steps - 1) % kf]
    assert np.array_equal(res["iterations"], r["iterations"])
    # the plain FP64 form (one scenario per gbpf_solve), same scenarios (c2)
    plain, plain_info = None, None
    if a.workload == "c2":
        P2, Q2, G2 = (x.reshape(n_scen, -1) for x in (Pl, Ql, Pg))
        plain, plain_info = plain_fp64_rate(gb, grids[0], dev, P2, Q2, G2, min(n_scen, 512), 1, 100)
    info = fast.info()
    pk = peaks()
    l2 = l2_copy_gbs(dev)
    # the dominant kernel: the warp kernel (or the block kernel when no
    # instance runs on warps); its own time per launch from CUDA events
    # recorded inside the graph around each kernel, on the stream it runs on
    kt = fast.kernel_times(max(3, a.steps // 4))
    pl_k = fast.plan()
    warp = info["warp_instances"] > 0
    kernel = (f"k_nr_warp<float, {pl_k['warp_state_global']}>" if warp else
              f"k_nr_block<float, {pl_k['block_state_global']}>")
    t_launch = (kt["warp"] if warp else kt["block"]) / 1e3
    ho = pl_k["handoff_it"]
    its = r["iterations"].astype(np.int64)
    kernel_its = np.minimum(its, ho) if (warp and ho > 0) else its
    # per instance-iteration bytes of each topology, weighted by its instances
    per_topo = [bytes_per_iteration(path_sizes(g), 4) for g in grids]
    alg = float(sum(per_topo[t] * kernel_its[gi == t].sum() for t in range(len(grids))))
    sizes = [path_sizes(g) for g in grids]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (fp32 LU)", "data": "synthetic",
        "config": {"workload": a.workload, "grid": desc, "grids": workload_files(a.workload),
                   "instances_per_gpu": n_scen, "tolerance": 1e-8, "no_max_iter": 100, "lim_inj_reat": 1,
                   "form": "batched, FP32 LU + FP64 mismatch/test/update, flat start (the learned start: workload c5)",
                   "converged_per_step": int(total_conv), "fp64_check": check,
                   "mean_iterations": float(np.mean(r["iterations"])),
                   "max_iterations": int(np.max(r["iterations"])),
                   "ns_per_instance_iteration": t_dev / a.steps / float(its.sum()) * 1e9,
                   "path_sizes": sizes if a.workload == "c4" else sizes[0],
                   "plain_fp64_solves_per_s": plain, "plain_fp64_solver": plain_info,
                   "batched_fp64_solves_per_s": batched64,
                   "speedup_vs_plain_fp64": (value / plain) if plain else None,
                   "in_flight": f"{IN_FLIGHT} batches of the same scenarios, one stream each, steps going round "
                                "them; each step a full solve of every scenario",
                   "serial_solves_per_s": serial,
                   "l2": (f"inputs+outputs {nb * 8 * 9 / 2**20:.0f} MiB > L2 (129 MB)" if nb * 72 > L2_BYTES else
                          f"inputs+outputs {nb * 8 * 9 / 2**20:.1f} MiB < L2; no flush"),
                   "batch": info, "plan": pl_k, "autotune": tune,
                   "in_flight_handoff_ms_per_step": handoff_trials or None,
                   "parallelism": f"scenarios sharded x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": nb * 8 * 3,
                "d2h_bytes_per_step": nb * 8 * 4 + n_scen * 20,
                "note": "per step: the caller's Pload, Qload, Pg arrays (pinned host memory) up as they are "
                        "(packed into Pliq, Qliq, "
                        "Qload on the device; the start is the grid's own, kept on the device), V, theta, Pcalc, "
                        f"Qcalc and the per-instance results down into the caller's arrays; {IN_FLIGHT} batches in "
                        f"flight (step k is launched before step k-{IN_FLIGHT - 1}'s results are read)"},
        "roofline": roofline(kernel, alg, t_launch, int(kernel_its.sum()), pk, l2,
                             "dependent-latency bound: the per-instance state, factor and topology stay in shared "
                             "memory and L2, so the algorithmic bytes come from on-chip memory; DRAM carries the "
                             "inputs and outputs", workload=a.workload),
        "clocks": clk.summary(),
        "gpu_launches": a.steps * launches_per_solve(pl_k),
    }
    line["roofline"]["kernel_ms_per_launch_all"] = kt
    if rank == 0 and not a.no_cpu_baseline and a.workload == "c2":
        line["cpu_baseline"] = cpu_baseline_scenarios(files[0], 1, draw_seed("c2", rank), n_scen)
    return line


def train_flops_per_step(nb, width, B, k_metric, n_in=None):
    """Multiply-add FLOPs of the tensor-core GEMMs of one training step."""
    kin, out = (n_in or 3 * nb), 2 * nb
    fwd = kin * width + 2 * width * width + width * out + kin * out
    metric = 2 * out * k_metric
    dh = out * width + 2 * width * width
    dw = width * kin + 2 * width * width + out * width + out * kin
    return 2.0 * B * (fwd + metric + dh + dw)


def fp64_check_c2(gb, np, dev, rank, n=N_SCEN_C2):
    """The FP32-LU form against FP64 on the c2 draw (118-bus grid, reactive
    limits on, n scenarios, default launch plans): fp64_check's record, with
    the grid and count named."""
    grid = gb.read_grid(grid_file("c2_base.cdf"))
    Pl, Ql, Pg = (x.ravel() for x in scenarios(np, grid.buses(), n, draw_seed("c2", rank)))
    res = []
    for prec in (gb.PREC_FP32_IR, gb.PREC_FP64):
        b = gb.Batch([grid], device=dev, precision=prec, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
        b.set_instances(np.zeros(n, np.int32), Pload=Pl, Qload=Ql, Pg=Pg)
        b.solve()
        res.append((b, b.results(state=True)))
    (b32, r32), (b64, r64) = res
    _, rec = fp64_check(np, b32, r32, b64, r64, b32.offsets)
    for b, _ in res:
        b.close()
    return {"grid": "c2_base.cdf (118 buses, reactive limits on)", **rec}


def bench_c5(a, gb, np, rank, dev, world, dist):
    n_train = a.train or C5_TRAIN
    n_test = a.scenarios or C5_TEST
    cdf = grid_file("c5_base.cdf.gz")
    grid = gb.read_grid(cdf)
    nB, base = grid.nB, grid.buses()
    opts = dict(tolerancia=1e-8, no_max_iter=30, lim_inj_reat=0)
    # training set: solutions of the plain Newton method (batched FP64, flat start)
    Pl, Ql, Pg = c5_scenarios(np, base, n_train, shard_seed(BASE_SEED + 5, rank))
    gen = gb.Batch([grid], device=dev, precision=gb.PREC_FP64, **opts)
    t0 = time.perf_counter()
    gen.set_instances(np.zeros(n_train, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    gen.solve()
    r = gen.results()
    t_gen = time.perf_counter() - t0
    ok = r["status"] == 0
    V, th = r["V"].reshape(-1, nB)[ok], r["theta"].reshape(-1, nB)[ok]
    # features [Pliq | Qliq]: every scenario starts from the grid's own
    # voltages, so V0 features would be constant (zeros once normalised)
    X = gb.warm_features(Pg[ok] - Pl[ok], base["Qg"] - Ql[ok])
    Y = gb.warm_targets(V, th)
    n_in = X.shape[1]
    gen.close()
    del r, Pl, Ql, Pg
    # batch 1024 at lr 2e-3, 120 epochs: against batch 256 at 1e-3 for 60
    # epochs, 3.5x the tensor-core rate (146 vs 42 TFLOP/s), 6.1 vs 10.8 s,
    # lower loss and fewer iterations from the predicted start (3.13 vs 3.27)
    width, batch, epochs, lam, lr0 = 512, 1024, 120, 1.0, 2e-3
    m = gb.MLP(n_in, 2 * nB, width=width, n_layers=3, skip=True, seed=BASE_SEED + 5, device=dev)
    m.set_data(X, Y)
    plain = gb.Solver(grid, device=dev, metodo=0, **opts)
    A = gb.warm_loss_metric(plain, V.mean(0), th.mean(0), m.norm()["out_scale"])
    plain.close()
    m.set_loss_metric(A, lam)
    loss, train_ms = m.train(epochs, batch=batch, lr=lr0, lr_final=1e-5, seed=BASE_SEED + 5)
    steps_per_epoch = len(X) // batch
    train_tflops = train_flops_per_step(nB, width, batch, (A.shape[1] + 7) // 8 * 8, n_in) * steps_per_epoch * epochs / (
        train_ms / 1e3) / 1e12
    del X, Y, V, th
    # held-out scenarios
    Pt, Qt, Gt = c5_scenarios(np, base, n_test, draw_seed("c5", rank))
    gi = np.zeros(n_test, np.int32)
    inputs = dict(Pload=Pt.ravel(), Qload=Qt.ravel(), Pg=Gt.ravel())
    ref = gb.Batch([grid], device=dev, precision=gb.PREC_FP64, **opts)
    ref.set_instances(gi, **inputs)
    ref.solve()
    r64 = ref.results()
    ms64 = ref.time(3) / 3
    fast = gb.Batch([grid], device=dev, precision=gb.PREC_FP32_IR, **opts)
    fast.set_instances(gi, **inputs)
    fast.solve()
    # launch plan: the autotuner's coordinate search on these instances from
    # the flat start (set-up, outside the timed region); the warm-started
    # launches use the same kernel and plan
    tune = None
    if not a.no_autotune:
        plan, ms0, ms1 = fast.autotune(repeats=3)
        tune = {"plan": plan, "ms_default_plan": ms0, "ms_chosen_plan": ms1}
        fast.solve()
    r32 = fast.results(state=False)
    ms32 = fast.time(3) / 3
    # a second batch of the same scenarios, for two warm-started solves in
    # flight (the timed steps and the end-to-end steps)
    twin = gb.Batch([grid], device=dev, precision=gb.PREC_FP32_IR, **opts)
    twin.set_instances(gi, **inputs)
    pl = fast.plan()
    twin.set_plan(**{k: pl[k] for k in PLAN_SET_KEYS})
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
    assert np.all(rw["final_mismatch"][rw["status"] == 0] <= 1e-8)
    # every warm-started FP32 answer against the FP64 flat-start solve of the
    # same scenario: only the confirmed ones count
    valid, check = fp64_check(np, fast, rw, ref, r64, fast.offsets)
    conv = int(valid.sum())
    t_dev = max_over_ranks(t_steps / 1e3, dist, dev)
    value = sum_over_ranks(conv, dist, dev) * a.steps / t_dev
    it_w = rw["iterations"] + np.where(kind == 2, w["warm_iterations"], 0)
    w64 = ref.solve_warm(m)
    r64w = ref.results(state=False)
    ref.close()
    # end to end through the public API with host buffers, double-buffered:
    # step k's inputs go up and its warm-started solve is launched before step
    # k-1's results are read back (two batches, one network)
    pair = [fast, twin]
    hinputs = {k: pinned(v) for k, v in inputs.items()}
    outs = [pinned_results(n_test, n_test * nB) for _ in range(2)]

    def e2e_steps(k):
        for i in range(k):
            b = pair[i % 2]
            b.set_instances(gi, **hinputs)
            if i > 0:
                b.follow(pair[(i - 1) % 2])  # one Newton launch at a time on the device
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
    plain_rate, plain_info = plain_fp64_rate(gb, grid, dev, Pt, Qt, Gt, min(n_test, 128), 0, 30)
    # the same FP32-LU form where PV buses switch (c5 has no reactive limits):
    # the c2 draw (118-bus grid, limits on), FP32 against FP64 scenario by
    # scenario, outside the timed region
    check_lim = fp64_check_c2(gb, np, dev, rank)
    pk = peaks()
    l2 = l2_copy_gbs(dev)
    sz = path_sizes(grid)
    # the Newton launch processes every iteration of every instance, the
    # failed predicted runs included
    inst_iters = int(it_w.sum())
    # iteration 0 of each predicted run is a chord step on the shared factor
    pred_it = np.where(kind == 1, rw["iterations"], np.where(kind == 2, w["warm_iterations"], 0))
    chords = int((pred_it >= 1).sum())
    alg = float(bytes_per_iteration(sz, 4) * inst_iters - chord_bytes_saved(sz, 4) * chords)
    kernel = f"k_nr_block<float, {fast.plan()['block_state_global']}>"
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": t_dev * 1e3 / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64 (fp32 LU)", "data": "synthetic",
        "config": {"workload": "c5", "grid": "1888-bus (16 tied 118-bus copies), limits off",
                   "grids": workload_files("c5"),
                   "instances_per_gpu": n_test, "tolerance": 1e-8, "no_max_iter": 30,
                   "form": "batched, FP32 LU + FP64 mismatch/test/update, learned warm start with flat-start "
                           "fallback; iteration 0 of a predicted run a chord step on the factor of the Jacobian "
                           "at the network's mean output (network inference, start choice and Newton inside the "
                           "timed region)",
                   "network": f"{n_in} ([Pliq | Qliq]) -> 3 x {width} GELU -> {2 * nB} + linear skip, bf16 weights, fp32 "
                              f"accumulation; loss |e A|^2 + {lam} |e|^2 (A = S J0^T); Adam lr {lr0:g} cosine to "
                              f"1e-5, {epochs} epochs, batch {batch}",
                   "train_solves": n_train, "train_converged": int(ok.sum()),
                   "train_generation_s": t_gen, "train_s": train_ms / 1e3,
                   "train_loss_first_last": [float(loss[0]), float(loss[-1])],
                   "converged_per_step": conv, "fp64_check": check, "fp64_check_with_reactive_limits": check_lim,
                   "in_flight": "2 batches of the same scenarios, one stream each, steps alternating, each step "
                                "started on the device when the previous one ends (the host enqueues ahead); each "
                                "step a full warm-started solve of every scenario",
                   "serial_solves_per_s": sum_over_ranks(conv, dist, dev) * a.steps
                                          / max_over_ranks(t_serial / 1e3, dist, dev),
                   "phases_ms": {k: round(v, 4) for k, v in phases.items()},
                   "ns_per_instance_iteration": phases["newton"] * 1e6 / inst_iters,
                   "chord_iterations_per_step": chords,
                   "path_sizes": sz,
                   "plan": fast.plan(), "autotune": tune,
                   "mean_iterations_flat_fp32": float(r32["iterations"].mean()),
                   "mean_iterations_warm_fp32": float(it_w.mean()),
                   "mean_iterations_flat_fp64": float(r64["iterations"].mean()),
                   "mean_iterations_warm_fp64": float((r64w["iterations"] + np.where(
                       w64["start_kind"] == 2, w64["warm_iterations"], 0)).mean()),
                   "start_kind_counts": {"flat_chosen": int((kind == 0).sum()), "predicted": int((kind == 1).sum()),
                                         "fallback": int((kind == 2).sum())},
                   "fallback_rate": float((kind == 2).mean()),
                   "plain_fp64_solves_per_s": plain_rate, "plain_fp64_solver": plain_info,
                   "batched_fp64_flat_solves_per_s": int((r64["status"] == 0).sum()) / (ms64 / 1e3),
                   "batched_fp32_flat_solves_per_s": int((r32["status"] == 0).sum()) / (ms32 / 1e3),
                   "speedup_vs_plain_fp64": value / plain_rate if plain_rate else None,
                   "l2": f"per-step inputs {n_test * nB * 8 * 9 / 2**20:.0f} MiB > L2",
                   "parallelism": f"scenarios sharded x{world}"},
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": n_test * nB * 8 * 3,
                "d2h_bytes_per_step": n_test * nB * 8 * 4 + n_test * 20},
        "roofline": roofline(kernel, alg, phases["newton"] / 1e3, inst_iters, pk, l2,
                             "one persistent Newton launch per step (restarts included), timed over its phase of "
                             "the step; dependent-load latency bound", workload="c5"),
        "roofline_training": {"bound": "tensor", "kernel": "k_gemm (tcgen05 bf16, all training GEMMs)",
                              "achieved": train_tflops, "peak": pk["bf16"], "unit": "TFLOP/s",
                              "frac": train_tflops / pk["bf16"],
                              "peak_source": ("MEASURED_PEAKS.json bf16_tflops_sustained" if pk["src"] == "measured"
                                              else "fallback")},
        "clocks": clk.summary(),
        # features, 4 network layers, start choice, queue order, Newton (restarts included)
        "gpu_launches": a.steps * (1 + 4 + 1 + 1 + 1),
    }
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_c5(cdf, Pt, Qt, Gt)
    return line


def bench_single(a, gb, np, rank, dev, world, dist):
    dense = a.workload.endswith("-dense")
    lim = 1
    if a.workload == "c3":
        desc = "15104-bus (128 tied 118-bus copies), limits on"
    elif a.workload == "c5-dense":
        desc, lim = "1888-bus (16 tied 118-bus copies), limits off", 0
    else:
        desc = "118-bus meshed (1 slack/53 PV/64 PQ, 186 branches), limits on"
    cdf = grid_file(workload_files(a.workload)[0])
    grid = gb.read_grid(cdf)
    s = gb.Solver(grid, device=dev, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=1 if dense else 0)
    first = s.solve(full=False)
    assert first["converged"] and first["final_mismatch"] <= 1e-8, first
    info = s.info()
    form = s.form()
    info["form"] = "persistent" if form["form"] == gb.FORM_PERSISTENT else "graph"
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
    pk = peaks()
    it = max(1, first["iterations"])
    t_it = t_dev / a.steps / it
    if dense:
        # metodo = denso: per Newton iteration the N x N FP64 matrix is written
        # by the fill and read and written once by the LU's panel sweep (lower
        # bound on its traffic); the LU does 2/3 N^3 + 2 N^2 flops
        N = 2 * (grid.nB - 1)
        achieved = 3 * N * N * 8 / t_it / 1e9
        top, prof = "dense fill + LU + solves", {"matrix_order": N, "iterations": first["iterations"],
                                                 "ms_per_iteration": 1e3 * t_it,
                                                 "lu_fp64_gflops": (2 / 3 * N ** 3 + 2 * N * N) / t_it / 1e9,
                                                 "phases": s.profile(5)}
        rl = {"bound": "hbm", "kernel_phase": top, "achieved": achieved, "peak": pk["hbm"], "unit": "GB/s",
              "frac": achieved / pk["hbm"], "peak_source": peak_src_note(pk["src"]), "traffic": None,
              "phases": prof}
    else:
        sz = path_sizes(grid)
        alg = bytes_per_iteration(sz, 8) * it
        rl = roofline("plain FP64 solve (" + ("one persistent launch" if form["form"] == gb.FORM_PERSISTENT else
                                             "CUDA graph of per-phase kernels") + ")",
                      alg, t_dev / a.steps, it, pk, l2_copy_gbs(dev),
                      "one solve of one grid: dependent latency of the elimination levels bounds it")
        rl["phases"] = s.profile(10)
        rl["path_sizes"] = sz
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": a.steps,
        "warmup": max(3, a.warmup), "ms_per_step": 1e3 * t_dev / a.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": a.workload, "grid": desc, "grids": workload_files(a.workload), "nB": grid.nB,
                   "tolerance": 1e-8, "lim_inj_reat": lim,
                   "form": ("metodo = denso: dense FP64 Jacobian and LU with partial pivoting, one solve per step"
                            if dense else "plain FP64, one solve per step"), "iterations": first["iterations"],
                   "ms_per_iteration": 1e3 * t_it,
                   "solver": info, "parallelism": f"replicas x{world}", "fp32_lu": fp32,
                   "l2": "working set fits in L2; no flush"},
        "e2e": {"value": world * a.steps / t_e2e, "unit": UNIT, "h2d_bytes_per_step": 4 * grid.nB * 8,
                "d2h_bytes_per_step": 4 * grid.nB * 8 + 32},
        "roofline": rl,
        "clocks": clk.summary(),
        "gpu_launches": a.steps * (form["launches"] + it * form["launches_per_iteration"]),
    }
    if rank == 0 and not a.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline_repeat(cdf, lim)
    return line


SECONDARY = ("c2", "c4", "c3")


def secondary_summaries(a, gb, np, rank, dev, world, dist):
    """The other configurations, run after the headline in the same process
    (N = 1 only) and reported inside its line: c2 (32,768 load scenarios of
    the 118-bus grid with reactive limits, FP32 LU checked against FP64, its
    plain FP64 form and the one-core oracle beside it), c4 (4,096 instances of
    14..472-bus grids) and c3 (one 15,104-bus solve, FP64 and FP32 LU).  Each
    is a full bench of its own (same timing rules and steps, at most 50);
    one that fails is reported with its error instead of ending the run."""
    import copy

    out = {}
    for wl in SECONDARY:
        b = copy.copy(a)
        b.workload = wl
        b.steps = min(a.steps, 50)
        b.warmup = max(3, min(a.warmup, 5))
        b.scenarios = 0
        b.no_cpu_baseline = wl != "c2"
        try:
            if wl in ("c2", "c4"):
                ln = bench_batch(b, gb, np, rank, dev, world, dist)
            else:
                ln = bench_single(b, gb, np, rank, dev, world, dist)
        except Exception as ex:  # reported, so that the headline line still prints
            out[wl] = {"error": f"{type(ex).__name__}: {ex}"[:400]}
            continue
        cfg = ln["config"]
        keep = ("form", "grid", "instances_per_gpu", "nB", "iterations", "mean_iterations", "max_iterations",
                "converged_per_step", "plain_fp64_solves_per_s", "batched_fp64_solves_per_s",
                "speedup_vs_plain_fp64", "ns_per_instance_iteration", "ms_per_iteration", "fp32_lu", "l2")
        summ = {"value": ln["value"], "unit": ln["unit"], "ms_per_step": ln["ms_per_step"], "steps": ln["steps"],
                "warmup": ln["warmup"], "dtype": ln["dtype"], "e2e": ln.get("e2e"), "clocks": ln.get("clocks"),
                "gpu_launches": ln.get("gpu_launches"),
                "config": {k: cfg[k] for k in keep if k in cfg}}
        if "fp64_check" in cfg:
            summ["config"]["fp64_check"] = cfg["fp64_check"]
        rl = ln.get("roofline") or {}
        summ["roofline"] = {k: rl.get(k) for k in ("bound", "kernel", "kernel_phase", "achieved", "peak", "unit",
                                                   "frac") if k in rl}
        if "cpu_baseline" in ln:
            summ["cpu_baseline"] = ln["cpu_baseline"]
        out[wl] = summ
    return out


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
        if world == 1 and not a.no_secondary and not a.scenarios and not a.train:
            line["secondary_workloads"] = secondary_summaries(a, gb, np, rank, local_rank, world, dist)
    else:
        line = bench_single(a, gb, np, rank, local_rank, world, dist)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
