"""Host-side logic of bench.py, without a GPU: the kernel count a bench line
claims per solve, and the CPU baseline's bounded sample (the oracle on one
core for about the requested time, not a fixed count that the oracle's
per-call set-up would shrink)."""
import os
import sys
import time

import pytest

from conftest import GOLDEN, ROOT

sys.path.insert(0, ROOT)
import bench  # noqa: E402


@pytest.mark.parametrize("warp,block,handoff,launches", [
    (32768, 0, 12, 2),   # warps and the hand-off launch
    (32768, 0, 0, 1),    # warps only (hand-off off, as chosen in flight)
    (0, 4096, 12, 1),    # every instance on a block
    (2751, 1345, 12, 3),  # both kernels and the hand-off (mixed sizes)
])
def test_launches_per_solve(warp, block, handoff, launches):
    plan = dict(warp_instances=warp, block_instances=block, handoff_it=handoff)
    assert bench.launches_per_solve(plan) == launches


def test_cpu_baseline_sample_is_bounded():
    cdf = os.path.join(GOLDEN, "c2_base.cdf")
    t0 = time.perf_counter()
    r = bench.cpu_baseline_scenarios(cdf, 1, bench.BASE_SEED + 7, 4096, target_s=1.0)
    wall = time.perf_counter() - t0
    assert r["kind"] == "port" and r["cores"] == 1 and r["value"] > 0
    n = int(r["sample"].split()[1])
    solve_s = float(r["sample"].split(" s single-threaded")[0].split()[-1])
    # the timed sample lands near the target (the calibration runs come on top)
    assert 64 <= n <= 4096
    assert 0.4 <= solve_s <= 3.0 or n == 4096, r["sample"]
    assert wall < 10


def test_path_sizes_follow_the_reference_rules(gb):
    """nnzY, nnzJ, dimJ by the reference's rules: the IEEE 118-bus case gives
    the figures measured on it (476, 1,051, 181); nnzLU is this solver's block
    factor ((blocks + 2 x off-diagonal blocks) x 4)."""
    from conftest import ieee_cases, ieee_path
    case = next(c for c in ieee_cases() if c["cdf"] == "ieee118.cdf")
    sz = bench.path_sizes(gb.read_grid(ieee_path(case)))
    assert (sz["nB"], sz["nnzY"], sz["nnzJ"], sz["dimJ"]) == (118, 476, 1051, 181)
    sz = bench.path_sizes(gb.read_grid(os.path.join(GOLDEN, "c2_base.cdf")))
    assert (sz["nnzY"], sz["nnzJ"], sz["dimJ"], sz["nnzLU"]) == (490, 1161, 181, 2364)
    # 36 nnzY + 12 nnzJ + 3 (v + 4) nnzLU + 112 nB + 32 dimJ (+4: the row pointer's extra entry)
    assert bench.bytes_per_iteration(sz, 4) == 36 * 490 + 12 * 1161 + 24 * 2364 + 112 * 118 + 32 * 181 + 4
    assert bench.bytes_per_iteration(sz, 8) - bench.bytes_per_iteration(sz, 4) == 12 * 2364


class _FakeBatch:
    def __init__(self, ev, n):
        self.ev, self.n = ev, n

    def events_all(self):
        return self.ev, self.n


def test_fp64_check_counts_only_confirmed_answers():
    """Per scenario: both converge, same switch path (bus, PV position, code),
    |V| and theta within 1e-6 of FP64; everything else is reported and left
    out of the count."""
    import numpy as np
    nb = 3
    n = 5
    V64 = np.ones(n * nb)
    th64 = np.zeros(n * nb)
    V32, th32 = V64.copy(), th64.copy()
    V32[1 * nb] += 5e-7          # 1: within tolerance
    th32[2 * nb + 1] += 2e-6     # 2: beyond tolerance
    ev64 = np.zeros((n, 16, 4), np.int32)
    ev32 = ev64.copy()
    n64 = np.zeros(n, np.int32)
    n32 = n64.copy()
    ev64[3, 0] = (4, 7, 1, 1)    # 3: FP64 switched a PV bus, FP32 did not
    n64[3] = 1
    st32 = np.array([0, 0, 0, 0, 0])
    st64 = np.array([0, 0, 0, 0, 1])  # 4: FP64 did not converge
    r32 = dict(status=st32, V=V32, theta=th32)
    r64 = dict(status=st64, V=V64, theta=th64)
    ok, rec = bench.fp64_check(np, _FakeBatch(ev32, n32), r32, _FakeBatch(ev64, n64), r64,
                               np.arange(0, (n + 1) * nb, nb))
    assert ok.tolist() == [True, True, False, False, False]
    assert rec["counted"] == 2 and rec["diverged_switch_path"] == 1 and rec["beyond_tolerance"] == 1
    assert rec["fp32_only_converged"] == 1 and rec["both_converged"] == 4
    assert abs(rec["max_abs_err_vs_fp64"]["V"] - 5e-7) < 1e-15 and rec["max_abs_err_vs_fp64"]["theta"] == 0
    assert abs(rec["max_abs_err_beyond_tolerance"]["theta"] - 2e-6) < 1e-15


@pytest.mark.parametrize("workload", ["c2", "c4", "c5"])
def test_reference_arm_draws_the_gpu_arms_scenarios(gb, workload):
    """The reference arm reads the committed grids with the oracle's reader
    and draws exactly the scenarios the GPU arm draws with the product's."""
    import numpy as np
    files = [bench.grid_file(f) for f in bench.workload_files(workload)]
    gi, Pl, Ql, Pg, off = bench.reference_sample(np, workload, files, 0)
    grids = [gb.read_grid(f) for f in files]
    if workload == "c4":
        gi2, (Pl2, Ql2, Pg2) = bench.c4_instances(np, [g.buses() for g in grids], bench.N_SCEN,
                                                  bench.draw_seed("c4", 0))
        assert np.array_equal(gi, gi2)
    else:
        draw = bench.scenarios if workload == "c2" else bench.c5_scenarios
        n = bench.N_SCEN_C2 if workload == "c2" else bench.C5_TEST
        Pl2, Ql2, Pg2 = (x.ravel() for x in draw(np, grids[0].buses(), n, bench.draw_seed(workload, 0)))
    for a, b in ((Pl, Pl2), (Ql, Ql2), (Pg, Pg2)):
        np.testing.assert_array_equal(a, b)
    assert off[-1] == len(Pl)


def test_reference_arm_runs_without_the_library(tmp_path):
    """--impl reference: the same steps and warm-up as asked, the port's
    line, and the product's library never loaded in its process."""
    import json
    import subprocess
    code = ("import runpy, sys; sys.argv = ['bench.py', '--impl', 'reference', '--workload', 'c2', '--steps', '2', "
            "'--warmup', '1']; runpy.run_path('bench.py', run_name='__main__'); "
            "maps = open('/proc/self/maps').read(); print('LOADED' if 'libgbpf' in maps else 'CLEAN')")
    out = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=600)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.strip().splitlines()
    assert lines[-1] == "CLEAN"
    line = json.loads(lines[-2])
    assert line["impl"] == "reference" and line["steps"] == 2 and line["warmup"] == 1
    assert line["cpu_baseline"]["kind"] == "port" and line["value"] > 0
    assert line["e2e"]["h2d_bytes_per_step"] == 0


def test_secondary_summaries_report_each_workload_and_survive_a_failure(monkeypatch):
    """The c5 line's secondary workloads: each benched with a copy of the
    arguments (the same timed steps, at most 50; the one-core oracle only beside c2), a
    summary of its line kept, and a failing one reported by its error while
    the others still run."""
    import argparse

    import numpy as np

    calls = []

    def fake_line(b, *rest):
        calls.append((b.workload, b.steps, b.no_cpu_baseline))
        if b.workload == "c4":
            raise RuntimeError("no device")
        line = {"value": 2.0, "unit": "solves/s", "ms_per_step": 1.5, "steps": b.steps, "warmup": b.warmup,
                "dtype": "f64", "e2e": {"value": 1.0}, "clocks": {}, "gpu_launches": 3,
                "config": {"form": "batched", "fp64_check": {"counted": 7}, "unrelated": 1},
                "roofline": {"bound": "hbm", "frac": 0.25, "traffic": 1}}
        if not b.no_cpu_baseline:
            line["cpu_baseline"] = {"value": 5.0}
        return line

    monkeypatch.setattr(bench, "bench_batch", fake_line)
    monkeypatch.setattr(bench, "bench_single", fake_line)
    a = argparse.Namespace(workload="c5", steps=20, warmup=3, scenarios=0, train=0, no_cpu_baseline=False,
                           no_autotune=False, no_secondary=False, gpus=1, impl="gbpf")
    out = bench.secondary_summaries(a, None, np, 0, 0, 1, None)
    assert calls == [("c2", 20, False), ("c4", 20, True), ("c3", 20, True)]
    assert a.workload == "c5" and a.steps == 20
    assert out["c4"] == {"error": "RuntimeError: no device"}
    assert out["c2"]["value"] == 2.0 and out["c2"]["cpu_baseline"] == {"value": 5.0}
    assert out["c2"]["config"] == {"form": "batched", "fp64_check": {"counted": 7}}
    assert out["c2"]["roofline"] == {"bound": "hbm", "frac": 0.25}
    assert "cpu_baseline" not in out["c3"]
