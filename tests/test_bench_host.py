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
