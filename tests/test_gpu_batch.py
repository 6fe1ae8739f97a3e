"""Batched solves (one thread block per instance, many instances per launch)
against the oracle, instance by instance.

FP64 form: identical iteration counts and switch events, |V| and theta within
1e-9.  FP32-LU form: max|g| <= 1e-8 evaluated in FP64 and |V|, theta within
1e-6 of the FP64 oracle."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, ieee_cases, ieee_path, load_golden

pytestmark = pytest.mark.gpu


def scenarios(og, n, seed, sigma=0.1):
    """Per-bus load x lognormal(sigma), generation x U(0.9, 1.1)."""
    rng = np.random.default_rng(seed)
    lf = np.exp(rng.normal(-0.5 * sigma * sigma, sigma, (n, og.nB)))
    gf = rng.uniform(0.9, 1.1, (n, og.nB))
    return og.Pload * lf, og.Qload * lf, og.Pg * gf


def oracle_solve(og, Pl, Ql, Pg, lim, tol=1e-8, maxit=100):
    og.set_bus(Pload=Pl, Qload=Ql, Pg=Pg)
    return og.solve(tol, maxit, bool(lim))


def run_batch(gb, grids, inst_grid, Pl, Ql, Pg, **opts):
    base = dict(tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    base.update(opts)
    b = gb.Batch(grids, **base)
    b.set_instances(inst_grid, Pload=Pl, Qload=Ql, Pg=Pg)
    b.solve()
    return b, b.results()


@pytest.mark.parametrize("cdf", ["c2_base.cdf", "c2_s3.cdf", "c2_tx.m"])
def test_batch_fp64_matches_oracle(gb, oracle, cdf):
    path = os.path.join(GOLDEN, cdf)
    og = oracle.Grid(path)
    n = 48
    Pl, Ql, Pg = scenarios(og, n, 7)
    b, r = run_batch(gb, [gb.read_grid(path)], np.zeros(n, np.int32), Pl.ravel(), Ql.ravel(), Pg.ravel())
    switched = 0
    for i in range(n):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
        assert ref["converged"]
        assert r["status"][i] == 0 and r["iterations"][i] == ref["iterations"], i
        assert r["final_mismatch"][i] <= 1e-8
        ev = b.events(i)
        assert ev == ref["events"][:16], i
        switched += len(ev) > 0
        assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9
        assert np.max(np.abs(b.slice(r["theta"], i) - ref["theta"])) < 1e-9
    assert b.info()["factors_in_smem"] == 1


@pytest.mark.parametrize("case", ieee_cases(max_buses=3776), ids=lambda c: c["golden"])
def test_batch_fp64_matches_reference_golden_on_ieee(gb, case):
    """The reference's own IEEE inputs as batch instances (three copies of the
    case's own loads): identical iterations and switch events, |V|, theta
    within 1e-9 of the reference-built golden, in every copy."""
    g = gb.read_grid(ieee_path(case))
    gold = load_golden(case["golden"])
    n = 3
    b, r = run_batch(gb, [g], np.zeros(n, np.int32), None, None, None, no_max_iter=case["max_iter"],
                     lim_inj_reat=case["lim"])
    for i in range(n):
        assert r["iterations"][i] == gold["iterations"], i
        assert (r["status"][i] == 0) == bool(gold["converged"]), i
        ev = [list(e) for e in b.events(i)]
        assert ev == gold["events"][:len(ev)] and len(ev) == min(16, len(gold["events"]))
        if gold["converged"]:
            assert r["final_mismatch"][i] <= gold["tol"]
            assert np.max(np.abs(b.slice(r["V"], i) - np.array(gold["V"]))) < 1e-9
            assert np.max(np.abs(b.slice(r["theta"], i) - np.array(gold["theta"]))) < 1e-9


def test_batch_rejects_grids_beyond_shared_memory(gb):
    """A block keeps each instance's substitution vectors and bus flags in
    shared memory; the 7,552-bus ieee118x64 needs more than a block has, which
    the batch reports (GBPF_E_UNSUPPORTED) instead of launching.  The
    single-grid solver takes that grid (test_gpu_parity)."""
    case = next(c for c in ieee_cases() if c["cdf"] == "ieee118x64.cdf")
    b = gb.Batch([gb.read_grid(ieee_path(case))], tolerancia=1e-8, no_max_iter=100)
    with pytest.raises(gb.GbpfError) as e:
        b.set_instances(np.zeros(2, np.int32))
    assert e.value.status == gb.E_UNSUPPORTED
    assert "shared memory" in str(e.value)


def test_batch_mixed_ieee_topologies_fp64(gb):
    """Every IEEE case up to 944 buses in one launch, instances interleaved."""
    cases = [c for c in ieee_cases(max_buses=944) if c["lim"] == 1]
    grids = [gb.read_grid(ieee_path(c)) for c in cases]
    golds = [load_golden(c["golden"]) for c in cases]
    inst = np.tile(np.arange(len(cases), dtype=np.int32), 4)
    b, r = run_batch(gb, grids, inst, None, None, None)
    for i, t in enumerate(inst):
        gold = golds[t]
        assert r["iterations"][i] == gold["iterations"], (i, cases[t]["cdf"])
        if gold["converged"]:
            assert np.max(np.abs(b.slice(r["V"], i) - np.array(gold["V"]))) < 1e-9
            assert np.max(np.abs(b.slice(r["theta"], i) - np.array(gold["theta"]))) < 1e-9


def test_batch_mixed_topologies_fp64(gb, oracle, tmp_path):
    paths = [os.path.join(GOLDEN, "c1.cdf"), os.path.join(GOLDEN, "c2_base.cdf")]
    for nb in (236, 472):
        g = gb.generate(4, 20261207 + nb, nbus=nb)
        p = str(tmp_path / f"g{nb}.cdf")
        g.write_cdf(p)
        paths.append(p)
    grids = [gb.read_grid(p) for p in paths]
    ogs = [oracle.Grid(p) for p in paths]
    rng = np.random.default_rng(3)
    inst = rng.integers(0, len(paths), 40).astype(np.int32)
    packs = [[], [], []]
    per = []
    for i, t in enumerate(inst):
        Pl, Ql, Pg = scenarios(ogs[t], 1, 100 + i)
        per.append((Pl[0], Ql[0], Pg[0]))
        for k in range(3):
            packs[k].append(per[-1][k])
    b, r = run_batch(gb, grids, inst, *[np.concatenate(p) for p in packs])
    info = b.info()
    assert info["topologies"] == 4 and info["instances"] == 40
    for i, t in enumerate(inst):
        ref = oracle_solve(ogs[t], *per[i], 1)
        assert r["iterations"][i] == ref["iterations"] and r["status"][i] == 0, (i, t)
        assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9
        assert np.max(np.abs(b.slice(r["theta"], i) - ref["theta"])) < 1e-9


@pytest.mark.parametrize("rotate", [0, 1], ids=["sincos", "rotation"])
def test_batch_fp32_lu_accuracy(gb, oracle, rotate):
    path = os.path.join(GOLDEN, "c2_base.cdf")
    og = oracle.Grid(path)
    n = 32
    Pl, Ql, Pg = scenarios(og, n, 11)
    b = gb.Batch([gb.read_grid(path)], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1, precision=gb.PREC_FP32_IR)
    b.set_plan(rotate=rotate)
    b.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    b.solve()
    r = b.results()
    for i in range(n):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
        assert r["status"][i] == 0 and r["final_mismatch"][i] <= 1e-8
        assert r["iterations"][i] <= ref["iterations"] + 3
        assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-6
        assert np.max(np.abs(b.slice(r["theta"], i) - ref["theta"])) < 1e-6


def test_batch_large_factor_in_scratch(gb, oracle, tmp_path):
    g = gb.generate(3, 20261208, tiles=16)
    p = str(tmp_path / "c5.cdf")
    g.write_cdf(p)
    og = oracle.Grid(p)
    n = 6
    Pl, Ql, Pg = scenarios(og, n, 5)
    b, r = run_batch(gb, [gb.read_grid(p)], np.zeros(n, np.int32), Pl.ravel(), Ql.ravel(), Pg.ravel(),
                     lim_inj_reat=0)
    assert b.info()["factors_in_smem"] == 0 and b.info()["scratch_bytes_per_block"] > 0
    for i in range(n):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 0)
        assert r["iterations"][i] == ref["iterations"]
        assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9


def test_batch_repeat_is_deterministic(gb):
    path = os.path.join(GOLDEN, "c2_s8.cdf")
    g = gb.read_grid(path)
    b = gb.Batch([g], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    b.set_instances(np.zeros(300, np.int32))
    b.solve()
    a = b.results()
    b.solve()
    c = b.results()
    np.testing.assert_array_equal(a["V"], c["V"])
    np.testing.assert_array_equal(a["iterations"], c["iterations"])
    # identical instances give identical answers whatever block ran them
    V = a["V"].reshape(300, g.nB)
    assert np.all(V == V[0])


def test_batch_handoff_of_long_instances(gb, oracle):
    """Instances still iterating at iteration 12 leave the warp-per-instance
    kernel for a thread block of their own, which continues from the parked
    state with the same arithmetic.  Scenarios of the bench workload that take
    14, 17, 23 and 100 (no convergence, limit cycling) iterations, among
    ordinary ones: FP64 iteration counts, statuses and switch events equal the
    oracle's, |V| and theta within 1e-9 for the converged.  The FP32-LU form
    converges on the same instances; where its PV -> PQ switch sequence is the
    FP64 one, |V| and theta are within 1e-6 of the oracle.  With reactive
    limits a generator whose Q sits within rounding of its limit when the
    check runs can switch on another iteration in FP32, and the solve then
    ends at another valid operating point: at most 2 of the 36 here."""
    import bench

    path = os.path.join(GOLDEN, "c2_base.cdf")
    og = oracle.Grid(path)
    base = dict(Pload=og.Pload.copy(), Qload=og.Qload.copy(), Pg=og.Pg.copy())
    Pl, Ql, Pg = bench.scenarios(np, base, 4096, bench.BASE_SEED + 7)
    pick = list(range(32)) + [1943, 2749, 3628, 4084]  # 23 (23 iterations) is among the first 32
    Pl, Ql, Pg = Pl[pick], Ql[pick], Pg[pick]
    n = len(pick)
    grid = gb.read_grid(path)
    b, r = run_batch(gb, [grid], np.zeros(n, np.int32), Pl.ravel(), Ql.ravel(), Pg.ravel())
    assert b.info()["warp_instances"] == n
    b32, r32 = run_batch(gb, [grid], np.zeros(n, np.int32), Pl.ravel(), Ql.ravel(), Pg.ravel(),
                         precision=gb.PREC_FP32_IR)
    long_ = other_path = 0
    for i in range(n):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
        assert r["iterations"][i] == ref["iterations"], i
        assert (r["status"][i] == 0) == ref["converged"], i
        assert b.events(i) == ref["events"][:16], i
        long_ += ref["iterations"] > 12
        if ref["converged"]:
            assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9
            assert np.max(np.abs(b.slice(r["theta"], i) - ref["theta"])) < 1e-9
            assert r32["status"][i] == 0 and r32["final_mismatch"][i] <= 1e-8
            if [e[1:] for e in b32.events(i)] == [e[1:] for e in ref["events"][:16]]:
                assert np.max(np.abs(b32.slice(r32["V"], i) - ref["V"])) < 1e-6
                assert np.max(np.abs(b32.slice(r32["theta"], i) - ref["theta"])) < 1e-6
            else:
                other_path += 1
        else:
            assert r["iterations"][i] == 100
    assert long_ == 5
    assert other_path <= 2


PLANS = [
    dict(),                                             # default: warps, grouped lanes, hand-off at 12
    dict(warp_group=0, resume_group=0),                 # one lane per pivot everywhere
    dict(handoff_it=0),                                 # no hand-off: long instances stay on their warp
    dict(handoff_it=6, warps_per_block=2),
    dict(warp_mode=0),                                  # every instance on a thread block
    dict(warp_mode=0, narrow=1),                        # ... narrow levels on one warp
    dict(lu1=0, narrow=1),                              # two passes per level (pivots, then entries)
    dict(warp_mode=0, lu1=0),
    dict(warp_lu1=1, handoff_it=8),                     # one-pass levels in the warps too
    dict(rotate=1),                                     # FP32 phasors by rotation (FP64 here: no effect)
    dict(warp_gstate=3, warps_per_block=0),             # warp state in global memory, 16 warps per block
    dict(warp_mode=0, gstate=4),                        # block state in global memory, 4 blocks per SM
]


@pytest.mark.parametrize("plan", PLANS, ids=lambda p: ",".join(f"{k}={v}" for k, v in p.items()) or "default")
def test_batch_plans_match_oracle(gb, oracle, plan):
    """Every launch plan the autotuner can choose gives the oracle's FP64
    answers: iteration counts, statuses, switch events, |V| and theta within
    1e-9 (plans differ only in the summation order of grouped lanes)."""
    import bench

    path = os.path.join(GOLDEN, "c2_base.cdf")
    og = oracle.Grid(path)
    base = dict(Pload=og.Pload.copy(), Qload=og.Qload.copy(), Pg=og.Pg.copy())
    Pl, Ql, Pg = bench.scenarios(np, base, 4096, bench.BASE_SEED + 7)
    pick = list(range(24)) + [1943, 2749, 3628, 4084]
    Pl, Ql, Pg = Pl[pick], Ql[pick], Pg[pick]
    n = len(pick)
    b = gb.Batch([gb.read_grid(path)], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    full = dict(warp_mode=1, warps_per_block=8, handoff_it=12, resume_group=1, warp_group=1, narrow=0, lu1=1,
                warp_lu1=0)
    full.update(plan)
    b.set_plan(**full)
    b.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
    b.solve()
    r = b.results()
    got = b.plan()
    assert got["warp_mode"] == full["warp_mode"] and got["handoff_it"] == full["handoff_it"]
    assert got["warp_instances"] == (n if full["warp_mode"] else 0)
    for i in range(n):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
        assert r["iterations"][i] == ref["iterations"], i
        assert (r["status"][i] == 0) == ref["converged"], i
        assert b.events(i) == ref["events"][:16], i
        if ref["converged"]:
            assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9
            assert np.max(np.abs(b.slice(r["theta"], i) - ref["theta"])) < 1e-9


def test_batch_autotune(gb, oracle):
    """The autotuner returns a valid plan no slower than the one it started
    from, and the batch solved with it still matches the oracle."""
    path = os.path.join(GOLDEN, "c2_s3.cdf")
    og = oracle.Grid(path)
    n = 512
    Pl, Ql, Pg = scenarios(og, n, 11)
    b, _ = run_batch(gb, [gb.read_grid(path)], np.zeros(n, np.int32), Pl.ravel(), Ql.ravel(), Pg.ravel(),
                     precision=gb.PREC_FP32_IR)
    plan, ms0, ms1 = b.autotune(repeats=2)
    assert 0 < ms1 <= ms0 * 1.05
    assert plan["warp_mode"] in (0, 1) and plan["handoff_it"] >= 0
    assert b.plan() == plan
    b.solve()
    r = b.results()
    for i in range(0, n, 37):
        ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
        assert (r["status"][i] == 0) == ref["converged"], i
        if ref["converged"]:
            assert r["final_mismatch"][i] <= 1e-8
            if [e[1:] for e in b.events(i)] == [e[1:] for e in ref["events"][:16]]:
                assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-6


def test_batch_starting_state_kept_or_replaced(gb):
    """The grids' own start stays on the device between calls with the same
    instances and no V0 / theta0; a given start replaces it and the next call
    without one restores it."""
    path = os.path.join(GOLDEN, "c2_s3.cdf")
    g = gb.read_grid(path)
    n = 64
    gi = np.zeros(n, np.int32)
    b = gb.Batch([g], tolerancia=1e-8, no_max_iter=50, lim_inj_reat=1)
    b.set_instances(gi)
    b.solve()
    ref = b.results()
    base = g.buses()
    V0 = np.tile(base["V0"], n) * 0.97
    b.set_instances(gi, V0=V0)
    b.solve()
    other = b.results()
    assert not np.array_equal(other["iterations"], ref["iterations"]) or \
        not np.array_equal(other["V"], ref["V"])
    for _ in range(2):
        b.set_instances(gi)
        b.solve()
        r = b.results()
        np.testing.assert_array_equal(r["iterations"], ref["iterations"])
        np.testing.assert_array_equal(r["V"], ref["V"])


@pytest.mark.parametrize("precision", [0, 1], ids=["fp64", "fp32"])
def test_batch_shared_flat_start_is_exact(gb, precision):
    """Iteration 0 from the grids' own start, computed once per topology and
    shared (plan flat_shared), gives bit-identical results to every instance
    computing it itself; a given start (V0) bypasses it."""
    import bench

    path = os.path.join(GOLDEN, "c2_base.cdf")
    g = gb.read_grid(path)
    base = g.buses()
    Pl, Ql, Pg = bench.scenarios(np, base, 4096, bench.BASE_SEED + 7)
    pick = list(range(40)) + [1943, 2749, 3628, 4084]
    Pl, Ql, Pg = Pl[pick].ravel(), Ql[pick].ravel(), Pg[pick].ravel()
    n = len(pick)
    out = []
    for flat in (1, 0):
        b = gb.Batch([g], precision=precision, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
        b.set_plan(flat_shared=flat)
        b.set_instances(np.zeros(n, np.int32), Pload=Pl, Qload=Ql, Pg=Pg)
        b.solve()
        r = b.results()
        r["events"] = [b.events(i) for i in range(n)]
        out.append(r)
    for k in ("iterations", "status", "final_mismatch", "V", "theta", "Pcalc", "Qcalc", "events"):
        if k == "events":
            assert out[0][k] == out[1][k]
        else:
            np.testing.assert_array_equal(out[0][k], out[1][k], err_msg=k)


def test_two_batches_in_flight(gb):
    """gbpf_batch_launch on two batches (own streams, overlapping on the GPU)
    gives each batch the results of a plain solve; time_pipelined runs."""
    path = os.path.join(GOLDEN, "c2_s8.cdf")
    g = gb.read_grid(path)
    base = g.buses()
    rng = np.random.default_rng(21)
    n = 256
    lf = np.exp(rng.normal(0, 0.1, (n, g.nB)))
    Pl, Ql = (base["Pload"] * lf).ravel(), (base["Qload"] * lf).ravel()
    gi = np.zeros(n, np.int32)
    ref = gb.Batch([g], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    ref.set_instances(gi, Pload=Pl, Qload=Ql)
    ref.solve()
    want = ref.results()
    pair = [gb.Batch([g], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1) for _ in range(2)]
    for b in pair:
        b.set_instances(gi, Pload=Pl, Qload=Ql)
    for _ in range(3):
        for b in pair:
            b.launch()
    for b in pair:
        b.wait()
        got = b.results()
        for k in ("iterations", "status", "V", "theta"):
            np.testing.assert_array_equal(got[k], want[k], err_msg=k)
    assert gb.time_pipelined(pair, 4) > 0


def test_block_mode_shared_flat_start(gb, oracle):
    """Thread-block instances take the shared iteration 0 too (a two-pass
    factor made once per topology, the blocks' own iterations after it):
    the oracle's FP64 answers with and without it."""
    path = os.path.join(GOLDEN, "c2_s3.cdf")
    og = oracle.Grid(path)
    n = 24
    Pl, Ql, Pg = scenarios(og, n, 13)
    for flat in (1, 0):
        b = gb.Batch([gb.read_grid(path)], tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
        b.set_plan(warp_mode=0, flat_shared=flat)
        b.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        b.solve()
        r = b.results()
        assert b.plan()["block_instances"] == n
        for i in range(n):
            ref = oracle_solve(og, Pl[i], Ql[i], Pg[i], 1)
            assert r["iterations"][i] == ref["iterations"] and b.events(i) == ref["events"][:16], (flat, i)
            if ref["converged"]:
                assert np.max(np.abs(b.slice(r["V"], i) - ref["V"])) < 1e-9


@pytest.mark.parametrize("prec", ["PREC_FP64", "PREC_FP32_IR"])
def test_block_state_in_global_memory_is_exact(gb, prec):
    """Thread-block instances with part of their state in global memory (plan
    gstate 2: the own-bus arrays; gstate 3: every per-bus array but the flags
    and y, z; gstate 4: that, compiled for four blocks per SM; the default
    picks the level with the most instances per SM, e.g. level 3 for a 1,888-bus
    grid) do the same arithmetic as with all of it in shared memory:
    iterations, statuses, switch events, |V| and theta bit for bit, for a grid
    whose factor is in shared memory and one whose factor is in global
    scratch."""
    import bench

    for grid in (gb.read_grid(os.path.join(GOLDEN, "c2_s3.cdf")), gb.generate(3, bench.BASE_SEED + 5, tiles=16)):
        base = grid.buses()
        rng = np.random.default_rng(8)
        n = 40
        lf = rng.uniform(0.7, 1.3, (n, grid.nB))
        Pl, Ql = base["Pload"] * lf, base["Qload"] * lf
        Pg = base["Pg"] * rng.uniform(0.85, 1.15, (n, grid.nB))
        out = []
        for gstate, level in ((0, 0), (2, 1), (3, 2), (4, 3)):
            b = gb.Batch([grid], precision=getattr(gb, prec), tolerancia=1e-8, no_max_iter=30, lim_inj_reat=1)
            b.set_plan(warp_mode=0, gstate=gstate)
            b.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
            b.solve()
            assert b.plan()["block_state_global"] == level
            out.append((b.results(), [b.events(i) for i in range(n)], b.info()))
        r0, e0, i0 = out[0]
        assert (r0["status"] == 0).mean() > 0.9
        for r1, e1, i1 in out[1:]:
            for k in ("iterations", "status", "n_events", "V", "theta", "Pcalc", "Qcalc", "final_mismatch"):
                np.testing.assert_array_equal(r1[k], r0[k], err_msg=k)
            assert e1 == e0
        assert out[2][2]["smem_bytes"] < out[1][2]["smem_bytes"] < i0["smem_bytes"]
        assert out[2][2]["factors_in_smem"] >= i0["factors_in_smem"]
        assert out[3][2]["blocks"] >= out[2][2]["blocks"]


@pytest.mark.parametrize("prec", ["PREC_FP64", "PREC_FP32_IR"])
def test_warp_state_in_global_memory_is_exact(gb, prec):
    """The warp kernel with its state placed in global memory (plan
    warp_gstate 2, 3, 4: levels 1, 2 and 3, the last at 64 registers a
    thread) gives what it gives with all of it in shared memory, bit for bit,
    stragglers handed to blocks included."""
    path = os.path.join(GOLDEN, "c2_s3.cdf")
    grid = gb.read_grid(path)
    base = grid.buses()
    rng = np.random.default_rng(9)
    n = 96
    lf = rng.uniform(0.8, 1.2, (n, grid.nB))
    Pl, Ql = base["Pload"] * lf, base["Qload"] * lf
    Pg = base["Pg"] * rng.uniform(0.9, 1.1, (n, grid.nB))
    out = []
    for wg, level in ((0, 0), (2, 1), (3, 2), (4, 3)):
        b = gb.Batch([grid], precision=getattr(gb, prec), tolerancia=1e-8, no_max_iter=30, lim_inj_reat=1)
        b.set_plan(warp_gstate=wg, handoff_it=6)
        b.set_instances(np.zeros(n, np.int32), Pload=Pl.ravel(), Qload=Ql.ravel(), Pg=Pg.ravel())
        b.solve()
        pl = b.plan()
        assert pl["warp_state_global"] == level and pl["warp_instances"] == n
        out.append((b.results(), [b.events(i) for i in range(n)]))
    r0, e0 = out[0]
    assert (r0["status"] == 0).mean() > 0.8 and (r0["iterations"] > 6).any()
    for r1, e1 in out[1:]:
        for k in ("iterations", "status", "n_events", "V", "theta", "Pcalc", "Qcalc", "final_mismatch"):
            np.testing.assert_array_equal(r1[k], r0[k], err_msg=k)
        assert e1 == e0


@pytest.mark.parametrize("workload,n", [("c2", 4096), ("c5", 1024)])
def test_fp32_bench_scenarios_against_fp64(gb, workload, n):
    """The bench's FP32-LU answers against batched FP64, scenario by scenario
    (bench.fp64_check: both converge, same switch path -- bus, PV position and
    code of every PV<->PQ switch -- and |V|, theta within 1e-6).  c2 (the
    118-bus grid with reactive limits): at most 0.2 % of the FP64-converged
    scenarios left out; c5 (1,888 buses, limits off): none.  The counted ones
    are within 1e-7."""
    import bench  # the repository root is on sys.path (conftest)
    grid = gb.read_grid(bench.grid_file(bench.workload_files(workload)[0]))
    draw = bench.scenarios if workload == "c2" else bench.c5_scenarios
    Pl, Ql, Pg = (x.ravel() for x in draw(np, grid.buses(), n, bench.draw_seed(workload, 0)))
    lim, maxit = (1, 100) if workload == "c2" else (0, 30)
    res = {}
    for prec in ("PREC_FP32_IR", "PREC_FP64"):
        b = gb.Batch([grid], tolerancia=1e-8, no_max_iter=maxit, lim_inj_reat=lim, precision=getattr(gb, prec))
        b.set_instances(np.zeros(n, np.int32), Pload=Pl, Qload=Ql, Pg=Pg)
        b.solve()
        res[prec] = (b, b.results(state=True))
    (b32, r32), (b64, r64) = res["PREC_FP32_IR"], res["PREC_FP64"]
    ok, rec = bench.fp64_check(np, b32, r32, b64, r64, b32.offsets)
    assert rec["compared"] == n
    left_out = rec["fp64_converged"] - rec["counted"]
    assert left_out <= (0.002 * n if workload == "c2" else 0), rec
    assert rec["max_abs_err_vs_fp64"]["V"] < 1e-7 and rec["max_abs_err_vs_fp64"]["theta"] < 1e-7, rec
    assert np.all(r32["final_mismatch"][ok] <= 1e-8)
