"""Parity of the GPU solve path with the oracle and with the golden vectors
produced by the reference's own code.  Every call goes through the C ABI
(libgbpf.so) and runs the sm_103a kernels.

Tolerances: |V|, theta within 1e-9 of the reference and the oracle (FP64 parity
target); iteration counts and PV/PQ switch events identical; final max|g| <=
tolerancia; kernel-level values (Ybus, P/Q, Jacobian) within 1e-12 relative,
Newton steps within 1e-9 relative (different LU orderings, same mathematics).
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN, case_path, committed_cases, ieee_cases, ieee_path, load_golden

pytestmark = pytest.mark.gpu

STATE_TOL = 1e-9


def solver(gb, path_or_grid, **opts):
    grid = gb.read_grid(path_or_grid) if isinstance(path_or_grid, str) else path_or_grid
    base = dict(tolerancia=1e-8, no_max_iter=100, lim_inj_reat=0, metodo=0)
    base.update(opts)
    return grid, gb.Solver(grid, **base)


def states(oracle_grid, n=3, seed=0):
    """Flat start, a perturbed state and a solved state of a grid."""
    rng = np.random.default_rng(seed)
    V0, th0 = oracle_grid.V0.copy(), oracle_grid.theta0.copy()
    out = [(V0, th0)]
    out.append((V0 * (1 + 0.03 * rng.standard_normal(len(V0))), th0 + 0.2 * rng.standard_normal(len(V0))))
    r = oracle_grid.solve(1e-8, 50, False)
    out.append((r["V"], r["theta"]))
    return out[:n]


# the .m files take calcYbusSp_Matpower's stamps (GPU/main.cu:78-81)
CDFS = ["c1.cdf", "c2_base.cdf", "c2_s3.cdf", "m_edge.m", "c2_tx.m"]


@pytest.mark.parametrize("name", CDFS)
def test_ybus_matches_oracle(gb, oracle, name):
    path = os.path.join(GOLDEN, name)
    grid, s = solver(gb, path)
    rp, col, re, im = s.ybus()
    orp, ocol, ore, oim = oracle.Grid(path).ybus()
    np.testing.assert_array_equal(rp, orp)
    np.testing.assert_array_equal(col, ocol)
    scale = np.max(np.abs(ore + 1j * oim))
    assert np.max(np.abs(re - ore)) <= 1e-13 * scale
    assert np.max(np.abs(im - oim)) <= 1e-13 * scale


@pytest.mark.parametrize("name", CDFS)
def test_injections_match_oracle(gb, oracle, name):
    path = os.path.join(GOLDEN, name)
    grid, s = solver(gb, path)
    og = oracle.Grid(path)
    for V, th in states(og):
        P, Q = s.eval_pq(V, th)
        oP, oQ = og.injections(V, th)
        scale = max(1.0, np.max(np.abs(oP)), np.max(np.abs(oQ)))
        assert np.max(np.abs(P - oP)) <= 1e-12 * scale
        assert np.max(np.abs(Q - oQ)) <= 1e-12 * scale


def _dense(rows, cols, vals, n):
    A = np.zeros((n, n))
    np.add.at(A, (rows, cols), vals)
    return A


@pytest.mark.parametrize("name", CDFS)
def test_jacobian_matches_oracle(gb, oracle, name):
    path = os.path.join(GOLDEN, name)
    grid, s = solver(gb, path)
    og = oracle.Grid(path)
    rng = np.random.default_rng(1)
    for V, th in states(og):
        for trial in range(2):
            limQ = np.zeros(og.nPV, np.int32) if trial == 0 else (rng.random(og.nPV) < 0.3).astype(np.int32)
            pqlim = np.sort(np.concatenate([og.pq, og.pv[limQ == 1]])).astype(np.int32)
            n = og.nB - 1 + len(pqlim)
            r, c, v = s.eval_jacobian(V, th, limQ)
            orp, ocol, oval = og.jacobian(V, th, pqlim)
            orow = np.repeat(np.arange(n), np.diff(orp))
            A = _dense(r, c, v, n)
            B = _dense(orow, ocol, oval, n)
            # same pattern (the reference's entries) and values
            assert set(zip(r.tolist(), c.tolist())) == set(zip(orow.tolist(), ocol.tolist()))
            assert np.max(np.abs(A - B)) <= 1e-12 * max(1.0, np.max(np.abs(B)))


@pytest.mark.parametrize("name", CDFS)
def test_newton_step_matches_oracle(gb, oracle, name):
    path = os.path.join(GOLDEN, name)
    grid, s = solver(gb, path)
    og = oracle.Grid(path)
    rng = np.random.default_rng(2)
    for V, th in states(og, n=2):
        limQ = (rng.random(og.nPV) < 0.25).astype(np.int32)
        pqlim = np.sort(np.concatenate([og.pq, og.pv[limQ == 1]])).astype(np.int32)
        orp, ocol, oval = og.jacobian(V, th, pqlim)
        g = rng.standard_normal(len(orp) - 1)
        dx = s.newton_step(V, th, g, limQ)
        ref = oracle.sparse_solve(orp, ocol, oval, g)
        assert np.max(np.abs(dx - ref)) <= 1e-9 * max(1.0, np.max(np.abs(ref)))


def check_solution(res, gold):
    assert res["iterations"] == gold["iterations"]
    assert res["converged"] == bool(gold["converged"])
    ev = [list(e) for e in res["events"]]
    assert ev[:len(gold["events"])] == gold["events"]
    if gold["converged"]:
        assert len(ev) == len(gold["events"])
        assert res["final_mismatch"] <= gold["tol"]
        assert np.max(np.abs(res["V"] - np.array(gold["V"]))) < STATE_TOL
        assert np.max(np.abs(res["theta"] - np.array(gold["theta"]))) < STATE_TOL
        for k in ("Pcalc", "Qcalc", "Pdp", "Ppd", "Qdp", "Qpd"):
            assert np.max(np.abs(res[k] - np.array(gold[k]))) < 1e-7, k


@pytest.mark.parametrize("form", ["graph", "persistent"])
@pytest.mark.parametrize("case", committed_cases() + ieee_cases(), ids=lambda c: c["golden"])
def test_solve_matches_reference_golden(gb, case, form):
    """Synthetic grids and the reference's own IEEE inputs (ieee14 ... the
    7,552-bus ieee118x64, with and without reactive limits, including the
    100-iteration PV/PQ cycle of ieee118x4 with limits), in both forms of
    gbpf_solve: the graph of per-phase kernels and the one persistent launch
    (grids whose state fits a block's shared memory)."""
    grid, s = solver(gb, case_path(case), tolerancia=case["tol"],
                     no_max_iter=case["max_iter"], lim_inj_reat=case["lim"])
    if form == "graph":
        s.set_form(gb.FORM_GRAPH)
    elif s.form()["form"] != gb.FORM_PERSISTENT:
        pytest.skip("the grid's state does not fit one block's shared memory")
    gold = load_golden(case["golden"])
    res = s.solve()
    check_solution(res, gold)
    # max|g| per iteration; a non-converging PV/PQ cycle amplifies rounding
    # differences over its 100 iterations, so there only the first ten count
    h = np.array(gold["hist"])[:-1] if gold["converged"] else np.array(gold["hist"])[:10]
    np.testing.assert_allclose(res["hist"][:len(h)], h, rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("case", [c for c in committed_cases() + ieee_cases() if c["lim"] == 1],
                         ids=lambda c: c["golden"])
def test_fp32_lu_solve_against_reference_golden(gb, case):
    """The FP32-LU form (FP32 factor and substitutions, FP64 mismatch, test
    and update) on the same inputs: max|g| <= tol in FP64 and |V|, theta
    within 1e-6 of the reference's FP64 solution where it takes the FP64
    switch path; the switch path itself is reported, not required."""
    grid, s = solver(gb, case_path(case), tolerancia=case["tol"], no_max_iter=case["max_iter"],
                     lim_inj_reat=case["lim"], precision=gb.PREC_FP32_IR)
    gold = load_golden(case["golden"])
    res = s.solve()
    if not gold["converged"]:
        return
    assert res["converged"] and res["final_mismatch"] <= gold["tol"]
    if [list(e[1:]) for e in res["events"]] == [e[1:] for e in gold["events"]]:
        assert np.max(np.abs(res["V"] - np.array(gold["V"]))) < 1e-6
        assert np.max(np.abs(res["theta"] - np.array(gold["theta"]))) < 1e-6


def compare_with_oracle(gb, oracle, grid, path, lim, tol=1e-8, max_iter=60):
    s = gb.Solver(grid, tolerancia=tol, no_max_iter=max_iter, lim_inj_reat=lim, metodo=0)
    res = s.solve()
    ref = oracle.Grid(path).solve(tol, max_iter, bool(lim))
    assert ref["converged"]
    assert res["iterations"] == ref["iterations"]
    assert [tuple(e) for e in res["events"]] == ref["events"]
    assert res["final_mismatch"] <= tol
    assert np.max(np.abs(res["V"] - ref["V"])) < STATE_TOL
    assert np.max(np.abs(res["theta"] - ref["theta"])) < STATE_TOL
    return s, res


@pytest.mark.parametrize("nbus", [14, 30, 57, 118, 236, 472])
def test_scaled_grids_match_oracle(gb, oracle, tmp_path, nbus):
    for seed in (1, 2):
        g = gb.generate(4, 20261207 + 100 * seed + nbus, nbus=nbus)
        p = str(tmp_path / f"g{nbus}_{seed}.cdf")
        g.write_cdf(p)
        compare_with_oracle(gb, oracle, gb.read_grid(p), p, lim=1)


@pytest.mark.parametrize("tiles", [16, 128])
def test_tiled_grids_match_oracle(gb, oracle, tmp_path, tiles):
    g = gb.generate(3, 20261206 + tiles, tiles=tiles)
    p = str(tmp_path / ("t.cdfx" if g.nB > 9999 else "t.cdf"))
    g.write_cdf(p)
    s, res = compare_with_oracle(gb, oracle, gb.read_grid(p), p, lim=1)
    info = s.info()
    assert info["blocks"] == g.nB - 1 and info["forward_levels"] > 0


def test_repeated_solves_are_bitwise_identical(gb):
    grid, s = solver(gb, os.path.join(GOLDEN, "c2_s3.cdf"), lim_inj_reat=1)
    a = s.solve()
    b = s.solve()
    np.testing.assert_array_equal(a["V"], b["V"])
    np.testing.assert_array_equal(a["theta"], b["theta"])
    assert a["events"] == b["events"]


def test_set_start_and_scenario(gb, oracle):
    path = os.path.join(GOLDEN, "c2_base.cdf")
    grid, s = solver(gb, path)
    og = oracle.Grid(path)
    scale = np.linspace(0.8, 1.2, og.nB)
    Pl, Ql = og.Pload * scale, og.Qload * scale
    s.set_start(Pliq=og.Pg - Pl, Qliq=og.Qg - Ql)
    res = s.solve()
    og.set_bus(Pload=Pl, Qload=Ql)
    ref = og.solve(1e-8, 100, False)
    assert res["iterations"] == ref["iterations"]
    assert np.max(np.abs(res["V"] - ref["V"])) < STATE_TOL


def test_iteration_cap_reports_noconv(gb):
    grid, s = solver(gb, os.path.join(GOLDEN, "c2_base.cdf"), no_max_iter=1)
    res = s.solve(full=False)
    assert res["status"] == gb.E_NOCONV and not res["converged"] and res["iterations"] == 1


def test_singular_jacobian_is_reported(gb):
    # bus 3 has no branch and no shunt: its rows of the Jacobian are zero
    g = gb.create_grid(bus_type=[3, 0, 0], V0=[1.0, 1.0, 1.0], theta0=[0, 0, 0], from_bus=[1], to_bus=[2],
                       r=[0.01], x=[0.1], Pload=[0, 0.5, 0.1], Qload=[0, 0.1, 0.05])
    s = gb.Solver(g, tolerancia=1e-8, no_max_iter=10, metodo=0)
    res = s.solve(full=False)
    assert res["status"] == gb.E_SINGULAR and not res["converged"]


def test_fp32_lu_single_grid(gb, oracle, tmp_path):
    """precision = FP32: the single-grid solver factors and substitutes in FP32
    (fill, mismatch, test and update in FP64); Newton itself refines the FP32
    steps.  Converges to max|g| <= tolerancia with |V|, theta within 1e-6 of
    the FP64 oracle, on the 118-bus fixtures and a 1,888-bus tiled grid."""
    cases = [(os.path.join(GOLDEN, "c2_base.cdf"), 0), (os.path.join(GOLDEN, "c2_s3.cdf"), 1)]
    g = gb.generate(3, 20261211, tiles=16)
    p = str(tmp_path / "t16.cdf")
    g.write_cdf(p)
    cases.append((p, 1))
    for path, lim in cases:
        s = gb.Solver(gb.read_grid(path), tolerancia=1e-8, no_max_iter=50, lim_inj_reat=lim, metodo=0,
                      precision=gb.PREC_FP32_IR)
        res = s.solve()
        ref = oracle.Grid(path).solve(1e-8, 50, bool(lim))
        assert res["converged"] and res["final_mismatch"] <= 1e-8, path
        if [e[1:] for e in res["events"]] == [e[1:] for e in ref["events"]]:
            assert np.max(np.abs(res["V"] - ref["V"])) < 1e-6, path
            assert np.max(np.abs(res["theta"] - ref["theta"])) < 1e-6, path
        assert res["iterations"] <= ref["iterations"] + 3


@pytest.mark.parametrize("prec", ["PREC_FP64", "PREC_FP32_IR"])
def test_lu_launch_forms_agree(gb, prec):
    """The LU and triangular solves launched one kernel per level and all in
    one single-block kernel (k_lu_fused) run the same per-step code (levels
    with long gather lists take a block per step in the per-level form, which
    sums in another order): same iterations and events, state within 1e-12,
    on a switching 118-bus grid and the 1,888-bus tiled grid."""
    import bench

    grids = [gb.read_grid(os.path.join(GOLDEN, "c2_s3.cdf")), gb.generate(3, bench.BASE_SEED + 5, tiles=16)]
    for g in grids:
        out = []
        for mode in (1, 2):
            s = gb.Solver(g, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1, metodo=0,
                          precision=getattr(gb, prec))
            s.set_lu_launch(mode)
            info = s.info()
            assert (info["kernels_per_iteration"] < info["forward_levels"]) == (mode == 2)
            out.append(s.solve())
        a, b = out
        assert a["iterations"] == b["iterations"] and a["events"] == b["events"]
        for k in ("V", "theta", "Pcalc", "Qcalc"):
            np.testing.assert_allclose(a[k], b[k], rtol=0, atol=1e-12, err_msg=k)


@pytest.mark.parametrize("precision,lim", [("PREC_FP64", 1), ("PREC_FP32_IR", 0)])
def test_persistent_form_equals_graph_form(gb, precision, lim):
    """The default FP64 form of a small grid is the persistent launch; on a
    grid that switches PV buses it gives what the graph form gives:
    iterations, events, max|g| per iteration, the limit-check iterations,
    state and flows (to rounding: the two sum the LU updates in different
    orders), also after set_start moves the start away from the grid's own
    and back.  The FP32-LU form (graph by default; persistent on request)
    without reactive limits: both within 1e-6 of each other."""
    path = os.path.join(GOLDEN, "c2_s8.cdf")
    grid = gb.read_grid(path)
    opts = dict(tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=0, precision=getattr(gb, precision))
    p, g = gb.Solver(grid, **opts), gb.Solver(grid, **opts)
    if precision == "PREC_FP64":
        assert p.form()["form"] == gb.FORM_PERSISTENT and p.form()["launches"] == 2
    else:
        assert p.form()["form"] == gb.FORM_GRAPH
        p.set_form(gb.FORM_PERSISTENT)
    g.set_form(gb.FORM_GRAPH)
    b = grid.buses()
    rng = np.random.default_rng(4)
    starts = [None, (b["V0"] * (1 + 0.01 * rng.standard_normal(grid.nB)), b["theta0"] + 0.05 * rng.standard_normal(grid.nB)),
              (b["V0"], b["theta0"])]
    tol = 1e-12 if precision == "PREC_FP64" else 1e-6
    for st in starts:
        if st is not None:
            for x in (p, g):
                x.set_start(V0=st[0], theta0=st[1])
        rp, rg = p.solve(), g.solve()
        assert rp["converged"] and rg["converged"]
        assert [e[1:] for e in rp["events"]] == [e[1:] for e in rg["events"]]
        assert rp["nPQlim"] == rg["nPQlim"]
        if st is None and lim:
            assert len(rp["events"]) > 0
        if precision == "PREC_FP64":
            assert rp["iterations"] == rg["iterations"] and rp["events"] == rg["events"]
            np.testing.assert_array_equal(p.triggers(), g.triggers())
            np.testing.assert_allclose(rp["hist"], rg["hist"], rtol=1e-6, atol=1e-12)
        for k in ("V", "theta"):
            assert np.max(np.abs(rp[k] - rg[k])) < tol, k
        for k in ("Pcalc", "Qcalc", "Pdp", "Ppd", "Qdp", "Qpd"):
            assert np.max(np.abs(rp[k] - rg[k])) < 1e3 * tol, k


def test_form_selection(gb):
    """The persistent form is offered where the grid's state fits one block's
    shared memory: not for the 7,552-bus ieee118x64, never for metodo = denso."""
    case = next(c for c in ieee_cases() if c["cdf"] == "ieee118x64.cdf")
    big = gb.Solver(gb.read_grid(ieee_path(case)), tolerancia=1e-8, no_max_iter=100, metodo=0)
    assert big.form()["form"] == gb.FORM_GRAPH
    with pytest.raises(gb.GbpfError) as e:
        big.set_form(gb.FORM_PERSISTENT)
    assert e.value.status == gb.E_UNSUPPORTED
    dense = gb.Solver(gb.read_grid(os.path.join(GOLDEN, "c1.cdf")), tolerancia=1e-8, no_max_iter=100, metodo=1)
    assert dense.form()["form"] == gb.FORM_GRAPH


@pytest.mark.parametrize("precision", ["PREC_FP64", "PREC_FP32_IR"])
@pytest.mark.parametrize("name,lim", [("c4_472.cdf.gz", 1), ("c3_base.cdfx.gz", 1)])
def test_split_heavy_levels_equal_block_per_step(gb, precision, name, lim):
    """The graph form's heavy elimination levels as two launches (pivots, then
    every off-diagonal entry on its own warp) give the same factor as one
    block per step walking its entries: bit-identical solves."""
    import bench
    grid = gb.read_grid(bench.grid_file(name))
    out = []
    for mode in (1, 3):
        s = gb.Solver(grid, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=lim, metodo=0,
                      precision=getattr(gb, precision))
        s.set_form(gb.FORM_GRAPH)
        s.set_lu_launch(mode)
        out.append(s.solve())
        s.close()
    a, b = out
    assert a["converged"] and a["iterations"] == b["iterations"] and a["events"] == b["events"]
    np.testing.assert_array_equal(a["V"], b["V"])
    np.testing.assert_array_equal(a["theta"], b["theta"])


@pytest.mark.parametrize("plan", [(1, 0, 1), (1, 0, 0), (1, 1, 1), (0, 0, 1), (0, 1, 0)],
                         ids=lambda p: f"lu1={p[0]},narrow={p[1]},quad={p[2]}")
@pytest.mark.parametrize("case", [c for c in committed_cases() + ieee_cases(max_buses=1888)
                                  if c["golden"] in ("c2_s3_lim1.json", "c1_lim1.json", "ieee_ieee118_lim1.json",
                                                     "ieee_ieee118x4_lim0.json", "ieee_ieee118x16_lim0.json.gz")],
                         ids=lambda c: c["golden"])
def test_persistent_plans_match_reference_golden(gb, case, plan):
    """gbpf_solver_set_plan: every LU plan of the persistent form (one- or
    two-pass levels, one-warp narrow levels or not, FP64 blocks on four lanes
    or one) holds the reference-built golden -- identical iterations and
    switch events, |V| and theta within 1e-9 -- and reports the plan it set."""
    grid, s = solver(gb, case_path(case), tolerancia=case["tol"], no_max_iter=case["max_iter"],
                     lim_inj_reat=case["lim"])
    if s.form()["form"] != gb.FORM_PERSISTENT:
        pytest.skip("the grid's state does not fit one block's shared memory")
    want = dict(lu1=plan[0], narrow=plan[1], quad=plan[2])
    assert s.set_plan(*plan) == want
    assert s.set_plan() == want
    check_solution(s.solve(), load_golden(case["golden"]))
