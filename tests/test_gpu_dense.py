"""metodo = denso on the GPU: the dense Jacobian, the LU with partial
pivoting and the triangular solves written here (in place of
GPU/Jacobiano.cuh:33-222 and the getrf/getrs calls of
GPU/newtonRaphson.cuh:507-530).  The dense Newton step equals the sparse one
up to rounding, so the same goldens and oracle comparisons hold: identical
iteration counts and switch events, |V| and theta within 1e-9, final max|g|
within the tolerance.  calcYbus's rule for off-diagonal entries (assigned
branch by branch) is checked on a grid with a reversed parallel branch,
against the oracle with the same rule."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, committed_cases, ieee_cases, ieee_path, load_golden
from test_gpu_parity import STATE_TOL, check_solution, solver

pytestmark = pytest.mark.gpu

DENSO = 1


# The .m goldens hold calcYbusSp_Matpower's solution; metodo = denso builds
# Ybus with calcYbus for every input (GPU/main.cu:73-76), checked below.
@pytest.mark.parametrize("case", [c for c in committed_cases() if not c["cdf"].endswith(".m")],
                         ids=lambda c: c["golden"])
def test_dense_solve_matches_reference_golden(gb, case):
    grid, s = solver(gb, os.path.join(GOLDEN, case["cdf"]), tolerancia=case["tol"],
                     no_max_iter=case["max_iter"], lim_inj_reat=case["lim"], metodo=DENSO)
    check_solution(s.solve(), load_golden(case["golden"]))


# The reference's IEEE inputs up to 1,888 buses (N = 3,774); their parallel
# branches all run in one direction, so calcYbus and calcYbusSp agree there.
@pytest.mark.parametrize("case", ieee_cases(max_buses=1888), ids=lambda c: c["golden"])
def test_dense_solve_matches_reference_golden_on_ieee(gb, case):
    grid, s = solver(gb, ieee_path(case), tolerancia=case["tol"], no_max_iter=case["max_iter"],
                     lim_inj_reat=case["lim"], metodo=DENSO)
    check_solution(s.solve(), load_golden(case["golden"]))


def _compare(gb, oracle, path, lim, dense_rule=True, max_iter=60):
    s = gb.Solver(gb.read_grid(path), tolerancia=1e-8, no_max_iter=max_iter, lim_inj_reat=lim, metodo=DENSO)
    res = s.solve()
    og = oracle.Grid(path)
    og.set_dense_ybus(dense_rule)
    ref = og.solve(1e-8, max_iter, bool(lim))
    assert ref["converged"]
    assert res["iterations"] == ref["iterations"]
    assert [tuple(e) for e in res["events"]] == ref["events"]
    assert res["final_mismatch"] <= 1e-8
    assert np.max(np.abs(res["V"] - ref["V"])) < STATE_TOL
    assert np.max(np.abs(res["theta"] - ref["theta"])) < STATE_TOL
    return res


@pytest.mark.parametrize("name,lim", [("m_edge.m", 0), ("m_edge.m", 1), ("c2_tx.m", 1)])
def test_dense_matpower_input_uses_calcybus(gb, oracle, name, lim):
    """A .m grid under metodo = denso: calcYbus's stamps and off-diagonal
    rule, not calcYbusSp_Matpower's."""
    _compare(gb, oracle, os.path.join(GOLDEN, name), lim)


@pytest.mark.parametrize("nbus", [14, 57, 118, 472])
def test_dense_scaled_grids_match_oracle(gb, oracle, tmp_path, nbus):
    g = gb.generate(4, 20261307 + nbus, nbus=nbus)
    p = str(tmp_path / f"g{nbus}.cdf")
    g.write_cdf(p)
    _compare(gb, oracle, p, lim=1)


def test_dense_1888_bus_grid_matches_oracle(gb, oracle, tmp_path):
    """N = 3,774: 118 panels, so the row interchanges, U12 solves and Schur
    updates between panels all take part."""
    g = gb.generate(3, 20261222, tiles=16)
    p = str(tmp_path / "t16.cdf")
    g.write_cdf(p)
    _compare(gb, oracle, p, lim=1)


def _reversed_branch_grid(gb, tmp_path):
    """c1 plus a second branch 2 -> 1 beside the file's 1 -> 2."""
    g = gb.read_grid(os.path.join(GOLDEN, "c1.cdf"))
    b, br = g.buses(), g.branches()
    pvpq = g.pvpq()
    Qmin, Qmax = np.zeros(g.nB), np.zeros(g.nB)
    Qmin[pvpq["pv"] - 1], Qmax[pvpq["pv"] - 1] = pvpq["Qmin"], pvpq["Qmax"]
    i = int(np.flatnonzero((br["from_bus"] == 1) | (br["to_bus"] == 1))[0])
    f, t = br["from_bus"], br["to_bus"]
    ext = lambda a, v: np.concatenate([a, [v]])
    g2 = gb.create_grid(b["type"], b["V0"], b["theta0"], ext(f, t[i]), ext(t, f[i]), ext(br["r"], 2 * br["r"][i]),
                        ext(br["x"], 2 * br["x"][i]), bch=ext(br["bch"], 0.0), tap_re=ext(br["tap_re"], 1.0),
                        tap_im=ext(br["tap_im"], 0.0), phase=ext(br["phase"], 0.0), Pload=b["Pload"],
                        Qload=b["Qload"], Pg=b["Pg"], Qg=b["Qg"], gsh=b["gsh"], bsh=b["bsh"], Qmax=Qmax,
                        Qmin=Qmin, id=b["id"])
    p = str(tmp_path / "rev.cdf")
    g2.write_cdf(p)
    return p


def test_dense_ybus_rule_with_reversed_branch(gb, oracle, tmp_path):
    p = _reversed_branch_grid(gb, tmp_path)
    dense = _compare(gb, oracle, p, lim=0, dense_rule=True)
    s = gb.Solver(gb.read_grid(p), tolerancia=1e-8, no_max_iter=60, lim_inj_reat=0, metodo=0)
    sparse = s.solve()
    ref = oracle.Grid(p).solve(1e-8, 60, False)
    assert np.max(np.abs(sparse["V"] - ref["V"])) < STATE_TOL
    # the two rules give different grids here
    assert np.max(np.abs(dense["V"] - sparse["V"])) > 1e-6


def test_dense_singular_jacobian_is_reported(gb):
    g = gb.create_grid(bus_type=[3, 0, 0], V0=[1.0, 1.0, 1.0], theta0=[0, 0, 0], from_bus=[1], to_bus=[2],
                       r=[0.01], x=[0.1], Pload=[0, 0.5, 0.1], Qload=[0, 0.1, 0.05])
    s = gb.Solver(g, tolerancia=1e-8, no_max_iter=10, metodo=DENSO)
    res = s.solve(full=False)
    assert res["status"] == gb.E_SINGULAR and not res["converged"]


def test_dense_rejects_grids_beyond_its_size(gb):
    g = gb.generate(3, 20261206, tiles=128)  # 15,104 buses: N = 30,206
    with pytest.raises(gb.GbpfError) as e:
        gb.Solver(g, tolerancia=1e-8, no_max_iter=10, metodo=DENSO)
    assert e.value.status == gb.E_UNSUPPORTED
