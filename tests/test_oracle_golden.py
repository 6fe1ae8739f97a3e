"""The CPU oracle against the golden vectors produced by the reference's own
solve-path code (oracle/_ref/ref_nr, see tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from conftest import GOLDEN, REFERENCE_GPU, committed_cases, ieee_cases, ieee_path, load_golden

STATE_TOL = 1e-9  # |V| and theta, from the parity target


def check(res, gold):
    assert res["iterations"] == gold["iterations"]
    assert res["converged"] == bool(gold["converged"])
    assert [list(e) for e in res["events"]][:len(gold["events"])] == gold["events"]
    if gold["converged"]:
        assert len(res["events"]) == len(gold["events"])
        assert res["final_mismatch"] <= gold["tol"]
        for k in ("V", "theta"):
            assert np.max(np.abs(res[k] - np.array(gold[k]))) < STATE_TOL, k
        for k in ("Pcalc", "Qcalc", "Pdp", "Ppd", "Qdp", "Qpd"):
            assert np.max(np.abs(res[k] - np.array(gold[k]))) < 1e-8, k
        h = np.array(gold["hist"])
        np.testing.assert_allclose(res["hist"][:len(h) - 1], h[:-1], rtol=1e-6, atol=1e-12)


@pytest.mark.parametrize("case", committed_cases(), ids=lambda c: c["golden"])
def test_oracle_matches_reference_on_synthetic(oracle, case):
    g = oracle.Grid(os.path.join(GOLDEN, case["cdf"]))
    check(g.solve(case["tol"], case["max_iter"], case["lim"]), load_golden(case["golden"]))


@pytest.mark.parametrize("case", ieee_cases(), ids=lambda c: c["golden"])
def test_oracle_matches_reference_on_ieee(oracle, case):
    g = oracle.Grid(ieee_path(case))
    check(g.solve(case["tol"], case["max_iter"], case["lim"]), load_golden(case["golden"]))


@pytest.mark.parametrize("case", [c for c in ieee_cases() if c["lim"] == 0], ids=lambda c: c["cdf"])
def test_ieee_fixture_is_the_reference_file(case):
    """The committed fixture holds the reference's input byte for byte."""
    src = os.path.join(REFERENCE_GPU, case["cdf"])
    if not os.path.exists(src):
        pytest.skip("reference checkout not present")
    with open(src, "rb") as f, open(ieee_path(case), "rb") as g:
        assert f.read() == g.read()


def test_switch_cases_are_covered():
    """The fixtures include PV->PQ switching and a non-converging switch cycle."""
    idx = committed_cases() + ieee_cases()
    assert sum(1 for c in idx if c["events"] > 0) >= 4
    assert any(c["iterations"] == c["max_iter"] for c in idx)


def test_oracle_sparse_solve_residual(oracle):
    g = oracle.Grid(os.path.join(GOLDEN, "c2_base.cdf"))
    rp, col, val = g.jacobian(g.V0, g.theta0)
    n = len(rp) - 1
    b = np.linspace(-1, 1, n)
    x = oracle.sparse_solve(rp, col, val, b)
    A = np.zeros((n, n))
    for r in range(n):
        A[r, col[rp[r]:rp[r + 1]]] = val[rp[r]:rp[r + 1]]
    assert np.max(np.abs(A @ x - b)) < 1e-10
    np.testing.assert_allclose(x, np.linalg.solve(A, b), rtol=1e-9, atol=1e-11)
