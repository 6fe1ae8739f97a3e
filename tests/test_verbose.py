"""verbose_mode = ON: the per-iteration dumps of the reference's Newton loop
(GPU/newtonRaphson.cuh:150-156,270-272,284-286,392-427,433-450,539-563;
GPU/Jacobiano.cuh:216-220,382-410; GPU/PQcalc.cuh:304-320,417-432 for denso).

The oracle writes the transcript from its own solve (`pforacle --verbose`);
the CPU tests hold that transcript to the reference-built goldens (banners,
limit lines, max(g) per iteration).  The GPU tests run the gbpf driver with
verbose_mode = ON -- gbpf_solve_traced, the graph form's kernels stage by
stage -- and compare its transcript with the oracle's line by line: the same
text, and every printed number equal up to one unit in its last printed
digit (values agree to ~1e-12; a printed digit can still round the other way),
max(g) in %e within 1e-6 relative or 1e-9 absolute."""
import os
import re
import shutil
import subprocess

import pytest

from conftest import GOLDEN, ROOT, load_golden

ORACLE_CLI = os.path.join(ROOT, "oracle", "_build", "pforacle")
NUM = re.compile(r"[-+]?\d+\.\d+(?:e[-+]\d+)?|[-+]?\d+")
BANNER = "****************************************************************** ITERACAO"

DATA = """metodo         = {metodo};
openmp         = OFF;
v_inicial      = 1.0;
theta_inicial  = 0.0;
tolerancia     = 0.00000001;
no_max_iter    = {maxit};
arq_entrada    = {cdf};
laconic_mode   = OFF;
output_bench   = OFF;
output_ans     = ON;
lim_inj_reat   = ON;
output_iter    = ON;
verbose_mode   = ON;
"""


def oracle_transcript(path, dense=False, maxit=100):
    if not os.path.exists(ORACLE_CLI):
        subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], check=True)
    cmd = [ORACLE_CLI, path, "--lim", "1", "--maxit", str(maxit), "--verbose"] + (["--dense"] if dense else [])
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    return out.stdout


def same_transcript(a, b):
    """Line-by-line comparison: identical text between the numbers, each number
    within one unit of its last printed digit (%e values: 1e-6 relative or
    1e-9 absolute)."""
    la, lb = a.splitlines(), b.splitlines()
    assert len(la) == len(lb), (len(la), len(lb))
    for i, (x, y) in enumerate(zip(la, lb)):
        if x == y:
            continue
        assert NUM.split(x) == NUM.split(y), (i, x, y)
        for p, q in zip(NUM.findall(x), NUM.findall(y)):
            if p == q:
                continue
            fp, fq = float(p), float(q)
            if "e" in p:
                tol = 1e-9 + 1e-6 * abs(fq)
            elif "." in p:
                tol = 1.01 * 10.0 ** -len(p.split(".")[1].split("e")[0])
            else:
                tol = 0.0
            assert abs(fp - fq) <= tol, (i, x, y)


def test_oracle_transcript_follows_the_golden_solve():
    """The oracle's transcript of the switching 14-bus case: one banner per
    tested state, printAlLim first, the limit lines of every check, max(g) of
    every iteration as in the reference-built golden, break! at the end."""
    gold = load_golden("c1_lim1.json")
    text = oracle_transcript(os.path.join(GOLDEN, "c1.cdf"))
    lines = text.splitlines()
    assert lines[0] == "nPQlim = 9" and lines[1] == "nPVlim = 4"
    banners = [l for l in lines if l.startswith(BANNER)]
    assert len(banners) == gold["iterations"] + 1
    assert banners[-1].split()[2] == str(gold["iterations"])
    barra = [l for l in lines if l.startswith("Barra ")]
    assert len(barra) == len(gold["events"])
    for l, (_, b, i, _) in zip(barra, gold["events"]):
        assert l.startswith(f"Barra {b} [{i}]: ")
    mg = [float(l.split("=")[1].split()[0]) for l in lines if l.startswith("max(g) = ")]
    # one per iteration, plus the repeat after break!
    assert len(mg) == gold["iterations"] + 2
    for a, b in zip(mg, gold["hist"]):
        assert abs(a - b) <= 1e-6 * abs(b) + 1e-12
    assert lines[-3] == "break!" and lines[-2].startswith("max(g) = ")
    # the value arrays: H, L, M, J per iteration, J the full fill
    for it in range(gold["iterations"]):
        for name in ("H", "L", "M", "J"):
            assert f"{name}^({it}) =" in lines


def test_oracle_dense_transcript_prints_the_dense_jacobian():
    gold = load_golden("c1_lim1.json")
    text = oracle_transcript(os.path.join(GOLDEN, "c1.cdf"), dense=True)
    lines = text.splitlines()
    assert sum(l == "JacobianoN =" for l in lines) == gold["iterations"]
    assert sum(l.startswith("P_1\t= ") for l in lines) == gold["iterations"] + 1
    first = lines.index("JacobianoN =")
    assert lines[first + 2].startswith("[")
    # dim = nB - 1 + nPQlim = 13 + 9 values a row at the first iteration
    assert len(lines[first + 2][1:].split()) == 22


@pytest.mark.gpu
@pytest.mark.parametrize("case,metodo,maxit", [("c1.cdf", "esparso", 100), ("m_edge.m", "esparso", 100),
                                               ("c1.cdf", "denso", 100), ("c2_s3.cdf", "esparso", 100),
                                               ("c1.cdf", "esparso", 3)])
def test_cli_verbose_matches_oracle(gb, tmp_path, case, metodo, maxit):
    shutil.copy(os.path.join(GOLDEN, case), tmp_path / case)
    (tmp_path / "data.txt").write_text(DATA.format(metodo=metodo, cdf=case, maxit=maxit))
    out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=300)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    assert "verbose_mode   = ON" in text.splitlines()
    start = text.index("nPQlim = ")
    end = text.index("\n\n                                 FLUXOS DE POTENCIA")
    mine = text[start:end]
    ref = oracle_transcript(os.path.join(GOLDEN, case), dense=metodo == "denso", maxit=maxit)
    same_transcript(mine, ref)
    # the per-bus table still follows
    assert "FLUXOS DE POTENCIA" in text[end:]


@pytest.mark.gpu
@pytest.mark.parametrize("case", ["c1.cdf", "c2_s3.cdf", "m_edge.m"])
def test_traced_solve_equals_graph_form(gb, case):
    """gbpf_solve_traced runs the graph form's kernels stage by stage: the
    same iterations, switch events, max(g) history and state bit for bit, one
    EVAL record per tested state (the last one converged, its max_g the
    history's last entry), and its Jacobian records equal gbpf_eval_jacobian at
    the same state."""
    import numpy as np

    grid = gb.read_grid(os.path.join(GOLDEN, case))
    s = gb.Solver(grid, tolerancia=1e-8, no_max_iter=100, lim_inj_reat=1)
    s.set_form(gb.FORM_GRAPH)
    a = s.solve()
    b = s.solve_traced()
    assert (a["iterations"], a["converged"], a["events"]) == (b["iterations"], b["converged"], b["events"])
    for k in ("V", "theta", "Pcalc", "Qcalc", "hist", "Pdp", "Qdp"):
        np.testing.assert_array_equal(a[k], b[k])
    ev = [r for r in b["trace"] if r["stage"] == gb.TRACE_EVAL]
    assert len(ev) == b["iterations"] + 1 and ev[-1]["converged"]
    np.testing.assert_array_equal([r["max_g"] for r in ev], b["hist"])
    assert sum(len(r["events"]) for r in ev) == len(b["events"])
    jac = [r for r in b["trace"] if r["stage"] == gb.TRACE_JACOBIAN]
    assert len(jac) == b["iterations"]
    for r in jac[:3]:
        limQ = r["limQ"].astype(np.int32)
        row, col, val = s.eval_jacobian(r["V"], r["theta"], limQ)
        order = np.lexsort((col, row))
        np.testing.assert_array_equal(row[order], r["jrow"])
        np.testing.assert_array_equal(col[order], r["jcol"])
        np.testing.assert_array_equal(val[order], r["jval"])
