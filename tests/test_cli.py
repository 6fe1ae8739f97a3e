"""The gbpf command-line driver as a process-level drop-in for the reference's
GPU executable: data.txt in the working directory, the option echo, the
method banner, the reactive-limit lines, the max(g) trace and the per-bus
table of impressao2 (GPU/impressao.h:47-80)."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

pytestmark = pytest.mark.gpu

EVENT_TEXT = {1: "PV -> PQ (limite superior)", 2: "PQ (limite inferior) -> PQ (limite superior)",
              3: "PV -> PQ (limite inferior)", 4: "PQ (limite superior) -> PQ (limite inferior)", 5: "PQ -> PV"}

DATA = """metodo         = {metodo};
openmp         = OFF;
v_inicial      = 1.0;
theta_inicial  = 0.0;
tolerancia     = 0.00000001;
no_max_iter    = 100;
arq_entrada    = {cdf};
laconic_mode   = OFF;
output_bench   = SCREEN;
output_ans     = ON;
lim_inj_reat   = ON;
output_iter    = ON;
"""


@pytest.mark.parametrize("metodo,banner", [("esparso", "[ESPARSO]"), ("hibridoC", "[HIBRIDO C]")])
def test_cli_output_matches_reference(gb, tmp_path, metodo, banner):
    cdf = "c2_s3.cdf"
    gold = load_golden("c2_s3_lim1.json")
    shutil.copy(os.path.join(GOLDEN, cdf), tmp_path / cdf)
    (tmp_path / "data.txt").write_text(DATA.format(metodo=metodo, cdf=cdf))
    out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    text = out.stdout
    lines = text.splitlines()
    assert lines[0] == f"metodo         = {metodo}"
    assert banner in lines
    # limit lines, in the order chkLimQ prints them
    barra = [l for l in lines if l.startswith("Barra ")]
    expect = [f"Barra {b} [{i}]: {EVENT_TEXT[c]}" for (_, b, i, c) in gold["events"]]
    assert barra == expect
    # one max(g) line per tested state
    mg = [l for l in lines if l.startswith("max(g) = ")]
    assert len(mg) == gold["iterations"] + 1
    # per-bus table
    start = lines.index("                                 FLUXOS DE POTENCIA")
    rows = [l for l in lines[start + 2:] if len(l) > 80 and l[6:10].strip().isdigit()]
    assert len(rows) == gold["nB"]
    V = np.array([float(r[10:21]) for r in rows])
    th = np.array([float(r[21:32]) for r in rows])
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 6e-6
    assert np.max(np.abs(th - np.array(gold["theta"]))) <= 6e-6


def test_cli_missing_data_txt(gb, tmp_path):
    out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=60)
    assert out.returncode != 0
    assert "ERRO: A ABERTURA DO ARQUIVO FALHOU!" in out.stdout
