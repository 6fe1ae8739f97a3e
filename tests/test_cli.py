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


def test_cli_benchmark_csv_and_report(gb, tmp_path):
    """benchmarksPrintFile / benchmarksPrint (GPU/impressao.h:125-558): the CSV
    out_double_esparso-<input>.csv with the reference's two header lines, one
    row per run numbered from 1, 17 ';'-separated fields with decimal commas;
    the screen report with the total time and the iteration count."""
    cdf = "c2_s3.cdf"
    gold = load_golden("c2_s3_lim1.json")
    shutil.copy(os.path.join(GOLDEN, cdf), tmp_path / cdf)
    (tmp_path / "data.txt").write_text(DATA.format(metodo="esparso", cdf=cdf).replace("SCREEN", "ALL"))
    for _ in range(2):
        out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=120)
        assert out.returncode == 0, out.stderr
    assert " Relatorio de execucao:" in out.stdout
    assert f" Numero de iteracoes: {gold['iterations']}." in out.stdout
    raw = (tmp_path / "out_double_esparso-c2_s3.csv").read_bytes()
    lines = raw.split(b"\n")
    assert lines[0] == (b"Execucao;Aviso;ms total;no iteracoes;ms Ybus;ms Init GPU;;;ms Inicializacao;ms calcPQ;;"
                        b"ms Jacobiano;;ms Sistema Linear;;ms Processo;ms Fluxo;")
    assert lines[1].startswith(b";;;;;total; Aloca\xef\xbf\xbd\xef\xbf\xbdo Vari\xef\xbf\xbdveis iniciais;")
    assert lines[-1] == b""
    rows = [l.decode() for l in lines[2:-1]]
    assert len(rows) == 2
    for k, row in enumerate(rows, start=1):
        f = row.split(";")
        assert len(f) == 18 and f[-1] == ""
        assert f[0] == str(k) and f[1] == ""
        assert f[3] == str(gold["iterations"])
        for x in f[2:3] + f[4:17]:
            assert "," in x and "." not in x
            assert float(x.replace(",", ".")) >= 0


def test_cli_matpower_input(gb, tmp_path):
    """arq_entrada naming a MATPOWER case: same lines and table as for the
    golden solve of the reference's own reader (m_edge.m, limits on: five
    switch events)."""
    m = "m_edge.m"
    gold = load_golden("m_edge_lim1.json")
    shutil.copy(os.path.join(GOLDEN, m), tmp_path / m)
    (tmp_path / "data.txt").write_text(DATA.format(metodo="esparso", cdf=m))
    out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    barra = [l for l in lines if l.startswith("Barra ")]
    assert barra == [f"Barra {b} [{i}]: {EVENT_TEXT[c]}" for (_, b, i, c) in gold["events"]]
    assert len([l for l in lines if l.startswith("max(g) = ")]) == gold["iterations"] + 1
    start = lines.index("                                 FLUXOS DE POTENCIA")
    rows = [l for l in lines[start + 2:] if len(l) > 80 and l[6:10].strip().isdigit()]
    assert len(rows) == gold["nB"]
    V = np.array([float(r[10:21]) for r in rows])
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 6e-6


def test_cli_fp32_lu_key(gb, tmp_path):
    """precisao = FP32 (the one added data.txt key) runs the single-grid
    solver's FP32-LU form: converged, same table within the print precision."""
    cdf = "c2_s3.cdf"
    gold = load_golden("c2_s3_lim1.json")
    shutil.copy(os.path.join(GOLDEN, cdf), tmp_path / cdf)
    (tmp_path / "data.txt").write_text(DATA.format(metodo="esparso", cdf=cdf) + "precisao       = FP32;\n")
    out = subprocess.run([gb.CLI_PATH], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stderr
    lines = out.stdout.splitlines()
    start = lines.index("                                 FLUXOS DE POTENCIA")
    rows = [l for l in lines[start + 2:] if len(l) > 80 and l[6:10].strip().isdigit()]
    V = np.array([float(r[10:21]) for r in rows])
    assert np.max(np.abs(V - np.array(gold["V"]))) <= 6e-6
