"""MATPOWER .m input without a GPU: the reader (lerArquivoMatPOWEReficiente +
storeMatPOWER, GPU/m.h:296-622) against the oracle's reader and against what
the reference's own reader made of the committed files (tests/golden/*.m,
expected values from oracle/_ref/ref_nr), the writer's round trip, the error
cases, and the oracle's calcYbusSp_Matpower Ybus (GPU/sistema.h:760-855)
against the reference's values."""
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN, load_golden

M_FILES = ["m_edge.m", "c2_tx.m"]


def _read_text(name):
    with open(os.path.join(GOLDEN, name), newline="") as f:
        return f.read()


def _write(tmp_path, name, text, newline="\n"):
    p = tmp_path / name
    with open(p, "w", newline=newline) as f:
        f.write(text)
    return str(p)


def _same_grid(a, b):
    assert (a.nB, a.nL, a.nPV, a.nPQ, a.slack) == (b.nB, b.nL, b.nPV, b.nPQ, b.slack)
    for x, y in ((a.buses(), b.buses()), (a.pvpq(), b.pvpq()), (a.branches(), b.branches())):
        for k in x:
            np.testing.assert_array_equal(x[k], y[k], err_msg=k)


@pytest.mark.parametrize("name", M_FILES)
def test_reader_matches_oracle_reader(gb, oracle, name):
    path = os.path.join(GOLDEN, name)
    g = gb.read_grid(path)
    o = oracle.Grid(path)
    assert g.ybus_form == gb.YBUS_MATPOWER and o.ybus_form == 1
    assert (g.nB, g.nL, g.nPV, g.nPQ, g.slack) == (o.nB, o.nL, o.nPV, o.nPQ, o.slack)
    b = g.buses()
    for k, ok in (("id", o.id), ("type", o.type), ("V0", o.V0), ("theta0", o.theta0), ("Pload", o.Pload),
                  ("Qload", o.Qload), ("Pg", o.Pg), ("Qg", o.Qg), ("gsh", o.gsh), ("bsh", o.bsh)):
        np.testing.assert_array_equal(b[k], ok, err_msg=k)
    p = g.pvpq()
    for k, ok in (("pv", o.pv), ("pq", o.pq), ("Qmin", o.Qmin), ("Qmax", o.Qmax), ("Vset", o.Vset)):
        np.testing.assert_array_equal(p[k], ok, err_msg=k)
    br = g.branches()
    for k, ok in (("from_bus", o.de), ("to_bus", o.para), ("r", o.z_re), ("x", o.z_im), ("bch", o.bsh_br),
                  ("tap_re", o.tap_re), ("tap_im", o.tap_im), ("phase", o.phi)):
        np.testing.assert_array_equal(br[k], ok, err_msg=k)


@pytest.mark.parametrize("name", M_FILES)
def test_reader_sizes_match_reference(gb, name):
    """Bus, branch, PV and PQ counts and the slack position the reference's
    reader reported for the same file."""
    g = gb.read_grid(os.path.join(GOLDEN, name))
    gold = load_golden(name.replace(".m", "_lim0.json"))
    assert (g.nB, g.nL, g.nPV, g.nPQ, g.slack) == (gold["nB"], gold["nL"], gold["nPV"], gold["nPQ"], gold["slack"])


def test_reader_corner_cases(gb):
    g = gb.read_grid(os.path.join(GOLDEN, "m_edge.m"))
    b, p, br = g.buses(), g.pvpq(), g.branches()
    np.testing.assert_array_equal(b["id"], [10, 20, 30, 40, 50, 60])
    np.testing.assert_array_equal(b["type"], [3, 2, 0, 0, 2, 0])  # MATPOWER PQ (1) is stored as the CDF's 0
    assert g.slack == 1 and b["V0"][0] == 1.02 and b["theta0"][0] == 5 * 3.14159265358979323846 / 180.
    assert b["V0"][2] == 1.0  # PQ buses start at v_inicial, not at Vm
    # the generator row of PQ bus 30 is never looked up
    assert b["Pg"][2] == 0 and b["Qg"][2] == 0
    # bus 50 has two generator rows: the first one is used
    assert b["Pg"][4] == 0.30 and p["Qmax"][1] == 0.25 and p["Qmin"][1] == -0.05
    # shunts in MW / MVAr at 1 p.u., divided by baseMVA
    assert b["gsh"][5] == 0.02 and b["bsh"][5] == -0.05 and b["bsh"][3] == 0.19
    # the repeated 10-20 branch is kept as two branches
    assert g.nL == 8
    np.testing.assert_array_equal(br["from_bus"][:2], [1, 1])
    np.testing.assert_array_equal(br["to_bus"][:2], [2, 2])
    # ratio 0 with a shift: a pure phase shifter e^{j phi}
    phi = -3 * 3.14159265358979323846 / 180.
    assert br["tap_re"][3] == math.cos(phi) and br["tap_im"][3] == math.sin(phi)
    assert br["tap_re"][4] == 1.03 * math.cos(2 * 3.14159265358979323846 / 180.)
    assert not g.notices


def test_crlf_and_blank_separated_rows_read_the_same(gb, tmp_path):
    text = _read_text("m_edge.m")
    a = gb.read_grid(os.path.join(GOLDEN, "m_edge.m"))
    _same_grid(a, gb.read_grid(_write(tmp_path, "crlf.m", text, newline="\r\n")))
    _same_grid(a, gb.read_grid(_write(tmp_path, "blank.m", text.replace("\t", "  "))))


def test_writer_round_trip(gb, tmp_path):
    src = gb.read_grid(os.path.join(GOLDEN, "c2_s3.cdf"))
    assert src.ybus_form == gb.YBUS_CDF
    p = str(tmp_path / "c2.m")
    src.write_m(p, "round trip")
    g = gb.read_grid(p)
    assert g.ybus_form == gb.YBUS_MATPOWER
    assert (g.nB, g.nL, g.nPV, g.nPQ, g.slack) == (src.nB, src.nL, src.nPV, src.nPQ, src.slack)
    for x, y in ((src.buses(), g.buses()), (src.pvpq(), g.pvpq()), (src.branches(), g.branches())):
        for k in x:
            np.testing.assert_allclose(y[k], x[k], rtol=1e-15, atol=1e-15, err_msg=k)
    # written again from the grid read back: the same bytes
    q = str(tmp_path / "again.m")
    g.write_m(q, "round trip")
    assert open(p).read() == open(q).read()


def test_writer_folds_pq_generation_into_load(gb, tmp_path):
    g = gb.create_grid(bus_type=[3, 0, 2], V0=[1.0, 1.0, 1.01], theta0=[0, 0, 0], from_bus=[1, 2], to_bus=[2, 3],
                       r=[0.01, 0.02], x=[0.1, 0.1], Pload=[0, 0.5, 0.1], Qload=[0, 0.1, 0.05], Pg=[0, 0.2, 0.3],
                       Qg=[0, 0.05, 0], Qmax=[0, 0, 0.4], Qmin=[0, 0, -0.4])
    p = str(tmp_path / "f.m")
    g.write_m(p)
    r = gb.read_grid(p).buses()
    b = g.buses()
    np.testing.assert_allclose(r["Pg"] - r["Pload"], b["Pg"] - b["Pload"], atol=1e-15)
    np.testing.assert_allclose(r["Qg"] - r["Qload"], b["Qg"] - b["Qload"], atol=1e-15)
    assert r["Pg"][1] == 0


def test_pv_bus_without_generator(gb, oracle, tmp_path):
    """The reference prints a notice and leaves that bus's Q limits unset; here
    they read as zero (GPU/m.h:318-326)."""
    text = _read_text("m_edge.m").replace("\t20\t40\t0\t30\t-10", "\t99\t40\t0\t30\t-10")
    p = _write(tmp_path, "nogen.m", text)
    g = gb.read_grid(p)
    assert any("de tipo PV" in n and "20" in n for n in g.notices)
    pv = g.pvpq()
    assert pv["Qmax"][0] == 0 and pv["Qmin"][0] == 0 and g.buses()["Pg"][1] == 0
    o = oracle.Grid(p)
    assert o.n_warn == 1 and o.Qmax[0] == 0 and o.Pg[1] == 0


def test_reader_errors(gb, oracle, tmp_path):
    text = _read_text("m_edge.m")
    bad = {
        "nobase.m": text.replace("mpc.baseMVA = 100;", ""),
        "twoslack.m": text.replace("\t20\t2\t20", "\t20\t3\t20"),
        "noslack.m": text.replace("\t10\t3\t0", "\t10\t2\t0"),
        "type4.m": text.replace("\t40\t1\t40", "\t40\t4\t40"),
        "nan.m": text.replace("\t0.015\t0.07", "\tx0.015\t0.07"),
        "short.m": text.replace("\t60\t1\t60\t12\t2\t-5\t1\t1\t0\t230\t1\t1.1\t0.9;", "\t60\t1\t60;"),
        "unknown.m": text.replace("\t20\t60\t0.03", "\t20\t61\t0.03"),
    }
    for name, t in bad.items():
        p = _write(tmp_path, name, t)
        with pytest.raises(gb.GbpfError) as e:
            gb.read_grid(p)
        assert e.value.status == gb.E_INPUT, name
        with pytest.raises(ValueError):
            oracle.Grid(p)
    with pytest.raises(gb.GbpfError):
        gb.read_grid(str(tmp_path / "missing.m"))


def test_ybus_form_setter(gb):
    g = gb.read_grid(os.path.join(GOLDEN, "c1.cdf"))
    assert g.ybus_form == gb.YBUS_CDF
    g.set_ybus_form(gb.YBUS_MATPOWER)
    assert g.ybus_form == gb.YBUS_MATPOWER
    with pytest.raises(gb.GbpfError):
        g.set_ybus_form(7)


@pytest.mark.parametrize("name", M_FILES)
def test_oracle_ybus_matches_reference_matpower_form(oracle, name):
    """calcYbusSp_Matpower's pattern and values, as the reference computed them."""
    gold = load_golden(name.replace(".m", "_lim0.json"))
    og = oracle.Grid(os.path.join(GOLDEN, name))
    rp, col, re, im = og.ybus()
    assert len(re) == gold["nnzY"] == len(gold["Y_re"])
    scale = np.max(np.abs(np.array(gold["Y_re"]) + 1j * np.array(gold["Y_im"])))
    assert np.max(np.abs(re - gold["Y_re"])) <= 1e-14 * scale
    assert np.max(np.abs(im - gold["Y_im"])) <= 1e-14 * scale


def test_matpower_form_differs_where_expected(oracle):
    """The two forms differ only on the from-side diagonal of branches with
    both an off-nominal tap and line charging, by (b/2)(1/|t|^2 - 1)."""
    og = oracle.Grid(os.path.join(GOLDEN, "c2_tx.m"))
    rp, col, re_m, im_m = og.ybus()
    og.set_ybus_form(0)
    _, _, re_c, im_c = og.ybus()
    tap2 = og.tap_re ** 2 + og.tap_im ** 2
    want = np.zeros(og.nB)
    np.add.at(want, og.de - 1, og.bsh_br / 2 * (1 / tap2 - 1))
    row = np.repeat(np.arange(og.nB), np.diff(rp))
    diag = col == row
    assert np.max(np.abs(re_m - re_c)) < 1e-12
    assert np.max(np.abs((im_m - im_c)[~diag])) < 1e-12
    np.testing.assert_allclose((im_m - im_c)[diag], want, atol=1e-12)
    assert np.count_nonzero(np.abs(want) > 1e-6) >= 5
