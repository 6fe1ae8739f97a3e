"""Host-side logic of libgbpf that needs no GPU: the C ABI surface, the data.txt
parser (loadFile semantics), the CDF/CDFX reader and writer, the seeded grid
generator and the symbolic analysis."""
import os
import re

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, ieee_cases, ieee_path

DATA_TXT = """metodo         = esparso;        // esparso, denso or hibridoC
openmp         = OFF;
v_inicial      = 1.0;             // flat start
theta_inicial  = 0.0;
tolerancia     = 0.00000001;
no_max_iter    = 25;
arq_entrada    = c1.cdf;     // input cdf file name
laconic_mode   = OFF;
output_bench   = SCREEN;
output_ans     = ON;
lim_inj_reat   = ON;
"""


def test_library_exports_every_declared_symbol(gb):
    header = open(os.path.join(ROOT, "include", "gbpf.h")).read()
    declared = sorted(set(re.findall(r"\b(gbpf_[a-z_]+)\s*\(", header)))
    assert len(declared) >= 30
    lib = gb.lib()
    for name in declared:
        assert hasattr(lib, name), name
    assert sorted(gb.EXPORTS) == declared


def test_options_defaults(gb):
    o = gb.Options()
    assert (o.v_inicial, o.theta_inicial, o.tolerancia, o.no_max_iter) == (1.0, 0.0, 1e-4, 100)
    assert (o.lim_inj_reat, o.laconic_mode, o.output_ans, o.streams) == (0, 0, 1, 1)
    assert o.arq_entrada == "ieee14.cdf"


def test_options_parse_all_keys(gb):
    o = gb.parse_options(DATA_TXT)
    assert o.metodo == gb.METODO["esparso"]
    assert o.tolerancia == 1e-8 and o.no_max_iter == 25 and o.lim_inj_reat == 1
    assert o.arq_entrada == "c1.cdf" and o.openmp == 0 and o.laconic_mode == 0
    assert o.output_bench == 1 and o.output_ans == 1
    # the echo loadFile prints when laconic_mode is OFF
    lines = o.echo.splitlines()
    assert lines[0] == "metodo         = esparso"
    assert "lim_inj_reat   = ON" in lines
    assert "tolerancia     = 1e-08" in lines
    assert "v_inicial      = 1.000000" in lines


@pytest.mark.parametrize("metodo,code", [("esparso", 0), ("denso", 1), ("hibridoA", 2), ("hibridoB", 3),
                                         ("hibridoC", 4), ("qr", 5)])
def test_options_metodo(gb, metodo, code):
    o = gb.parse_options(DATA_TXT.replace("= esparso;", f"= {metodo};"))
    assert o.metodo == code


def test_options_absent_key_reads_first_value(gb):
    """An absent key makes loadFile's npos arithmetic wrap: it reads the value of
    the first '=' near the start of the text (GPU/sistInfo.h:120-130)."""
    text = DATA_TXT.replace("lim_inj_reat   = ON;\n", "")
    assert gb.parse_options(text).lim_inj_reat == 0  # first value "esparso" is neither ON nor OFF
    text_on = "verbose_mode = ON;\n" + text
    assert gb.parse_options(text_on).lim_inj_reat == 1  # first value is ON
    assert "lim_inj_reat" not in gb.parse_options(text).echo


def test_options_laconic_and_precision(gb):
    o = gb.parse_options(DATA_TXT.replace("laconic_mode   = OFF", "laconic_mode   = ON") + "precisao = FP32;\n")
    assert o.laconic_mode == 1 and o.echo == "" and o.precision == gb.PREC_FP32_IR


def test_options_bad_integer(gb):
    with pytest.raises(gb.GbpfError) as e:
        gb.parse_options(DATA_TXT.replace("no_max_iter    = 25", "no_max_iter    = many"))
    assert e.value.status == gb.E_INPUT


def test_options_load_missing_file(gb, tmp_path):
    with pytest.raises(gb.GbpfError):
        gb.load_options(str(tmp_path / "nope.txt"))


def _cases():
    out = [os.path.join(GOLDEN, f) for f in sorted(os.listdir(GOLDEN)) if f.endswith(".cdf")]
    # the reference's own IEEE inputs (committed fixtures)
    out += [c for c in ieee_cases() if c["lim"] == 0]
    return out


@pytest.mark.parametrize("path", _cases(), ids=lambda p: p["cdf"] if isinstance(p, dict) else os.path.basename(p))
def test_reader_matches_oracle_reader(gb, oracle, path):
    if isinstance(path, dict):
        path = ieee_path(path)
    g = gb.read_grid(path)
    o = oracle.Grid(path)
    assert (g.nB, g.nL, g.nPV, g.nPQ, g.slack) == (o.nB, o.nL, o.nPV, o.nPQ, o.slack)
    b = g.buses()
    for k, ok in (("id", o.id), ("type", o.type), ("V0", o.V0), ("theta0", o.theta0), ("Pload", o.Pload),
                  ("Qload", o.Qload), ("Pg", o.Pg), ("Qg", o.Qg), ("gsh", o.gsh), ("bsh", o.bsh)):
        np.testing.assert_array_equal(b[k], ok, err_msg=k)
    p = g.pvpq()
    np.testing.assert_array_equal(p["pv"], o.pv)
    np.testing.assert_array_equal(p["pq"], o.pq)
    np.testing.assert_array_equal(p["Qmin"], o.Qmin)
    np.testing.assert_array_equal(p["Qmax"], o.Qmax)
    br = g.branches()
    for k, ok in (("from_bus", o.de), ("to_bus", o.para), ("r", o.z_re), ("x", o.z_im), ("bch", o.bsh_br),
                  ("tap_re", o.tap_re), ("tap_im", o.tap_im), ("phase", o.phi)):
        np.testing.assert_array_equal(br[k], ok, err_msg=k)


def test_parallel_branch_merge_notices(gb):
    p = ieee_path(next(c for c in ieee_cases() if c["cdf"] == "ieee118.cdf"))
    g = gb.read_grid(p)
    assert g.nL == 179  # 186 branch lines, 7 parallel pairs merged
    assert sum(n.startswith("Ramo ") for n in g.notices) == 7


def _write(tmp_path, name, text):
    p = tmp_path / name
    p.write_text(text)
    return str(p)


def test_reader_errors(gb, tmp_path):
    good = open(os.path.join(GOLDEN, "c1.cdf"), newline="").read().split("\r\n")
    with pytest.raises(gb.GbpfError):
        gb.read_grid(str(tmp_path / "missing.cdf"))
    bad_type = list(good)
    bad_type[3] = bad_type[3][:24] + " 7" + bad_type[3][26:]
    with pytest.raises(gb.GbpfError):
        gb.read_grid(_write(tmp_path, "t.cdf", "\r\n".join(bad_type)))
    two_slack = list(good)
    two_slack[3] = two_slack[3][:24] + " 3" + two_slack[3][26:]
    with pytest.raises(gb.GbpfError):
        gb.read_grid(_write(tmp_path, "s.cdf", "\r\n".join(two_slack)))
    short = list(good)
    short[4] = short[4][:30]
    with pytest.raises(gb.GbpfError):
        gb.read_grid(_write(tmp_path, "h.cdf", "\r\n".join(short)))
    with pytest.raises(gb.GbpfError) as e:
        gb.read_grid(_write(tmp_path, "x.m", "mpc = 1;"))  # a .m file with no mpc.baseMVA
    assert e.value.status == gb.E_INPUT
    with pytest.raises(gb.GbpfError) as e:
        gb.read_grid(_write(tmp_path, "x.pwf", "TITU"))
    assert e.value.status == gb.E_INPUT


def test_generator_shapes_and_determinism(gb):
    a = gb.generate(1, 20261204)
    assert (a.nB, a.nL, a.nPV, a.nPQ) == (14, 20, 4, 9)
    assert (a.buses()["bsh"] == 0.19).sum() == 1
    tr = a.branches()
    assert (tr["tap_re"] != 1.0).sum() == 3 and np.all(tr["bch"][tr["tap_re"] != 1.0] == 0)
    b = gb.generate(2, 20261205)
    assert (b.nB, b.nL, b.nPV, b.nPQ) == (118, 186, 53, 64)
    assert (b.branches()["tap_re"] != 1.0).sum() == 9
    b2 = gb.generate(2, 20261205)
    for k, v in b.buses().items():
        np.testing.assert_array_equal(v, b2.buses()[k])
    for n in (14, 30, 57, 118, 236, 472):
        c = gb.generate(4, 7, nbus=n)
        assert c.nB == n and c.nL == (20 if n == 14 else round(1.6 * n))  # 14 buses: config 1 itself
        assert 0.2 * (n - 1) - 1 <= c.nPV <= 0.45 * (n - 1) + 1


def test_tiled_grid_and_cdfx_roundtrip(gb, tmp_path):
    t = gb.generate(3, 20261206, tiles=128)
    assert (t.nB, t.nL) == (15104, 128 * 186 + 3 * 127)
    assert t.nPV == 128 * 53 + 127 and t.nPQ == 128 * 64
    p = str(tmp_path / "c3.cdfx")
    t.write_cdf(p)
    r = gb.read_grid(p)
    assert (r.nB, r.nL, r.nPV, r.nPQ, r.slack) == (t.nB, t.nL, t.nPV, t.nPQ, t.slack)
    np.testing.assert_allclose(r.buses()["Pload"], t.buses()["Pload"], atol=1e-5)
    np.testing.assert_allclose(r.branches()["x"], t.branches()["x"], atol=1e-6)


def test_cdf_roundtrip_precision(gb, tmp_path):
    g = gb.generate(2, 99)
    p = str(tmp_path / "g.cdf")
    g.write_cdf(p)
    r = gb.read_grid(p)
    for k in ("Pload", "Qload", "Pg", "V0", "bsh"):
        np.testing.assert_allclose(r.buses()[k], g.buses()[k], atol=5e-5, err_msg=k)
    for k in ("r", "x", "bch", "tap_re"):
        np.testing.assert_allclose(r.branches()[k], g.branches()[k], atol=5e-5, err_msg=k)


def test_grid_from_arrays(gb):
    g = gb.create_grid(bus_type=[3, 2, 0], V0=[1.0, 1.02, 1.0], theta0=[0, 0, 0], from_bus=[1, 2, 1],
                       to_bus=[2, 3, 3], r=[0.01, 0.02, 0.03], x=[0.1, 0.2, 0.3], Pload=[0, 0, 0.5],
                       Qload=[0, 0, 0.2], Pg=[0, 0.3, 0], Qmax=[0, 1, 0], Qmin=[0, -1, 0])
    assert (g.nB, g.nL, g.nPV, g.nPQ, g.slack) == (3, 3, 1, 1, 1)
    with pytest.raises(gb.GbpfError):
        gb.create_grid(bus_type=[0, 0], V0=[1, 1], theta0=[0, 0], from_bus=[1], to_bus=[2], r=[0.1], x=[0.1])


@pytest.mark.parametrize("kind,kw", [(1, {}), (2, {}), (3, {"tiles": 16}), (4, {"nbus": 472})])
def test_symbolic_analysis(gb, kind, kw):
    a = gb.generate(kind, 5, **kw).analyse()
    assert a["closed"] == 1
    assert a["forward_levels"] >= 1 and a["backward_levels"] >= 1
    assert a["factor_blocks"] >= (a["jacobian_blocks"] - a["blocks"]) // 2


@pytest.mark.parametrize("name,blocks,levels", [("c2_base.cdf", 237, 21)])
def test_height_reduced_ordering(gb, name, blocks, levels):
    """The factor's ordering: minimum degree, then a perfect elimination order
    of its filled graph with the shortest elimination tree.  On the 118-bus
    grid: the minimum-degree fill (237 off-diagonal blocks, 145 update pairs)
    in 21 levels instead of 30; the pattern stays closed under fill."""
    a = gb.read_grid(os.path.join(GOLDEN, name)).analyse()
    assert a["closed"] == 1
    assert a["factor_blocks"] == blocks and a["update_pairs"] == 145
    assert a["forward_levels"] == a["backward_levels"] == levels


def test_height_reduction_on_the_tiled_grids(gb):
    """1,888 and 15,104 buses: fewer levels than minimum degree alone (35 and
    109) with no more factor blocks (4,253 and 36,872)."""
    import bench
    for f, lv, fb in (("c5_base.cdf.gz", 35, 4253), ("c3_base.cdfx.gz", 109, 36872)):
        a = gb.read_grid(bench.grid_file(f)).analyse()
        assert a["closed"] == 1
        assert a["forward_levels"] < lv and a["factor_blocks"] <= fb, (f, a)


def test_table_sincos_method_error_bound():
    """The table method the batch kernels use for the bus angles' sine and
    cosine (sincos_tab in csrc/batch.cu: theta = k h + d, h = 2 pi / 256, a
    256-entry table of cos and sin of k h, Taylor polynomials of degree 6 and
    7 in d, angle-sum formulas), restated in numpy with the same constants and
    operation order (fused multiply-adds emulated in extended precision):
    within 4 ulp of the library sine and cosine for angles in [-20, 20] rad,
    the range bus angles live in by orders of magnitude."""
    import numpy as np

    ld = np.longdouble

    def fma(a, b, c):
        return np.float64(ld(a) * ld(b) + ld(c))

    two_pi = ld("6.283185307179586476925286766559005768")
    tab = [(np.float64(np.cos(two_pi * i / 256)), np.float64(np.sin(two_pi * i / 256))) for i in range(256)]
    inv_h = np.float64("40.74366543152520595683424342336")
    h_hi = np.float64("6.28318530717958623199592693708837") / 256.0
    h_lo = np.float64("2.44929359829470635445e-16") / 256.0
    rng = np.random.default_rng(11)
    th = np.concatenate([rng.uniform(-20, 20, 4000), rng.uniform(-1e-3, 1e-3, 500),
                         np.arange(-1024, 1025) * (2 * np.pi / 256), [0.0, np.pi, -np.pi, 1e-300]])
    worst = 0.0
    for t in th:
        k = np.rint(t * inv_h)
        d = fma(-k, h_lo, fma(-k, h_hi, t))
        tc, ts = tab[int(k) & 255]
        d2 = d * d
        cd = fma(d2, fma(d2, fma(d2, -1.0 / 720.0, 1.0 / 24.0), -0.5), 1.0)
        sd = fma(d * d2, fma(d2, fma(d2, -1.0 / 5040.0, 1.0 / 120.0), -1.0 / 6.0), d)
        c = fma(tc, cd, -(ts * sd))
        s = fma(ts, cd, tc * sd)
        rc, rs = np.cos(ld(t)), np.sin(ld(t))
        for got, ref in ((c, rc), (s, rs)):
            ulp = np.spacing(np.float64(max(abs(ref), 1e-300)))
            worst = max(worst, float(abs(ld(got) - ref) / ld(ulp)) if abs(ref) > 1e-8 else float(abs(ld(got) - ref) / ld(2.0 ** -52)))
    assert worst <= 4.0, worst
