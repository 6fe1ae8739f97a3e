"""The oracle's Ybus under calcYbus's rule (metodo = denso,
GPU/sistema.h:673-703): off-diagonal entries assigned branch by branch, so with
a branch 1 -> 2 and a reversed branch 2 -> 1 the (1,2) entry is the later
branch's stamp alone, while calcYbusSp sums both; diagonal entries and grids
without reversed pairs are the same under both rules."""
import os

import numpy as np

from conftest import GOLDEN
from test_gpu_dense import _reversed_branch_grid


def _dense_y(og):
    rp, c, re, im = og.ybus()
    Y = np.zeros((og.nB, og.nB), complex)
    for r in range(og.nB):
        for p in range(rp[r], rp[r + 1]):
            Y[r, c[p]] = re[p] + 1j * im[p]
    return Y


def test_dense_rule_keeps_the_later_branch(gb, oracle, tmp_path):
    og = oracle.Grid(_reversed_branch_grid(gb, tmp_path))
    sp = _dense_y(og)
    og.set_dense_ybus(True)
    dn = _dense_y(og)
    f, t = og.de[-1] - 1, og.para[-1] - 1  # the added reversed branch
    off = ~np.eye(og.nB, dtype=bool)
    diff = np.abs(dn - sp) > 1e-12
    assert diff[f, t] and diff[t, f]
    assert np.count_nonzero(diff & off) == 2
    np.testing.assert_allclose(np.diag(dn), np.diag(sp), rtol=0, atol=1e-12)
    # the later branch alone (no tap): its stamps -y at (de, para) and (para, de), y = 1 / z
    y = 1.0 / (og.z_re[-1] + 1j * og.z_im[-1])
    assert abs(dn[f, t] + y) < 1e-12 and abs(dn[t, f] + y) < 1e-12


def test_dense_rule_changes_nothing_without_reversed_pairs(oracle):
    og = oracle.Grid(os.path.join(GOLDEN, "c2_base.cdf"))
    sp = _dense_y(og)
    og.set_dense_ybus(True)
    np.testing.assert_array_equal(_dense_y(og), sp)
