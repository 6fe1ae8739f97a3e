"""ctypes wrapper of the CPU oracle (oracle/pf_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py`` as the checker.  The product never
imports this module.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB_PATH = os.path.join(BUILD, "libpforacle.so")
CLI_PATH = os.path.join(BUILD, "pforacle")

_lib = None

EVENT_TEXT = {
    1: "PV -> PQ (limite superior)",
    2: "PQ (limite inferior) -> PQ (limite superior)",
    3: "PV -> PQ (limite inferior)",
    4: "PQ (limite superior) -> PQ (limite inferior)",
    5: "PQ -> PV",
}


def build():
    """Compile the oracle with its Makefile (gcc, a few seconds)."""
    subprocess.run(["make", "-s", "-C", HERE], check=True)


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.orc_h_open.restype = P
        L.orc_h_open.argtypes = [ctypes.c_char_p, ctypes.c_double, ctypes.c_double,
                                 ctypes.c_char_p, ctypes.c_int]
        for name in ("orc_h_close", "orc_h_dims", "orc_h_bus", "orc_h_pv", "orc_h_branch",
                     "orc_h_set_bus", "orc_h_ybus", "orc_h_pq", "orc_h_result", "orc_h_set_dense_ybus", "orc_h_set_ybus_form"):
            getattr(L, name).restype = None
        L.orc_h_ybus_form.restype = ctypes.c_int
        L.orc_h_jacobian.restype = ctypes.c_int
        L.orc_h_solve.restype = ctypes.c_int
        L.orc_h_sparse_solve.restype = ctypes.c_int
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


class Grid:
    """One grid read by the oracle's reader: CDF (GPU/sistema.h:386-638) or
    MATPOWER .m (GPU/m.h:296-622, Ybus by calcYbusSp_Matpower)."""

    def __init__(self, path, v_inicial=1.0, theta_inicial=0.0):
        L = lib()
        err = ctypes.create_string_buffer(256)
        h = L.orc_h_open(os.fsencode(path), v_inicial, theta_inicial, err, 256)
        if not h:
            raise ValueError(err.value.decode())
        self.h = ctypes.c_void_p(h)
        d = np.zeros(8, np.int32)
        L.orc_h_dims(self.h, _p(d))
        self.nB, self.nL, self.nPV, self.nPQ, self.slack, self.nnzY, self.n_warn, base = (int(x) for x in d)
        self.baseMVA = float(base)
        n = self.nB
        self.id = np.zeros(n, np.int32)
        self.type = np.zeros(n, np.int32)
        f = [np.zeros(n) for _ in range(8)]
        L.orc_h_bus(self.h, _p(self.id), _p(self.type), *[_p(a) for a in f])
        self.V0, self.theta0, self.Pload, self.Qload, self.Pg, self.Qg, self.gsh, self.bsh = f
        self.pv = np.zeros(self.nPV, np.int32)
        self.pq = np.zeros(self.nPQ, np.int32)
        self.Qmin = np.zeros(self.nPV)
        self.Qmax = np.zeros(self.nPV)
        self.Vset = np.zeros(self.nPV)
        L.orc_h_pv(self.h, _p(self.pv), _p(self.Qmin), _p(self.Qmax), _p(self.Vset), _p(self.pq))
        m = self.nL
        self.de = np.zeros(m, np.int32)
        self.para = np.zeros(m, np.int32)
        b = [np.zeros(m) for _ in range(6)]
        L.orc_h_branch(self.h, _p(self.de), _p(self.para), *[_p(a) for a in b])
        self.z_re, self.z_im, self.bsh_br, self.tap_re, self.tap_im, self.phi = b
        self.ybus_form = int(L.orc_h_ybus_form(self.h))

    def close(self):
        if self.h:
            lib().orc_h_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_bus(self, Pload=None, Qload=None, Pg=None, Qg=None, V=None, theta=None):
        args = []
        keep = []
        for a in (Pload, Qload, Pg, Qg, V, theta):
            if a is None:
                args.append(None)
            else:
                a = np.ascontiguousarray(a, np.float64)
                keep.append(a)
                args.append(_p(a))
        lib().orc_h_set_bus(self.h, *args)
        if Pload is not None:
            self.Pload = np.array(Pload, np.float64)
        if Qload is not None:
            self.Qload = np.array(Qload, np.float64)
        if Pg is not None:
            self.Pg = np.array(Pg, np.float64)
        if Qg is not None:
            self.Qg = np.array(Qg, np.float64)
        if V is not None:
            self.V0 = np.array(V, np.float64)
        if theta is not None:
            self.theta0 = np.array(theta, np.float64)

    def set_dense_ybus(self, dense=True):
        """Ybus by calcYbus's rule (metodo = denso: off-diagonal entries
        assigned branch by branch, GPU/sistema.h:673-703) or calcYbusSp's."""
        lib().orc_h_set_dense_ybus(self.h, int(bool(dense)))

    def set_ybus_form(self, form):
        """0: calcYbusSp_eficinte's branch stamps, 1: calcYbusSp_Matpower's."""
        lib().orc_h_set_ybus_form(self.h, int(form))
        self.ybus_form = int(form)

    def ybus(self):
        rp = np.zeros(self.nB + 1, np.int32)
        c = np.zeros(self.nnzY, np.int32)
        re = np.zeros(self.nnzY)
        im = np.zeros(self.nnzY)
        lib().orc_h_ybus(self.h, _p(rp), _p(c), _p(re), _p(im))
        return rp, c, re, im

    def injections(self, V, theta):
        V = np.ascontiguousarray(V, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        P = np.zeros(self.nB)
        Q = np.zeros(self.nB)
        lib().orc_h_pq(self.h, _p(V), _p(theta), _p(P), _p(Q))
        return P, Q

    def jacobian(self, V, theta, pqlim=None):
        """CSR Jacobian in the reference order for PQ list ``pqlim`` (1-based)."""
        V = np.ascontiguousarray(V, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        pqlim = np.ascontiguousarray(self.pq if pqlim is None else pqlim, np.int32)
        dim = self.nB - 1 + len(pqlim)
        cap = 4 * self.nnzY + 16
        rp = np.zeros(dim + 1, np.int32)
        c = np.zeros(cap, np.int32)
        v = np.zeros(cap)
        nnz = lib().orc_h_jacobian(self.h, _p(V), _p(theta), _p(pqlim), len(pqlim), _p(rp), _p(c), _p(v), cap)
        assert nnz >= 0
        return rp, c[:nnz].copy(), v[:nnz].copy()

    def solve(self, tol=1e-8, max_iter=100, lim_inj_reat=False):
        L = lib()
        info = np.zeros(6, np.int32)
        fm = ctypes.c_double()
        L.orc_h_solve(self.h, ctypes.c_double(tol), int(max_iter), int(bool(lim_inj_reat)), _p(info), ctypes.byref(fm))
        it, conv, st, nev, npqlim, nh = (int(x) for x in info)
        n, m = self.nB, self.nL
        out = {k: np.zeros(n) for k in ("V", "theta", "Pcalc", "Qcalc")}
        fl = {k: np.zeros(m) for k in ("Pdp", "Ppd", "Qdp", "Qpd")}
        hist = np.zeros(max(nh, 1))
        ev = np.zeros(max(4 * nev, 4), np.int32)
        limQ = np.zeros(max(self.nPV, 1), np.int32)
        L.orc_h_result(self.h, _p(out["V"]), _p(out["theta"]), _p(out["Pcalc"]), _p(out["Qcalc"]),
                       _p(fl["Pdp"]), _p(fl["Ppd"]), _p(fl["Qdp"]), _p(fl["Qpd"]), _p(hist), _p(ev), _p(limQ))
        out.update(fl)
        out.update(iterations=it, converged=bool(conv), status=st, final_mismatch=fm.value,
                   nPQlim=npqlim, hist=hist[:nh].copy(),
                   events=[tuple(int(x) for x in ev[4 * i:4 * i + 4]) for i in range(nev)],
                   limQ=limQ[:self.nPV].copy())
        return out


def sparse_solve(rowptr, col, val, b):
    rowptr = np.ascontiguousarray(rowptr, np.int32)
    col = np.ascontiguousarray(col, np.int32)
    val = np.ascontiguousarray(val, np.float64)
    b = np.ascontiguousarray(b, np.float64)
    x = np.zeros_like(b)
    st = lib().orc_h_sparse_solve(len(b), _p(rowptr), _p(col), _p(val), _p(b), _p(x))
    if st:
        raise ArithmeticError("singular")
    return x
