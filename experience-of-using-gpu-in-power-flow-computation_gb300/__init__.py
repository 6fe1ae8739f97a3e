"""gbpf: GB300-native Newton-Raphson AC power flow (Python host mirror).

Thin ctypes layer over ``lib/libgbpf.so`` (C ABI declared in include/gbpf.h).
It mirrors the reference's process-level interface: ``load_options`` reads a
data.txt exactly like ``loadFile`` (GPU/sistInfo.h:62-242), ``read_grid`` reads
a common-data-format file like ``lerArquivoEAlocarMemoria``
(GPU/arquivo.h:250-295), and ``Solver.solve`` runs ``mNR``
(GPU/newtonRaphson.cuh:171-623) on the GPU.  There is no CPU fallback: when the
library is missing or no GPU is present, the solver raises.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libgbpf.so")
CLI_PATH = os.path.join(HERE, "lib", "gbpf")

OK, E_INPUT, E_SINGULAR, E_NOCONV, E_CUDA, E_TIMEOUT, E_OOM, E_ARG, E_UNSUPPORTED = range(9)
METODO = {"esparso": 0, "denso": 1, "hibridoA": 2, "hibridoB": 3, "hibridoC": 4, "nda": 5}
PREC_FP64, PREC_FP32_IR = 0, 1
FORM_GRAPH, FORM_PERSISTENT = 1, 2
YBUS_CDF, YBUS_MATPOWER = 0, 1
EVENT_TEXT = {
    1: "PV -> PQ (limite superior)",
    2: "PQ (limite inferior) -> PQ (limite superior)",
    3: "PV -> PQ (limite inferior)",
    4: "PQ (limite superior) -> PQ (limite inferior)",
    5: "PQ -> PV",
}

# Every entry point include/gbpf.h declares (checked by the CPU test suite).
EXPORTS = [
    "gbpf_options_default", "gbpf_options_parse", "gbpf_options_load",
    "gbpf_grid_read", "gbpf_grid_create", "gbpf_grid_free", "gbpf_grid_dims", "gbpf_grid_buses",
    "gbpf_grid_pvpq", "gbpf_grid_branches", "gbpf_grid_set_buses", "gbpf_grid_write_cdf",
    "gbpf_generate", "gbpf_grid_analyse", "gbpf_solver_create", "gbpf_solver_free", "gbpf_solve", "gbpf_solver_set_start",
    "gbpf_solver_state", "gbpf_solver_events", "gbpf_solver_history", "gbpf_solver_triggers",
    "gbpf_solver_flows", "gbpf_solver_info", "gbpf_solver_time", "gbpf_solver_profile", "gbpf_ybus", "gbpf_eval_pq",
    "gbpf_eval_jacobian", "gbpf_newton_step", "gbpf_device_info", "gbpf_last_error", "gbpf_status_str",
    "gbpf_batch_create", "gbpf_batch_free", "gbpf_batch_set_instances", "gbpf_batch_solve", "gbpf_batch_time",
    "gbpf_batch_results", "gbpf_batch_events", "gbpf_batch_info", "gbpf_batch_solve_noalloc",
    "gbpf_mlp_create", "gbpf_mlp_free", "gbpf_mlp_dims", "gbpf_mlp_set_data", "gbpf_mlp_train", "gbpf_mlp_predict",
    "gbpf_mlp_gradients", "gbpf_mlp_params", "gbpf_mlp_set_params", "gbpf_mlp_norm", "gbpf_mlp_set_norm",
    "gbpf_batch_solve_warm", "gbpf_mlp_set_loss_metric", "gbpf_solver_setup_times", "gbpf_batch_kernel_times",
    "gbpf_grid_write_m", "gbpf_grid_ybus_form", "gbpf_grid_set_ybus_form",
    "gbpf_batch_get_plan", "gbpf_batch_set_plan", "gbpf_batch_autotune",
    "gbpf_batch_launch", "gbpf_batch_wait", "gbpf_batch_time_pipelined", "gbpf_batch_warm_phases",
    "gbpf_batch_solve_warm_launch", "gbpf_batch_solve_warm_wait", "gbpf_solver_set_lu_launch",
    "gbpf_batch_time_warm_pipelined", "gbpf_batch_events_all", "gbpf_mlp_set_wait_limit",
    "gbpf_solver_set_form", "gbpf_solver_get_form", "gbpf_batch_follow", "gbpf_solve_traced",
    "gbpf_solver_set_plan",
]


class GbpfError(RuntimeError):
    def __init__(self, status, where):
        self.status = status
        msg = ""
        try:
            msg = _lib.gbpf_last_error().decode(errors="replace")
        except Exception:
            pass
        super().__init__(f"{where}: status {status} ({_status_str(status)}) {msg}")


class _Options(ctypes.Structure):
    _fields_ = [
        ("metodo", ctypes.c_int), ("v_inicial", ctypes.c_double), ("theta_inicial", ctypes.c_double),
        ("tolerancia", ctypes.c_double), ("no_max_iter", ctypes.c_int), ("lim_inj_reat", ctypes.c_int),
        ("openmp", ctypes.c_int), ("laconic_mode", ctypes.c_int), ("verbose_mode", ctypes.c_int),
        ("output_ans", ctypes.c_int), ("output_iter", ctypes.c_int), ("streams", ctypes.c_int),
        ("output_bench", ctypes.c_int), ("precision", ctypes.c_int), ("arq_entrada", ctypes.c_char * 1024),
    ]


class _Result(ctypes.Structure):
    _fields_ = [("status", ctypes.c_int), ("converged", ctypes.c_int), ("iterations", ctypes.c_int),
                ("n_events", ctypes.c_int), ("nPQlim", ctypes.c_int), ("final_mismatch", ctypes.c_double)]


class _GridDesc(ctypes.Structure):
    _fields_ = [("nB", ctypes.c_int), ("nL", ctypes.c_int), ("baseMVA", ctypes.c_double),
                ("id", ctypes.c_void_p), ("bus_type", ctypes.c_void_p)] + \
               [(n, ctypes.c_void_p) for n in ("V0", "theta0", "Pload", "Qload", "Pg", "Qg", "gsh", "bsh",
                                               "Qmax", "Qmin", "from_bus", "to_bus", "r", "x", "bch",
                                               "tap_re", "tap_im", "phase")]


_lib = None


def lib():
    """Loads libgbpf.so; raises when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise OSError(f"{LIB_PATH} is missing: run __graft_entry__.build() (nvcc, sm_103a)")
        L = ctypes.CDLL(LIB_PATH)
        for name in EXPORTS:
            getattr(L, name).restype = ctypes.c_int
        L.gbpf_last_error.restype = ctypes.c_char_p
        L.gbpf_status_str.restype = ctypes.c_char_p
        L.gbpf_grid_free.restype = None
        L.gbpf_solver_free.restype = None
        L.gbpf_batch_free.restype = None
        L.gbpf_mlp_free.restype = None
        _lib = L
    return _lib


def _status_str(st):
    try:
        return lib().gbpf_status_str(int(st)).decode()
    except Exception:
        return str(st)


def _check(st, where):
    if st != OK:
        raise GbpfError(st, where)


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f64(a):
    return None if a is None else np.ascontiguousarray(a, np.float64)


def _i32(a):
    return None if a is None else np.ascontiguousarray(a, np.int32)


# --------------------------------------------------------------------- options
class Options:
    """The data.txt options (namespace global of GPU/sistInfo.h:37-60)."""

    def __init__(self, raw=None):
        if raw is None:
            raw = _Options()
            lib().gbpf_options_default(ctypes.byref(raw))
        self._o = raw
        self.echo = ""

    def __getattr__(self, k):
        if k.startswith("_") or k == "echo":
            raise AttributeError(k)
        v = getattr(self._o, k)
        return v.decode() if isinstance(v, bytes) else v

    def __setattr__(self, k, v):
        if k in ("_o", "echo"):
            object.__setattr__(self, k, v)
        elif k == "arq_entrada":
            self._o.arq_entrada = os.fsencode(v)
        else:
            setattr(self._o, k, v)


def parse_options(text):
    o = Options()
    echo = ctypes.create_string_buffer(1 << 16)
    _check(lib().gbpf_options_parse(text.encode() if isinstance(text, str) else text,
                                    ctypes.byref(o._o), echo, len(echo)), "gbpf_options_parse")
    o.echo = echo.value.decode(errors="replace")
    return o


def load_options(path="data.txt"):
    o = Options()
    echo = ctypes.create_string_buffer(1 << 16)
    _check(lib().gbpf_options_load(os.fsencode(path), ctypes.byref(o._o), echo, len(echo)), "gbpf_options_load")
    o.echo = echo.value.decode(errors="replace")
    return o


# ----------------------------------------------------------------------- grids
class Grid:
    """One grid (struct sistema / barra / ramo of GPU/sistema.h:24-126)."""

    def __init__(self, handle):
        self.h = ctypes.c_void_p(handle)
        d = np.zeros(8, np.int32)
        _check(lib().gbpf_grid_dims(self.h, _p(d)), "gbpf_grid_dims")
        self.nB, self.nL, self.nPV, self.nPQ, self.slack, self.nnzY, base, self.n_notices = (int(x) for x in d)
        self.baseMVA = float(base)

    def close(self):
        if getattr(self, "h", None):
            lib().gbpf_grid_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def buses(self):
        n = self.nB
        i = [np.zeros(n, np.int32) for _ in range(2)]
        f = [np.zeros(n) for _ in range(8)]
        _check(lib().gbpf_grid_buses(self.h, *[_p(a) for a in i + f]), "gbpf_grid_buses")
        keys = ("id", "type", "V0", "theta0", "Pload", "Qload", "Pg", "Qg", "gsh", "bsh")
        return dict(zip(keys, i + f))

    def pvpq(self):
        pv = np.zeros(self.nPV, np.int32)
        pq = np.zeros(self.nPQ, np.int32)
        f = [np.zeros(self.nPV) for _ in range(3)]
        _check(lib().gbpf_grid_pvpq(self.h, _p(pv), *[_p(a) for a in f], _p(pq)), "gbpf_grid_pvpq")
        return dict(pv=pv, Qmin=f[0], Qmax=f[1], Vset=f[2], pq=pq)

    def branches(self):
        m = self.nL
        i = [np.zeros(m, np.int32) for _ in range(2)]
        f = [np.zeros(m) for _ in range(6)]
        _check(lib().gbpf_grid_branches(self.h, *[_p(a) for a in i + f]), "gbpf_grid_branches")
        return dict(zip(("from_bus", "to_bus", "r", "x", "bch", "tap_re", "tap_im", "phase"), i + f))

    def set_buses(self, Pload=None, Qload=None, Pg=None, Qg=None, V0=None, theta0=None):
        arrs = [_f64(a) for a in (Pload, Qload, Pg, Qg, V0, theta0)]
        _check(lib().gbpf_grid_set_buses(self.h, *[_p(a) for a in arrs]), "gbpf_grid_set_buses")

    def analyse(self):
        """Host-only symbolic analysis of the Newton Jacobian (no GPU needed)."""
        a = np.zeros(8, np.int64)
        _check(lib().gbpf_grid_analyse(self.h, _p(a)), "gbpf_grid_analyse")
        keys = ("blocks", "factor_blocks", "update_pairs", "forward_levels", "backward_levels", "nnzY",
                "jacobian_blocks", "closed")
        return dict(zip(keys, (int(x) for x in a)))

    def write_cdf(self, path, title="synthetic grid"):
        _check(lib().gbpf_grid_write_cdf(self.h, os.fsencode(path), title.encode()), "gbpf_grid_write_cdf")

    def write_m(self, path, title="synthetic grid"):
        """MATPOWER case (version 2) that read_grid and the reference's .m reader read back."""
        _check(lib().gbpf_grid_write_m(self.h, os.fsencode(path), title.encode()), "gbpf_grid_write_m")

    @property
    def ybus_form(self):
        """YBUS_CDF (calcYbusSp_eficinte) or YBUS_MATPOWER (calcYbusSp_Matpower, .m input)."""
        return int(lib().gbpf_grid_ybus_form(self.h))

    def set_ybus_form(self, form):
        _check(lib().gbpf_grid_set_ybus_form(self.h, int(form)), "gbpf_grid_set_ybus_form")


def time_pipelined(batches, steps):
    """gbpf_batch_time_pipelined: device ms of `steps` solves spread
    round-robin over the batches, each on its own stream."""
    arr = (ctypes.c_void_p * len(batches))(*[b.h.value for b in batches])
    ms = ctypes.c_double()
    _check(lib().gbpf_batch_time_pipelined(arr, len(batches), int(steps), ctypes.byref(ms)),
           "gbpf_batch_time_pipelined")
    return ms.value


def time_warm_pipelined(batches, mlp, steps):
    """gbpf_batch_time_warm_pipelined: device ms of `steps` warm-started
    solves spread round-robin over the batches, each on its own stream."""
    arr = (ctypes.c_void_p * len(batches))(*[b.h.value for b in batches])
    ms = ctypes.c_double()
    _check(lib().gbpf_batch_time_warm_pipelined(arr, len(batches), mlp.h, int(steps), ctypes.byref(ms)),
           "gbpf_batch_time_warm_pipelined")
    return ms.value


def read_grid(path, v_inicial=1.0, theta_inicial=0.0):
    h = ctypes.c_void_p()
    msg = ctypes.create_string_buffer(1 << 16)
    _check(lib().gbpf_grid_read(os.fsencode(path), ctypes.c_double(v_inicial), ctypes.c_double(theta_inicial),
                                ctypes.byref(h), msg, len(msg)), f"gbpf_grid_read({path})")
    g = Grid(h.value)
    g.notices = [l for l in msg.value.decode(errors="replace").split("\n") if l]
    return g


def create_grid(bus_type, V0, theta0, from_bus, to_bus, r, x, bch=None, tap_re=None, tap_im=None,
                phase=None, Pload=None, Qload=None, Pg=None, Qg=None, gsh=None, bsh=None,
                Qmax=None, Qmin=None, id=None, baseMVA=100.0):
    keep = {}

    def put(name, a, conv):
        if a is None:
            return None
        a = conv(a)
        keep[name] = a
        return _p(a)

    d = _GridDesc()
    d.nB = len(bus_type)
    d.nL = len(from_bus)
    d.baseMVA = baseMVA
    d.id = put("id", id, _i32)
    d.bus_type = put("bus_type", bus_type, _i32)
    for n, a in (("V0", V0), ("theta0", theta0), ("Pload", Pload), ("Qload", Qload), ("Pg", Pg), ("Qg", Qg),
                 ("gsh", gsh), ("bsh", bsh), ("Qmax", Qmax), ("Qmin", Qmin), ("r", r), ("x", x), ("bch", bch),
                 ("tap_re", tap_re), ("tap_im", tap_im), ("phase", phase)):
        setattr(d, n, put(n, a, _f64))
    d.from_bus = put("from_bus", from_bus, _i32)
    d.to_bus = put("to_bus", to_bus, _i32)
    h = ctypes.c_void_p()
    _check(lib().gbpf_grid_create(ctypes.byref(d), ctypes.byref(h)), "gbpf_grid_create")
    return Grid(h.value)


def generate(kind, seed, tiles=0, nbus=0):
    """Seeded synthetic grid: 1 = 14-bus, 2 = 118-bus, 3 = tiled 118-bus, 4 = scaled 14-bus style."""
    h = ctypes.c_void_p()
    _check(lib().gbpf_generate(int(kind), ctypes.c_ulonglong(seed), int(tiles), int(nbus), ctypes.byref(h)),
           "gbpf_generate")
    return Grid(h.value)


def device_info(device=0):
    cnt = ctypes.c_int()
    name = ctypes.create_string_buffer(256)
    props = np.zeros(6, np.int32)
    st = lib().gbpf_device_info(int(device), ctypes.byref(cnt), name, 256, _p(props))
    if st not in (OK, E_ARG):
        raise GbpfError(st, "gbpf_device_info")
    return dict(count=cnt.value, name=name.value.decode(), props=props)


# ---------------------------------------------------------------------- solver
_PI, _PD = ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_double)


class _Trace(ctypes.Structure):
    """gbpf_trace (include/gbpf.h): one stage record of gbpf_solve_traced."""
    _fields_ = [("stage", ctypes.c_int), ("iteration", ctypes.c_int), ("nB", ctypes.c_int), ("nPV", ctypes.c_int),
                ("nPQlim", ctypes.c_int), ("nPVlim", ctypes.c_int), ("done", ctypes.c_int),
                ("converged", ctypes.c_int), ("max_g", ctypes.c_double), ("limit_check", ctypes.c_int),
                ("n_events", ctypes.c_int), ("events", _PI), ("P", _PD), ("Q", _PD), ("V", _PD), ("theta", _PD),
                ("QliqLim", _PD), ("limQ", _PI), ("pv_lim", _PI), ("pq_lim", _PI), ("n_g", ctypes.c_int),
                ("g", _PD), ("nnzJ", ctypes.c_int), ("jrow", _PI), ("jcol", _PI), ("jval", _PD)]


_TRACE_FN = ctypes.CFUNCTYPE(None, ctypes.POINTER(_Trace), ctypes.c_void_p)
TRACE_EVAL, TRACE_JACOBIAN, TRACE_STEP, TRACE_UPDATE = 0, 1, 2, 3


class Solver:
    """mNR on one GPU: device-resident Newton loop captured in a CUDA graph."""

    def __init__(self, grid, options=None, device=0, **overrides):
        o = options if options is not None else Options()
        if isinstance(o, dict):
            oo = Options()
            for k, v in o.items():
                setattr(oo, k, v)
            o = oo
        for k, v in overrides.items():
            setattr(o, k, v)
        self.grid = grid
        self.options = o
        self.h = ctypes.c_void_p()
        _check(lib().gbpf_solver_create(grid.h, ctypes.byref(o._o), int(device), ctypes.byref(self.h)),
               "gbpf_solver_create")

    def close(self):
        if getattr(self, "h", None):
            lib().gbpf_solver_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def solve(self, full=True):
        r = _Result()
        st = lib().gbpf_solve(self.h, ctypes.byref(r))
        if st not in (OK, E_NOCONV, E_SINGULAR):
            raise GbpfError(st, "gbpf_solve")
        out = dict(status=r.status, converged=bool(r.converged), iterations=r.iterations,
                   n_events=r.n_events, nPQlim=r.nPQlim, final_mismatch=r.final_mismatch)
        if full:
            out.update(self.state())
            out["events"] = self.events()
            out["hist"] = self.history()
            out.update(self.flows())
        return out

    def solve_traced(self, fn=None):
        """gbpf_solve_traced: the solve stage by stage (the graph form's kernels,
        one host sync per stage).  Returns the result dict of solve() plus
        "trace", one dict per stage record (gbpf_trace: stage, iteration,
        P, Q, V, theta, QliqLim, limQ, pv_lim, pq_lim, g, J rows/cols/values,
        events, ...); fn(record) is also called with each record when given."""
        recs = []

        def cb(tp, _user):
            t = tp.contents
            nB, nPV = t.nB, t.nPV
            arr = lambda ptr, n, dt: np.ctypeslib.as_array(ptr, shape=(n,)).astype(dt) if n > 0 and ptr else \
                np.zeros(0, dt)
            rec = dict(stage=t.stage, iteration=t.iteration, nPQlim=t.nPQlim, nPVlim=t.nPVlim, done=t.done,
                       converged=t.converged, max_g=t.max_g, limit_check=t.limit_check,
                       events=[tuple(int(x) for x in arr(t.events, 4 * t.n_events, np.int32)[4 * i:4 * i + 4])
                               for i in range(t.n_events)],
                       P=arr(t.P, nB, np.float64), Q=arr(t.Q, nB, np.float64), V=arr(t.V, nB, np.float64),
                       theta=arr(t.theta, nB, np.float64), QliqLim=arr(t.QliqLim, nB, np.float64),
                       limQ=arr(t.limQ, nPV, np.int32), pv_lim=arr(t.pv_lim, t.nPVlim, np.int32),
                       pq_lim=arr(t.pq_lim, t.nPQlim, np.int32), g=arr(t.g, t.n_g, np.float64),
                       jrow=arr(t.jrow, t.nnzJ, np.int32), jcol=arr(t.jcol, t.nnzJ, np.int32),
                       jval=arr(t.jval, t.nnzJ, np.float64))
            recs.append(rec)
            if fn is not None:
                fn(rec)

        c_cb = _TRACE_FN(cb)
        r = _Result()
        st = lib().gbpf_solve_traced(self.h, ctypes.byref(r), c_cb, None)
        if st not in (OK, E_NOCONV, E_SINGULAR):
            raise GbpfError(st, "gbpf_solve_traced")
        out = dict(status=r.status, converged=bool(r.converged), iterations=r.iterations,
                   n_events=r.n_events, nPQlim=r.nPQlim, final_mismatch=r.final_mismatch)
        out.update(self.state())
        out["events"] = self.events()
        out["hist"] = self.history()
        out.update(self.flows())
        out["trace"] = recs
        return out

    def set_start(self, V0=None, theta0=None, Pliq=None, Qliq=None):
        arrs = [_f64(a) for a in (V0, theta0, Pliq, Qliq)]
        _check(lib().gbpf_solver_set_start(self.h, *[_p(a) for a in arrs]), "gbpf_solver_set_start")

    def state(self):
        n = self.grid.nB
        a = [np.zeros(n) for _ in range(4)]
        _check(lib().gbpf_solver_state(self.h, *[_p(x) for x in a]), "gbpf_solver_state")
        return dict(zip(("V", "theta", "Pcalc", "Qcalc"), a))

    def flows(self):
        m = self.grid.nL
        a = [np.zeros(m) for _ in range(4)]
        _check(lib().gbpf_solver_flows(self.h, *[_p(x) for x in a]), "gbpf_solver_flows")
        return dict(zip(("Pdp", "Ppd", "Qdp", "Qpd"), a))

    def events(self, cap=4096):
        ev = np.zeros(4 * cap, np.int32)
        n = ctypes.c_int()
        st = lib().gbpf_solver_events(self.h, _p(ev), cap, ctypes.byref(n))
        if st not in (OK, E_ARG):
            raise GbpfError(st, "gbpf_solver_events")
        return [tuple(int(x) for x in ev[4 * i:4 * i + 4]) for i in range(n.value)]

    def history(self):
        cap = self.options.no_max_iter + 2
        h = np.zeros(cap)
        n = ctypes.c_int()
        _check(lib().gbpf_solver_history(self.h, _p(h), cap, ctypes.byref(n)), "gbpf_solver_history")
        return h[:n.value].copy()

    def triggers(self):
        cap = self.options.no_max_iter + 2
        t = np.zeros(cap, np.int32)
        n = ctypes.c_int()
        _check(lib().gbpf_solver_triggers(self.h, _p(t), cap, ctypes.byref(n)), "gbpf_solver_triggers")
        return t[:n.value].copy()

    def set_lu_launch(self, mode):
        """gbpf_solver_set_lu_launch: 0 auto, 1 one kernel per level (heavy
        levels as pivots + entries), 2 all levels in one single-block kernel,
        3 as 1 with heavy levels one block per step."""
        _check(lib().gbpf_solver_set_lu_launch(self.h, int(mode)), "gbpf_solver_set_lu_launch")

    def set_plan(self, lu1=-1, narrow=-1, quad=-1):
        """gbpf_solver_set_plan: the persistent form's LU plan (lu1 one-pass
        levels, narrow one-warp levels on warp 0, quad FP64 blocks on four
        lanes); -1 keeps a knob.  Returns the plan in force as a dict."""
        out = np.zeros(3, np.int32)
        _check(lib().gbpf_solver_set_plan(self.h, int(lu1), int(narrow), int(quad), _p(out)),
               "gbpf_solver_set_plan")
        return dict(lu1=int(out[0]), narrow=int(out[1]), quad=int(out[2]))

    def set_form(self, form):
        """gbpf_solver_set_form: FORM_GRAPH (per-phase kernels in a CUDA graph)
        or FORM_PERSISTENT (the whole Newton loop in one block-kernel launch)."""
        _check(lib().gbpf_solver_set_form(self.h, int(form)), "gbpf_solver_set_form")

    def form(self):
        """gbpf_solver_get_form: the form gbpf_solve runs and its kernel
        launches per solve (plus, for the graph form, per iteration)."""
        a = np.zeros(3, np.int32)
        _check(lib().gbpf_solver_get_form(self.h, _p(a)), "gbpf_solver_get_form")
        return dict(form=int(a[0]), launches=int(a[1]), launches_per_iteration=int(a[2]))

    def info(self):
        a = np.zeros(8, np.int64)
        _check(lib().gbpf_solver_info(self.h, _p(a)), "gbpf_solver_info")
        keys = ("nB", "blocks", "factor_blocks", "update_pairs", "forward_levels", "backward_levels",
                "graph_nodes", "kernels_per_iteration")
        return dict(zip(keys, (int(x) for x in a)))

    def time(self, repeats):
        ms = ctypes.c_double()
        _check(lib().gbpf_solver_time(self.h, int(repeats), ctypes.byref(ms)), "gbpf_solver_time")
        return ms.value

    def profile(self, repeats=20):
        ms = np.zeros(4)
        by = np.zeros(4, np.int64)
        _check(lib().gbpf_solver_profile(self.h, int(repeats), _p(ms), _p(by)), "gbpf_solver_profile")
        if int(self.options.metodo) == METODO["denso"]:
            names = ("injections_mismatch", "dense_fill", "dense_lu", "dense_solve")
        else:
            names = ("injections_mismatch", "jacobian_fill", "factor_forward", "backward")
        return {k: dict(ms=float(m), bytes=int(b)) for k, m, b in zip(names, ms, by)}

    # kernel-level entry points
    def ybus(self):
        n, nnz = self.grid.nB, self.grid.nnzY
        rp = np.zeros(n + 1, np.int32)
        c = np.zeros(nnz, np.int32)
        re = np.zeros(nnz)
        im = np.zeros(nnz)
        _check(lib().gbpf_ybus(self.h, _p(rp), _p(c), _p(re), _p(im)), "gbpf_ybus")
        return rp, c, re, im

    def eval_pq(self, V, theta):
        V, theta = _f64(V), _f64(theta)
        P = np.zeros(self.grid.nB)
        Q = np.zeros(self.grid.nB)
        _check(lib().gbpf_eval_pq(self.h, _p(V), _p(theta), _p(P), _p(Q)), "gbpf_eval_pq")
        return P, Q

    def eval_jacobian(self, V, theta, limQ=None):
        V, theta = _f64(V), _f64(theta)
        limQ = _i32(np.zeros(self.grid.nPV, np.int32) if limQ is None else limQ)
        cap = 4 * self.grid.nnzY + 16
        row = np.zeros(cap, np.int32)
        col = np.zeros(cap, np.int32)
        val = np.zeros(cap)
        n = ctypes.c_int()
        _check(lib().gbpf_eval_jacobian(self.h, _p(V), _p(theta), _p(limQ), _p(row), _p(col), _p(val), cap,
                                        ctypes.byref(n)), "gbpf_eval_jacobian")
        k = n.value
        return row[:k].copy(), col[:k].copy(), val[:k].copy()

    def newton_step(self, V, theta, g, limQ=None):
        V, theta, g = _f64(V), _f64(theta), _f64(g)
        limQ = _i32(np.zeros(self.grid.nPV, np.int32) if limQ is None else limQ)
        dx = np.zeros_like(g)
        _check(lib().gbpf_newton_step(self.h, _p(V), _p(theta), _p(limQ), _p(g), _p(dx)), "gbpf_newton_step")
        return dx


# ---------------------------------------------------------------------- batch
class Batch:
    """Many scenarios of one or several topologies, solved in one persistent
    launch (one thread block per instance at a time)."""

    def __init__(self, grids, options=None, device=0, **overrides):
        o = options if options is not None else Options()
        for k, v in overrides.items():
            setattr(o, k, v)
        self.grids = list(grids)
        self.options = o
        arr = (ctypes.c_void_p * len(self.grids))(*[g.h.value for g in self.grids])
        self.h = ctypes.c_void_p()
        _check(lib().gbpf_batch_create(arr, len(self.grids), ctypes.byref(o._o), int(device), ctypes.byref(self.h)),
               "gbpf_batch_create")
        self.n_inst = 0
        self.offsets = None

    def close(self):
        if getattr(self, "h", None):
            lib().gbpf_batch_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_instances(self, grid_of_inst, Pload=None, Qload=None, Pg=None, Qg=None, V0=None, theta0=None):
        gi = _i32(grid_of_inst)
        prev = getattr(self, "grid_of_inst", None)
        if prev is None or prev.shape != gi.shape or not np.array_equal(prev, gi):
            nbs = np.array([g.nB for g in self.grids], np.int64)
            self.offsets = np.concatenate([[0], np.cumsum(nbs[gi])])
            self.grid_of_inst = gi.copy()
        arrs = [_f64(a) for a in (Pload, Qload, Pg, Qg, V0, theta0)]
        for a in arrs:
            if a is not None and len(a) != self.offsets[-1]:
                raise ValueError("packed bus arrays must have sum(nB) entries")
        _check(lib().gbpf_batch_set_instances(self.h, len(gi), _p(gi), *[_p(a) for a in arrs]),
               "gbpf_batch_set_instances")
        self.n_inst = len(gi)

    def solve(self):
        _check(lib().gbpf_batch_solve(self.h), "gbpf_batch_solve")

    def launch(self):
        """gbpf_batch_launch: the solve without waiting for it."""
        _check(lib().gbpf_batch_launch(self.h), "gbpf_batch_launch")

    def wait(self):
        _check(lib().gbpf_batch_wait(self.h), "gbpf_batch_wait")

    def time(self, repeats):
        ms = ctypes.c_double()
        _check(lib().gbpf_batch_time(self.h, int(repeats), ctypes.byref(ms)), "gbpf_batch_time")
        return ms.value

    def kernel_times(self, repeats=3):
        """Device ms per launch of each kernel of the batch graph: block,
        warp, hand-off (gbpf_batch_kernel_times)."""
        ms = np.zeros(3)
        _check(lib().gbpf_batch_kernel_times(self.h, int(repeats), _p(ms)), "gbpf_batch_kernel_times")
        return dict(block=float(ms[0]), warp=float(ms[1]), handoff=float(ms[2]))

    def results(self, state=True, out=None):
        """Per-instance results and (state=True) the packed V, theta, Pcalc,
        Qcalc.  out: the dict of an earlier call of the same batch, whose
        arrays are filled in place (no new allocation per solve)."""
        n, nb = self.n_inst, int(self.offsets[-1])

        def arr(key, size, dt):
            a = out.get(key) if out else None
            return a if a is not None and a.shape == (size,) and a.dtype == dt else np.empty(size, dt)

        it = arr("iterations", n, np.int32)
        st = arr("status", n, np.int32)
        mm = arr("final_mismatch", n, np.float64)
        ne = arr("n_events", n, np.int32)
        V = arr("V", nb, np.float64) if state else None
        th = arr("theta", nb, np.float64) if state else None
        P = arr("Pcalc", nb, np.float64) if state else None
        Q = arr("Qcalc", nb, np.float64) if state else None
        _check(lib().gbpf_batch_results(self.h, _p(it), _p(st), _p(mm), _p(ne), _p(V), _p(th), _p(P), _p(Q)),
               "gbpf_batch_results")
        return dict(iterations=it, status=st, final_mismatch=mm, n_events=ne, V=V, theta=th, Pcalc=P, Qcalc=Q)

    def events(self, inst, cap=16):
        ev = np.zeros(4 * cap, np.int32)
        n = ctypes.c_int()
        st = lib().gbpf_batch_events(self.h, int(inst), _p(ev), cap, ctypes.byref(n))
        if st not in (OK, E_ARG):
            raise GbpfError(st, "gbpf_batch_events")
        return [tuple(int(x) for x in ev[4 * i:4 * i + 4]) for i in range(n.value)]

    def events_all(self, cap=16):
        """Switch events of every instance (gbpf_batch_events_all): an array
        [n_inst, cap, 4] (iteration, bus, PV position, code; zero-padded) and
        the per-instance event counts."""
        ev = np.zeros(self.n_inst * cap * 4, np.int32)
        n = np.zeros(self.n_inst, np.int32)
        _check(lib().gbpf_batch_events_all(self.h, _p(ev), int(cap), _p(n)), "gbpf_batch_events_all")
        return ev.reshape(self.n_inst, cap, 4), n

    PLAN_KEYS = ("warp_mode", "warps_per_block", "handoff_it", "resume_group", "warp_group", "narrow", "lu1",
                 "warp_lu1", "flat_shared", "rotate", "gstate", "warp_gstate", "warps_per_block_used",
                 "warp_instances", "block_instances", "block_state_global", "warp_state_global")

    def plan(self):
        """The launch plan (gbpf_batch_get_plan)."""
        a = np.zeros(20, np.int32)
        _check(lib().gbpf_batch_get_plan(self.h, _p(a)), "gbpf_batch_get_plan")
        return dict(zip(self.PLAN_KEYS, (int(x) for x in a)))

    def set_plan(self, warp_mode=1, warps_per_block=8, handoff_it=12, resume_group=1, warp_group=1, narrow=0,
                 lu1=1, warp_lu1=0, flat_shared=1, rotate=0, gstate=1, warp_gstate=1):
        a = np.array([warp_mode, warps_per_block, handoff_it, resume_group, warp_group, narrow, lu1, warp_lu1,
                      flat_shared, rotate, gstate, warp_gstate], np.int32)
        _check(lib().gbpf_batch_set_plan(self.h, _p(a)), "gbpf_batch_set_plan")

    def autotune(self, repeats=3):
        """Coordinate search over the launch plan on the current instances;
        returns (plan, ms of the starting plan, ms of the chosen plan)."""
        a = np.zeros(20, np.int32)
        ms = np.zeros(2, np.float32)
        _check(lib().gbpf_batch_autotune(self.h, int(repeats), _p(a), _p(ms)), "gbpf_batch_autotune")
        return dict(zip(self.PLAN_KEYS, (int(x) for x in a))), float(ms[0]), float(ms[1])

    def info(self):
        a = np.zeros(8, np.int64)
        _check(lib().gbpf_batch_info(self.h, _p(a)), "gbpf_batch_info")
        keys = ("topologies", "instances", "buses", "blocks", "smem_bytes", "factors_in_smem",
                "scratch_bytes_per_block", "warp_instances")
        return dict(zip(keys, (int(x) for x in a)))

    def solve_noalloc(self, grid_of_inst, V0, theta0, Pliq, Qliq, Qload, V, theta, Pcalc, Qcalc,
                      iterations, status, final_mismatch, stream=0):
        """gbpf_batch_solve_noalloc: every array argument except grid_of_inst
        is a device address (int); asynchronous on `stream`."""
        gi = _i32(grid_of_inst)
        vp = ctypes.c_void_p
        _check(lib().gbpf_batch_solve_noalloc(
            self.h, len(gi), _p(gi), vp(V0), vp(theta0), vp(Pliq), vp(Qliq), vp(Qload), vp(V), vp(theta),
            vp(Pcalc), vp(Qcalc), vp(iterations), vp(status), vp(final_mismatch), vp(stream)),
            "gbpf_batch_solve_noalloc")

    def follow(self, prev):
        """gbpf_batch_follow: this batch's next warm-started solve starts on
        the device after prev's last one has ended."""
        _check(lib().gbpf_batch_follow(self.h, prev.h), "gbpf_batch_follow")

    def solve_warm_launch(self, mlp):
        """gbpf_batch_solve_warm_launch: the warm-started solve without
        waiting for it; solve_warm_wait() returns what solve_warm returns."""
        _check(lib().gbpf_batch_solve_warm_launch(self.h, mlp.h), "gbpf_batch_solve_warm_launch")

    def solve_warm_wait(self):
        kind = np.zeros(self.n_inst, np.int32)
        wit = np.zeros(self.n_inst, np.int32)
        ms = ctypes.c_double()
        _check(lib().gbpf_batch_solve_warm_wait(self.h, _p(kind), _p(wit), ctypes.byref(ms)),
               "gbpf_batch_solve_warm_wait")
        ph = np.zeros(3)
        _check(lib().gbpf_batch_warm_phases(self.h, _p(ph)), "gbpf_batch_warm_phases")
        return dict(start_kind=kind, warm_iterations=wit, ms=ms.value,
                    phases_ms=dict(network=ph[0], start_choice=ph[1], newton=ph[2]))

    def solve_warm(self, mlp):
        """gbpf_batch_solve_warm: Newton from the network's predicted start
        (flat-start fallback).  Returns start_kind (0 own start, 1 predicted
        start converged, 2 predicted start failed and was replaced),
        warm_iterations, the device time in ms and its phases
        (gbpf_batch_warm_phases)."""
        kind = np.zeros(self.n_inst, np.int32)
        wit = np.zeros(self.n_inst, np.int32)
        ms = ctypes.c_double()
        _check(lib().gbpf_batch_solve_warm(self.h, mlp.h, _p(kind), _p(wit), ctypes.byref(ms)),
               "gbpf_batch_solve_warm")
        ph = np.zeros(3)
        _check(lib().gbpf_batch_warm_phases(self.h, _p(ph)), "gbpf_batch_warm_phases")
        return dict(start_kind=kind, warm_iterations=wit, ms=ms.value,
                    phases_ms=dict(network=ph[0], start_choice=ph[1], newton=ph[2]))

    def slice(self, arr, inst):
        return arr[self.offsets[inst]:self.offsets[inst + 1]]


# ---------------------------------------------------------------- warm start
def warm_features(Pliq, Qliq, V0=None):
    """Network features of scenarios of one grid: rows [Pliq | Qliq | V0]
    (arrays [n, nB] or [nB]), or [Pliq | Qliq] without V0 (a network of
    2 nB inputs, for scenarios whose starting voltages do not vary)."""
    cols = [np.atleast_2d(Pliq), np.atleast_2d(Qliq)] + ([] if V0 is None else [np.atleast_2d(V0)])
    return np.concatenate(cols, axis=1).astype(np.float32)


def warm_targets(V, theta):
    """Network outputs of solved scenarios: rows [|V| | theta]."""
    return np.concatenate([np.atleast_2d(V), np.atleast_2d(theta)], axis=1).astype(np.float32)


def warm_loss_metric(solver, V, theta, out_scale):
    """A for MLP.set_loss_metric: S J0^T with J0 the Newton Jacobian at
    (V, theta) (a typical solution, e.g. the mean of the training targets)
    and S taking normalised outputs [|V| | theta] (scaled by out_scale) to
    J0's columns (theta of non-slack buses, |V| of PQ buses); scaled so that
    |A|_F^2 = n_out.  e A is then the linearised mismatch of a start whose
    normalised error is e."""
    g = solver.grid
    nB = g.nB
    row, col, val = solver.eval_jacobian(V, theta)
    types = g.buses()["type"]
    ns = np.where(types != 3)[0]
    pq = np.where(types <= 1)[0]
    dim = len(ns) + len(pq)
    out_of_col = np.concatenate([nB + ns, pq])
    scale = np.asarray(out_scale, np.float64)[out_of_col]
    J = np.zeros((dim, dim))
    np.add.at(J, (row, col), val)
    A = np.zeros((2 * nB, dim))
    A[out_of_col] = scale[:, None] * J.T
    A *= np.sqrt((2 * nB) / max(np.sum(A * A), 1e-300))
    return A.astype(np.float32)


class MLP:
    """The warm-start network (gbpf_mlp_*): n_in -> n_layers x width (GELU) ->
    n_out, trained on the GPU by the library's tensor-core kernels."""

    def __init__(self, n_in, n_out, width=512, n_layers=3, skip=True, seed=0, device=0):
        self.h = ctypes.c_void_p()
        _check(lib().gbpf_mlp_create(int(n_in), int(width), int(n_layers), int(n_out), int(bool(skip)),
                                     ctypes.c_ulonglong(seed), int(device), ctypes.byref(self.h)), "gbpf_mlp_create")
        self.n_in, self.n_out, self.width, self.n_layers = int(n_in), int(n_out), int(width), int(n_layers)
        self.skip = bool(skip)

    def close(self):
        if getattr(self, "h", None):
            lib().gbpf_mlp_free(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def layer_shapes(self):
        """(out, in) of every layer, the skip last when present."""
        dims = [self.n_in] + [self.width] * self.n_layers + [self.n_out]
        return [(dims[i + 1], dims[i]) for i in range(self.n_layers + 1)] + ([(self.n_out, self.n_in)] if self.skip else [])

    def set_data(self, X, Y):
        X = np.ascontiguousarray(X, np.float32)
        Y = np.ascontiguousarray(Y, np.float32)
        _check(lib().gbpf_mlp_set_data(self.h, _p(X), _p(Y), len(X)), "gbpf_mlp_set_data")

    def train(self, epochs, batch=256, lr=1e-3, lr_final=None, seed=0):
        """Adam from lr, decaying along a cosine to lr_final (default: lr,
        i.e. constant); returns (mean loss per epoch, device ms)."""
        loss = np.zeros(max(1, epochs), np.float32)
        ms = ctypes.c_double()
        lf = lr if lr_final is None else lr_final
        _check(lib().gbpf_mlp_train(self.h, int(epochs), int(batch), ctypes.c_float(lr), ctypes.c_float(lf),
                                    ctypes.c_ulonglong(seed), _p(loss), ctypes.byref(ms)), "gbpf_mlp_train")
        return loss[:epochs], ms.value

    def set_loss_metric(self, A=None, lam=0.01):
        """Loss (|e A|^2 + lam |e|^2) / (rows * n_out) on the normalised
        residual e, A [n_out, k]; A None: mean squared error."""
        Ac = None if A is None else np.ascontiguousarray(A, np.float32)
        k = 0 if A is None else Ac.shape[1]
        _check(lib().gbpf_mlp_set_loss_metric(self.h, _p(Ac), int(k), ctypes.c_float(lam)),
               "gbpf_mlp_set_loss_metric")

    def set_wait_limit(self, cycles=0):
        """gbpf_mlp_set_wait_limit: the GEMMs' operand-ring wait limit in SM
        clock cycles (0: the default, about 2 s)."""
        _check(lib().gbpf_mlp_set_wait_limit(self.h, ctypes.c_longlong(int(cycles))), "gbpf_mlp_set_wait_limit")

    def predict(self, X):
        X = np.ascontiguousarray(np.atleast_2d(X), np.float32)
        Y = np.zeros((len(X), self.n_out), np.float32)
        _check(lib().gbpf_mlp_predict(self.h, _p(X), len(X), _p(Y)), "gbpf_mlp_predict")
        return Y

    def gradients(self, Xn, Yn):
        """Loss and per-layer (dW, db) on normalised rows, without an update
        (the skip, when present, last with db None)."""
        Xn = np.ascontiguousarray(Xn, np.float32)
        Yn = np.ascontiguousarray(Yn, np.float32)
        shapes = self.layer_shapes()
        nl = self.n_layers + 1
        dW = np.zeros(sum(o * i for o, i in shapes), np.float32)
        db = np.zeros(sum(o for o, _ in shapes[:nl]), np.float32)
        loss = ctypes.c_float()
        _check(lib().gbpf_mlp_gradients(self.h, _p(Xn), _p(Yn), len(Xn), ctypes.byref(loss), _p(dW), _p(db)),
               "gbpf_mlp_gradients")
        out, ow, ob = [], 0, 0
        for l, (o, i) in enumerate(shapes):
            out.append((dW[ow:ow + o * i].reshape(o, i), db[ob:ob + o] if l < nl else None))
            ow += o * i
            ob += o
        return loss.value, out

    def params(self):
        """[(W, b)] of every layer; the skip, when present, last as (S, None)."""
        out = []
        nl = self.n_layers + 1
        for l, (o, i) in enumerate(self.layer_shapes()):
            W = np.zeros((o, i), np.float32)
            b = np.zeros(o, np.float32) if l < nl else None
            _check(lib().gbpf_mlp_params(self.h, l, _p(W), _p(b)), "gbpf_mlp_params")
            out.append((W, b))
        return out

    def set_params(self, params):
        for l, (W, b) in enumerate(params):
            W = np.ascontiguousarray(W, np.float32)
            b = None if b is None else np.ascontiguousarray(b, np.float32)
            _check(lib().gbpf_mlp_set_params(self.h, l, _p(W), _p(b)), "gbpf_mlp_set_params")

    def norm(self):
        a, b = np.zeros(self.n_in, np.float32), np.zeros(self.n_in, np.float32)
        c, d = np.zeros(self.n_out, np.float32), np.zeros(self.n_out, np.float32)
        _check(lib().gbpf_mlp_norm(self.h, _p(a), _p(b), _p(c), _p(d)), "gbpf_mlp_norm")
        return dict(in_mean=a, in_scale=b, out_mean=c, out_scale=d)

    def set_norm(self, in_mean, in_scale, out_mean, out_scale):
        arrs = [np.ascontiguousarray(x, np.float32) for x in (in_mean, in_scale, out_mean, out_scale)]
        _check(lib().gbpf_mlp_set_norm(self.h, *[_p(x) for x in arrs]), "gbpf_mlp_set_norm")
