"""Regenerates the golden fixtures in this directory.

Every expected output here comes from the reference's own solve-path code:
oracle/_ref/ref_nr, built by oracle/ref/Makefile from the reference's CPU/ tree
sources (reader, Ybus, injections, Jacobian pattern and values) with a driver
that replays the reference GPU Newton loop and its limit rules.  Inputs are

* the synthetic grids written here (c1.cdf: 14-bus, c2_*.cdf: 118-bus, and the
  MATPOWER cases m_edge.m and c2_tx.m), which are committed so that the GPU
  box, which has no reference checkout, reads the very same bytes, and
* the reference's IEEE cases (GPU/ieee14.cdf ... GPU/ieee118x64.cdf), copied
  byte for byte from the reference checkout into ieee/*.cdf.gz (gzip, no name
  or time stamp, so a rerun writes the same bytes), so that the GPU tests read
  the reference's own inputs; their solutions are ieee_*.json (.json.gz above
  1,000 buses).

Run from the repository root after building the library and the harness:
    python -c "import __graft_entry__ as g; g.build()"
    python tests/golden/make_golden.py [/path/to/reference]
"""
import gzip
import importlib
import json
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
gb = importlib.import_module("experience-of-using-gpu-in-power-flow-computation_gb300")

REF_NR = os.path.join(ROOT, "oracle", "_ref", "ref_nr")
BASE_SEED = 20261203
IEEE = ["ieee14", "ieee30", "ieee57", "ieee118", "ieee118x2", "ieee118x4", "ieee118x8", "ieee118x16", "ieee118x32",
        "ieee118x64"]
IEEE_DIR = os.path.join(HERE, "ieee")
STATE_KEYS = ("V", "theta", "Pcalc", "Qcalc", "Pdp", "Ppd", "Qdp", "Qpd")


def run_ref(path, tol, maxit, lim):
    out = subprocess.run([REF_NR, path, repr(tol), str(maxit), str(int(lim))], capture_output=True,
                         text=True, check=True).stdout
    r = json.loads(out)
    if not path.endswith(".m"):  # .m cases keep calcYbusSp_Matpower's values
        r.pop("Y_re", None)
        r.pop("Y_im", None)
    r["file"] = os.path.basename(path)
    return r


# A hand-written MATPOWER case for the reader's corner cases: non-consecutive
# bus ids, a generator row on a PQ bus (never looked up), two generator rows on
# one PV bus (the first is used), a repeated branch (kept as two branches), a
# transformer with line charging (where calcYbusSp_Matpower's from-side
# (1/z + jb/2)/|t|^2 differs from the CDF form), a phase shifter written with
# ratio 0, comments, a blank line and a gencost block the reader skips.
M_EDGE = """function mpc = m_edge
%% six buses, eight branches
mpc.version = '2';
mpc.baseMVA = 100;

%% bus data
%\tbus_i\ttype\tPd\tQd\tGs\tBs\tarea\tVm\tVa\tbaseKV\tzone\tVmax\tVmin
mpc.bus = [
\t10\t3\t0\t0\t0\t0\t1\t1.02\t5\t230\t1\t1.1\t0.9;
\t20\t2\t20\t10\t0\t0\t1\t1.01\t0\t230\t1\t1.1\t0.9;
\t30\t1\t45\t15\t0\t0\t1\t1\t0\t230\t1\t1.1\t0.9;\t% a generator row names this PQ bus
\t40\t1\t40\t5\t0\t19\t1\t1\t0\t230\t1\t1.1\t0.9;

\t50\t2\t10\t3\t0\t0\t1\t0.995\t0\t230\t1\t1.1\t0.9;
\t60\t1\t60\t12\t2\t-5\t1\t1\t0\t230\t1\t1.1\t0.9;
];

%% generator data
mpc.gen = [
\t10\t0\t0\t300\t-300\t1.02\t100\t1\t300\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0;
\t20\t40\t0\t30\t-10\t1.01\t100\t1\t100\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0;
\t30\t25\t5\t10\t-10\t1\t100\t1\t50\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0;
\t50\t30\t0\t25\t-5\t0.995\t100\t1\t60\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0;
\t50\t99\t0\t99\t-99\t1\t100\t1\t99\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0\t0;
];

%% branch data
%\tfbus\ttbus\tr\tx\tb\trateA\trateB\trateC\tratio\tangle\tstatus\tangmin\tangmax
mpc.branch = [
\t10\t20\t0.01\t0.06\t0.05\t0\t0\t0\t0\t0\t1\t-360\t360;
\t10\t20\t0.02\t0.08\t0.04\t0\t0\t0\t0\t0\t1\t-360\t360;
\t20\t30\t0.005\t0.05\t0.03\t0\t0\t0\t0.97\t0\t1\t-360\t360;
% a phase shifter written with ratio 0
\t30\t40\t0\t0.04\t0\t0\t0\t0\t0\t-3\t1\t-360\t360;
\t40\t50\t0.02\t0.1\t0.02\t0\t0\t0\t1.03\t2\t1\t-360\t360;
\t50\t60\t0.015\t0.07\t0.02\t0\t0\t0\t0\t0\t1\t-360\t360;
\t60\t10\t0.01\t0.05\t0.03\t0\t0\t0\t0\t0\t1\t-360\t360;
\t20\t60\t0.03\t0.12\t0.025\t0\t0\t0\t0\t0\t1\t-360\t360;
];

%% generator cost data
mpc.gencost = [
\t2\t0\t0\t3\t0.01\t40\t0;
];
"""


def with_transformer_charging(grid):
    """The grid with line charging on its off-nominal-tap branches, so that the
    two Ybus forms differ (same buses and branches otherwise)."""
    b, br, pv = grid.buses(), grid.branches(), grid.pvpq()
    tap = np.hypot(br["tap_re"], br["tap_im"])
    bch = np.where(np.abs(tap - 1) > 1e-12, 0.04, br["bch"])
    qmax = np.zeros(grid.nB)
    qmin = np.zeros(grid.nB)
    qmax[pv["pv"] - 1] = pv["Qmax"]
    qmin[pv["pv"] - 1] = pv["Qmin"]
    return gb.create_grid(b["type"], b["V0"], b["theta0"], br["from_bus"], br["to_bus"], br["r"], br["x"], bch,
                          br["tap_re"], br["tap_im"], br["phase"], b["Pload"], b["Qload"], b["Pg"], b["Qg"],
                          b["gsh"], b["bsh"], qmax, qmin, b["id"], grid.baseMVA)


def write(name, rec):
    text = json.dumps(rec, indent=0, separators=(",", ":")) + "\n"
    if name.endswith(".gz"):
        with open(os.path.join(HERE, name), "wb") as f:
            f.write(gzip.compress(text.encode(), compresslevel=9, mtime=0))
    else:
        with open(os.path.join(HERE, name), "w") as f:
            f.write(text)


def copy_fixture(src, case):
    """The reference's input file as a gzip fixture (deterministic bytes)."""
    os.makedirs(IEEE_DIR, exist_ok=True)
    with open(src, "rb") as f:
        data = f.read()
    with open(os.path.join(IEEE_DIR, case + ".cdf.gz"), "wb") as f:
        f.write(gzip.compress(data, compresslevel=9, mtime=0))
    return "ieee/" + case + ".cdf.gz"


def main():
    ref_root = sys.argv[1] if len(sys.argv) > 1 else "/root/reference"
    # synthetic 14-bus grid (config 1) and 118-bus grids (config 2); extra 118-bus
    # seeds are picked for PV->PQ switching with the limits on
    g = gb.generate(1, BASE_SEED + 1)
    g.write_cdf(os.path.join(HERE, "c1.cdf"), "config 1 14-bus")
    cases = [("c1.cdf", 1e-8, 100, 0), ("c1.cdf", 1e-8, 100, 1)]
    g = gb.generate(2, BASE_SEED + 2)
    g.write_cdf(os.path.join(HERE, "c2_base.cdf"), "config 2 118-bus")
    cases += [("c2_base.cdf", 1e-8, 100, 0), ("c2_base.cdf", 1e-8, 100, 1)]
    picked = 0
    for s in range(1, 60):
        if picked == 4:
            break
        g = gb.generate(2, BASE_SEED + 1000 * s)
        tmp = os.path.join(HERE, "_probe.cdf")
        g.write_cdf(tmp, "probe")
        r = run_ref(tmp, 1e-8, 100, 1)
        if r["converged"] and r["events"]:
            name = f"c2_s{s}.cdf"
            os.replace(tmp, os.path.join(HERE, name))
            cases += [(name, 1e-8, 100, 1)]
            picked += 1
    if os.path.exists(os.path.join(HERE, "_probe.cdf")):
        os.remove(os.path.join(HERE, "_probe.cdf"))
    # MATPOWER cases: the corner-case file above and the 118-bus base grid with
    # charged transformers, both read by the reference's own .m reader
    with open(os.path.join(HERE, "m_edge.m"), "w") as f:
        f.write(M_EDGE)
    cases += [("m_edge.m", 1e-8, 100, 0), ("m_edge.m", 1e-8, 100, 1)]
    with_transformer_charging(gb.read_grid(os.path.join(HERE, "c2_base.cdf"))).write_m(
        os.path.join(HERE, "c2_tx.m"), "config 2 118-bus, charged transformers")
    cases += [("c2_tx.m", 1e-8, 100, 0), ("c2_tx.m", 1e-8, 100, 1)]
    index = []
    for name, tol, maxit, lim in cases:
        r = run_ref(os.path.join(HERE, name), tol, maxit, lim)
        out = f"{os.path.splitext(name)[0]}_lim{lim}.json"
        write(out, r)
        index.append(dict(cdf=name, golden=out, tol=tol, max_iter=maxit, lim=lim, iterations=r["iterations"],
                          events=len(r["events"])))
    # IEEE cases of the reference: the input as a fixture, and its solutions
    for case in IEEE:
        path = os.path.join(ref_root, "GPU", case + ".cdf")
        if not os.path.exists(path):
            continue
        fixture = copy_fixture(path, case)
        for lim in (0, 1):
            r = run_ref(path, 1e-8, 100, lim)
            if not r["converged"]:  # diverging switch cycles: keep the history, not the state
                for k in STATE_KEYS:
                    r.pop(k, None)
                r["events"] = r["events"][:40]
            out = f"ieee_{case}_lim{lim}.json" + (".gz" if r.get("nB", 0) > 1000 else "")
            write(out, r)
            index.append(dict(cdf=case + ".cdf", fixture=fixture, golden=out, tol=1e-8, max_iter=100, lim=lim,
                              iterations=r["iterations"], events=len(r["events"])))
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)
        f.write("\n")
    print(json.dumps(index, indent=1))


if __name__ == "__main__":
    main()
