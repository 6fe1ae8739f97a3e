"""Regenerates the golden fixtures in this directory.

Every expected output here comes from the reference's own solve-path code:
oracle/_ref/ref_nr, built by oracle/ref/Makefile from the reference's CPU/ tree
sources (reader, Ybus, injections, Jacobian pattern and values) with a driver
that replays the reference GPU Newton loop and its limit rules.  Inputs are

* the synthetic grids written here (c1.cdf: 14-bus, c2_*.cdf: 118-bus), which
  are committed so that the GPU machine, which has no reference checkout, reads the
  very same bytes, and
* the reference's IEEE cases, read in place from the reference checkout (only
  their solutions are stored, as ieee_*.json).

Run from the repository root after building the library and the harness:
    python -c "import __graft_entry__ as g; g.build()"
    python tests/golden/make_golden.py [/path/to/reference]
"""
import importlib
import json
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
gb = importlib.import_module("experience-of-using-gpu-in-power-flow-computation_gb300")

REF_NR = os.path.join(ROOT, "oracle", "_ref", "ref_nr")
BASE_SEED = 20261203
IEEE = ["ieee14", "ieee30", "ieee57", "ieee118", "ieee118x2", "ieee118x4", "ieee118x8"]
STATE_KEYS = ("V", "theta", "Pcalc", "Qcalc", "Pdp", "Ppd", "Qdp", "Qpd")


def run_ref(path, tol, maxit, lim):
    out = subprocess.run([REF_NR, path, repr(tol), str(maxit), str(int(lim))], capture_output=True,
                         text=True, check=True).stdout
    r = json.loads(out)
    r.pop("Y_re", None)
    r.pop("Y_im", None)
    r["file"] = os.path.basename(path)
    return r


def write(name, rec):
    with open(os.path.join(HERE, name), "w") as f:
        json.dump(rec, f, indent=0, separators=(",", ":"))
        f.write("\n")


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
    index = []
    for name, tol, maxit, lim in cases:
        r = run_ref(os.path.join(HERE, name), tol, maxit, lim)
        out = f"{os.path.splitext(name)[0]}_lim{lim}.json"
        write(out, r)
        index.append(dict(cdf=name, golden=out, tol=tol, max_iter=maxit, lim=lim, iterations=r["iterations"],
                          events=len(r["events"])))
    # IEEE cases of the reference, solutions only
    for case in IEEE:
        path = os.path.join(ref_root, "GPU", case + ".cdf")
        if not os.path.exists(path):
            continue
        for lim in (0, 1):
            r = run_ref(path, 1e-8, 100, lim)
            if not r["converged"]:  # diverging switch cycles: keep the history, not the state
                for k in STATE_KEYS:
                    r.pop(k, None)
                r["events"] = r["events"][:40]
            out = f"ieee_{case}_lim{lim}.json"
            write(out, r)
            index.append(dict(cdf=case + ".cdf", golden=out, tol=1e-8, max_iter=100, lim=lim,
                              iterations=r["iterations"], events=len(r["events"])))
    with open(os.path.join(HERE, "index.json"), "w") as f:
        json.dump(index, f, indent=1)
        f.write("\n")
    print(json.dumps(index, indent=1))


if __name__ == "__main__":
    main()
