"""In-tree build of libgbpf.so and the gbpf command-line driver for sm_103a.

Compiles the C++ host units with g++ and the CUDA units with nvcc
(-gencode arch=compute_103a,code=sm_103a), in parallel, into ``lib/`` next to
this file.  No cmake; a rebuild happens only when a source is newer than the
library.  nvcc cross-compiles without a GPU, so this also runs on CPU-only hosts.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB_DIR = os.path.join(HERE, "lib")
LIB = os.path.join(LIB_DIR, "libgbpf.so")
CLI = os.path.join(LIB_DIR, "gbpf")

ARCH = "-gencode=arch=compute_103a,code=sm_103a"
CXX_UNITS = ["host_io.cpp", "symbolic.cpp", "capi_misc.cpp"]
CU_UNITS = ["solver.cu", "batch.cu", "mlp.cu"]


def _cuda_home():
    for c in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if c and os.path.exists(os.path.join(c, "bin", "nvcc")):
            return c
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found: set CUDA_HOME")


def _sources():
    units = [u for u in CXX_UNITS + CU_UNITS if os.path.exists(os.path.join(CSRC, u))]
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers.append(os.path.join(INCLUDE, "gbpf.h"))
    return units, headers


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def build(verbose=False, force=False):
    """Builds lib/libgbpf.so and lib/gbpf; returns the library path."""
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    units, headers = _sources()
    jobs = []
    objs = []
    for u in units:
        src = os.path.join(CSRC, u)
        obj = os.path.join(BUILD, u + ".o")
        objs.append(obj)
        if not force and not _stale(obj, [src] + headers):
            continue
        if u.endswith(".cu"):
            cmd = [nvcc, ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                   "-I" + INCLUDE, "-I" + CSRC, "-c", src, "-o", obj]
            if verbose:
                cmd.insert(1, "-Xptxas=-v")
        else:
            cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-Wall", "-Wno-unused-function",
                   "-I" + INCLUDE, "-I" + CSRC, "-I" + os.path.join(cuda, "include"), "-c", src, "-o", obj]
        jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or _stale(LIB, objs):
        _run([nvcc, ARCH, "-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"])
    cli_src = os.path.join(CSRC, "cli.cpp")
    if os.path.exists(cli_src) and (force or _stale(CLI, [cli_src, LIB] + headers)):
        _run(["g++", "-O2", "-std=c++17", "-I" + INCLUDE, cli_src, "-o", CLI,
              "-L" + LIB_DIR, "-lgbpf", "-Wl,-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    print(LIB)
