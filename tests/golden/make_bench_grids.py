"""Writes the benchmark's input grids as committed fixtures.

bench.py reads these files in both of its arms: the GPU arm through the
product's reader, the reference arm through the oracle's reader, so that the two
solve byte-identical inputs and the reference arm never loads the product.
Each file is the product's seeded generator output for one workload, written in
the reference's common data format (.cdf; .cdfx above 9,999 buses) and gzipped
without a name or time stamp, so that a rerun writes the same bytes:

  c2_base.cdf        118-bus config-2 grid (seed 20261203 + 2; already a golden
                     input, written by make_golden.py)
  c3_base.cdfx.gz    15,104 buses: 128 tied 118-bus copies (seed + 3)
  c4_<n>.cdf.gz      the six config-4 grids, n in 14, 30, 57, 118, 236, 472
                     buses (seed + 4 + 1000 i)
  c5_base.cdf.gz     1,888 buses: 16 tied 118-bus copies (seed + 5)

Run from the repository root after building the library:
    python tests/golden/make_bench_grids.py
"""
import gzip
import importlib
import os
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
BASE_SEED = 20261203
C4_SIZES = (14, 30, 57, 118, 236, 472)


def grids(gb):
    """(file name, generated grid) of every benchmark input."""
    out = [("c3_base.cdfx.gz", gb.generate(3, BASE_SEED + 3, tiles=128))]
    out += [(f"c4_{nb}.cdf.gz", gb.generate(4, BASE_SEED + 4 + 1000 * i, nbus=nb)) for i, nb in enumerate(C4_SIZES)]
    out += [("c5_base.cdf.gz", gb.generate(3, BASE_SEED + 5, tiles=16))]
    return out


def cdf_bytes(grid, name):
    """The grid in the reference's file format, as the bytes the writer gives."""
    d = tempfile.mkdtemp(prefix="gbpf_grid_")
    path = os.path.join(d, name[:-3])
    grid.write_cdf(path, "benchmark grid " + name[:-3])
    with open(path, "rb") as f:
        data = f.read()
    os.remove(path)
    os.rmdir(d)
    return data


def main():
    sys.path.insert(0, ROOT)
    gb = importlib.import_module("experience-of-using-gpu-in-power-flow-computation_gb300")
    for name, g in grids(gb):
        with open(os.path.join(HERE, name), "wb") as f:
            f.write(gzip.compress(cdf_bytes(g, name), compresslevel=9, mtime=0))
        print(name, g.nB, "buses", g.nL, "branches")


if __name__ == "__main__":
    main()
