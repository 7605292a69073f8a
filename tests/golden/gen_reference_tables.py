"""Generates tests/golden/ref_tables_d{D}.npz from the reference's own host code.

Runs oracle/ref_build.sh (compiles the reference's FunctionData/PPolynomial host
code, read in place from the reference tree, with oracle/ref_tables_driver.cu)
and stores, for each maxDepth, the non-zero entries of the three inner-product
tables (dotTable, dDotTable, d2DotTable, FunctionData.inl:159-205) and the
normalised base function F/F(0).

Usage:  python tests/golden/gen_reference_tables.py [depth ...]   (default 5 8)
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))


def main(depths):
    exe = subprocess.check_output(["sh", os.path.join(REPO, "oracle", "ref_build.sh")], text=True).strip()
    for D in depths:
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "t.bin")
            out = subprocess.check_output([exe, str(D), path], text=True)
            res = (1 << (D + 1)) - 1
            t = np.fromfile(path, dtype=np.float64).reshape(3, res * res)
        pieces = np.array([[float.fromhex(x) for x in line.split()] for line in out.strip().splitlines()],
                          dtype=np.float64)
        arrs = {"res": np.int64(res), "base_function": pieces}
        for name, tab in zip(("dot", "ddot", "d2dot"), t):
            idx = np.nonzero(tab)[0].astype(np.int64)
            arrs[name + "_idx"] = idx
            arrs[name + "_val"] = tab[idx]
        np.savez_compressed(os.path.join(HERE, "ref_tables_d%d.npz" % D), **arrs)
        print("depth", D, {k: v.shape for k, v in arrs.items()})


if __name__ == "__main__":
    main([int(a) for a in sys.argv[1:]] or [5, 8])
