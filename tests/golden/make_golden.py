"""Regenerates the committed golden fixtures from the reference tree.

Run in a container where the reference checkout exists (it is not needed at
test time):  python tests/golden/make_golden.py /path/to/faust
Writes:
  config_compared_palm2_data.npy  the 500 x 32 'data' matrix of
      misc/config_file/mat/config_compared_palm2.mat, the fixture of the
      reference's palm4msa2 test (misc/test/src/C++/palm4msa_2020.cpp.in:81-121).
  config_HADAMARD_32_params.json  the hierarchical parameters of
      misc/config_file/mat/config_HADAMARD_32.mat (the configuration of the
      reference's Hadamard factorization tests, misc/test/CMakeLists.txt:46,339):
      nfacts, niter1, niter2, update_way, nrow, ncol and the 2 x (nfacts-1)
      constraint cells as [name, parameter, rows, cols].
"""
import json
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    d = sio.loadmat(os.path.join(ref_root, "misc", "config_file", "mat", "config_compared_palm2.mat"))
    np.save(os.path.join(HERE, "config_compared_palm2_data.npy"), np.asfortranarray(d["data"], np.float64))

    p = sio.loadmat(os.path.join(ref_root, "misc", "config_file", "mat", "config_HADAMARD_32.mat"))["params"][0, 0]
    cells = p["cons"]
    cons = [[[str(c[0, 0][0]), int(c[0, 1][0, 0]), int(c[0, 2][0, 0]), int(c[0, 3][0, 0])]
             for c in cells[r]] for r in range(cells.shape[0])]
    out = {k: int(p[k][0, 0]) for k in ("nfacts", "niter1", "niter2", "update_way", "nrow", "ncol")}
    out["cons"] = cons
    with open(os.path.join(HERE, "config_HADAMARD_32_params.json"), "w") as f:
        json.dump(out, f, indent=1)
        f.write("\n")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python tests/golden/make_golden.py <path of the FAuST reference checkout>")
    main(sys.argv[1])
