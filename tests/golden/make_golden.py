"""Regenerates the committed golden fixtures from the reference tree.

Run in a container where the reference checkout exists (it is not needed at
test time):  python tests/golden/make_golden.py /path/to/faust
Writes:
  config_compared_palm2_data.npy  the 500 x 32 'data' matrix of
      misc/config_file/mat/config_compared_palm2.mat, the fixture of the
      reference's palm4msa2 test (misc/test/src/C++/palm4msa_2020.cpp.in:81-121).
"""
import os
import sys

import numpy as np
import scipy.io as sio

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    d = sio.loadmat(os.path.join(ref_root, "misc", "config_file", "mat", "config_compared_palm2.mat"))
    np.save(os.path.join(HERE, "config_compared_palm2_data.npy"), np.asfortranarray(d["data"], np.float64))


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
