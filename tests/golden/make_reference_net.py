"""Freezes the net of the reference's contact test into a fixture.

    python tests/golden/make_reference_net.py [path to the EndoBeams.jl checkout]

test/test_beams2rigid_contact_1_analytical.jl:14-18 reads its net from
test/input/pos_net.txt (node positions, one row per node) and
test/input/conn_net.txt (1-based node pairs, one row per element).  This
script reads those two files as the test does (whitespace-separated numbers)
and stores them unchanged in tests/golden/reference_net.npz, so the GPU tests
can run the reference's own contact scene where the reference tree is absent.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def main(ref_root):
    pos = np.loadtxt(os.path.join(ref_root, "test", "input", "pos_net.txt"), dtype=np.float64)
    conn = np.loadtxt(os.path.join(ref_root, "test", "input", "conn_net.txt"), dtype=np.int64)
    assert pos.ndim == 2 and pos.shape[1] == 3 and conn.ndim == 2 and conn.shape[1] == 2
    assert conn.min() >= 1 and conn.max() <= pos.shape[0]
    out = os.path.join(HERE, "reference_net.npz")
    np.savez_compressed(out, positions=pos, connectivity=conn)
    print("wrote", out, pos.shape, conn.shape)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
