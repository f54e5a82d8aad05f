"""Regenerate the force-kernel tables shipped in this directory.

The fine (16^3 x 3) and coarse (4^3 x 3) force tables are DATA inputs of the
reference, read at start-up by kernel_f (CUBEnu/work/main/kernel_f.f90:14-23,
file CUBEnu/kernels/wfxyzf.3.ascii) and kernel_c (kernel_c.f90:31-39, file
CUBEnu/kernels/wfxyzc.2.ascii).  This script parses those ASCII files once and
stores the values as little-endian float32 in the reference's array layouts:

  fine_force_table.f32    fk_table(i,j,k,d), Fortran order, i fastest, 16x16x16x3
  coarse_force_table.f32  ck_table(d,i,j,k), Fortran order, d fastest, 3x4x4x4

Usage: python make_tables.py <path to CUBEnu/kernels>
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_fine(path):
    # rows are "i j k fx fy fz" with k outermost, i innermost (kernel_f.f90:14-20)
    tab = np.zeros((3, 16, 16, 16), dtype=np.float32)  # (d, k, j, i) C order
    rows = [ln.split() for ln in open(path) if ln.strip()]
    assert len(rows) == 16 ** 3
    n = 0
    for k in range(16):
        for j in range(16):
            for i in range(16):
                r = rows[n]
                n += 1
                assert (int(r[0]), int(r[1]), int(r[2])) == (i + 1, j + 1, k + 1)
                for d in range(3):
                    tab[d, k, j, i] = np.float32(r[3 + d])
    return tab


def parse_coarse(path):
    # '(3i4,3e16.8)' rows, k outermost (kernel_c.f90:31-37)
    tab = np.zeros((4, 4, 4, 3), dtype=np.float32)  # (k, j, i, d) C order
    rows = [ln.split() for ln in open(path) if ln.strip()]
    assert len(rows) == 64
    n = 0
    for k in range(4):
        for j in range(4):
            for i in range(4):
                r = rows[n]
                n += 1
                for d in range(3):
                    tab[k, j, i, d] = np.float32(r[3 + d])
    return tab


def main(kdir):
    fine = parse_fine(os.path.join(kdir, "wfxyzf.3.ascii"))
    coarse = parse_coarse(os.path.join(kdir, "wfxyzc.2.ascii"))
    fine.astype("<f4").tofile(os.path.join(HERE, "fine_force_table.f32"))
    coarse.astype("<f4").tofile(os.path.join(HERE, "coarse_force_table.f32"))


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: python make_tables.py <path to CUBEnu/kernels>")
    main(sys.argv[1])
