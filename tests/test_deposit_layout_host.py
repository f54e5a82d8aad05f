"""The deposit kernel's layout invariants, checked on the CPU for every instance.

`k_deposit_det` (cafproject_gb300/csrc/cube_pm.cu) clears its shared-memory
accumulators with 16-byte stores and, where it deposits onto a mesh finer
than the coarse cells (MPC > 1: the PM fine mesh, the power-spectrum meshes
at 2 and 4 points per coarse cell), converts and writes KX neighbouring x
cells per thread through 8-byte stores into the padded mesh (row stride
n+2).  Those wide accesses are only in bounds and aligned if, for every
instance launched and every brick of every valid mesh size:

* 2*MX*MY*MZ (low words + carry words) is a multiple of 4;
* KX divides MX, the brick's extent MPC*B[0] (B[0] clipped at the mesh's
  edge) and MPC, so a thread's KX cells stay inside its brick's row;
* the mesh index of the first cell, x + (n+2)*(y + n*z), is even, so the
  float2 stores start 8-byte aligned.

The source cells' coordinates travel in 16-bit fields, which the context's
size check (nc <= 16384) keeps in range.  The instance list is read from the
kernel's source so that a new brick shape is checked too.
"""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "cafproject_gb300", "csrc", "cube_pm.cu")


def instances():
    src = open(SRC).read()
    out = []
    for m in re.finditer(r"launch_deposit<(\d+), (\d+), (\d+), (\d+), (\d+), (\d+)(, true)?>", src):
        mpc, bx, by, bz, lo, hi = (int(v) for v in m.groups()[:6])
        out.append((mpc, bx, by, bz, lo, hi, m.group(7) is not None))
    return out


def test_every_shape_is_listed():
    inst = instances()
    assert len(inst) == 11
    assert sum(1 for i in inst if i[6]) == 3  # power-spectrum meshes at 1, 2 and 4 points per coarse cell


@pytest.mark.parametrize("inst", instances(), ids=lambda i: "x".join(map(str, i[:6])) + ("pk" if i[6] else ""))
def test_wide_accesses_stay_aligned_and_in_the_brick(inst):
    mpc, bx, by, bz, lo, hi, pk = inst
    mx, my, mz = mpc * bx, mpc * by, mpc * bz
    assert (2 * mx * my * mz) % 4 == 0
    if mpc == 1:
        return  # the coarse mesh is written one cell a thread
    kx = 4 if mpc >= 4 else 2
    assert mx % kx == 0 and mpc % kx == 0
    # every valid coarse size: nc >= 16, up to a few bricks past a whole number
    for nc in list(range(16, 80)) + [128, 255, 256, 1000, 16384]:
        n = mpc * nc  # the PM fine mesh (4 nc) or the power-spectrum mesh (ng = mpc nc)
        assert n % 2 == 0
        for c0 in range(0, nc, bx):
            b0 = min(bx, nc - c0)
            assert (mpc * b0) % kx == 0
            for x in range(0, mpc * b0, kx):
                assert (mpc * c0 + x) % 2 == 0 and (n + 2) % 2 == 0
                assert x + kx <= mpc * b0  # the thread's cells stay in the brick's row


def test_frame_fields_fit_sixteen_bits():
    # tile-local coordinates run 1..nt and global ones 0..nc-1, nt <= nc <= 16384
    assert 16384 < 1 << 16
    src = open(SRC).read()
    assert "<< (16 * d)" in src and "& 0xffffu" in src
    api = open(os.path.join(ROOT, "cafproject_gb300", "csrc", "cube_api.cu")).read()
    assert "p->nc > 16384" in api
