"""Every brick shape of the two deposits writes the same meshes.

The deposits (pm.f90:52-107 fine, pm.f90:205-253 coarse) accumulate their
real(4) CIC weights in 2^-s fixed point with integer atomics, so the brick
shape picked with CUBE_OPT_DEPOSIT_FINE / CUBE_OPT_DEPOSIT_COARSE changes
which block adds a weight, never the sum: the meshes and their totals must be
bitwise equal for every shape, also where the mesh is not a whole number of
bricks (nc = 40) and in dense clumps.
"""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

SHAPES = range(4)  # 0 = the default shape, 1..3 the alternatives


@pytest.mark.parametrize("izipx", [1, 2])
def test_deposit_shapes_bitwise(izipx):
    p = P.small(nc=40, nnt=2, izipx=izipx, izipv=2)
    st = synth.random_state(p, mean_per_cell=4.0, seed=11 + izipx, clump=3, clump_mult=500)
    g = C.CubeGPU(p)
    try:
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        fine, coarse = {}, {}
        for s in SHAPES:
            g.set_option(C.OPT_DEPOSIT_FINE, s)
            g.set_option(C.OPT_DEPOSIT_COARSE, s)
            a = g.fine_density()
            b = g.coarse_density()
            fine[s] = (g.get_field(C.FIELD_RHO_F).view(np.uint32).copy(), a["testrhof"])
            coarse[s] = (g.get_field(C.FIELD_RHO_C).view(np.uint32).copy(), b["testrhoc"])
        n = st["xp"].shape[0]
        for s in SHAPES:
            assert np.array_equal(fine[s][0], fine[0][0]) and fine[s][1] == fine[0][1]
            assert np.array_equal(coarse[s][0], coarse[0][0]) and coarse[s][1] == coarse[0][1]
        # every particle's unit mass lands somewhere: the totals are the particle count
        assert abs(fine[0][1] - n * p.mass_p) <= 1e-6 * n * p.mass_p
        assert abs(coarse[0][1] - n * p.mass_p) <= 1e-6 * n * p.mass_p
    finally:
        g.close()
