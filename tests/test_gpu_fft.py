"""The fine force chain through this library's own transforms (cube_fft.cu,
power-of-two meshes) against the same chain through cuFFT with separate
multiply and maxima passes (CUBE_OPT_CUFFT): same density, forces within
FP32 round-off of each other, the same |F|^2 maximum, and the kicks that
follow identical except where a code sits on a rounding edge."""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("nc,nnt", [(16, 1), (32, 2), (64, 2), (128, 2)])
def test_own_transforms_match_cufft(nc, nnt):
    p = P.CubeParams(nc=nc, nnt=nnt, pp_on=True, rsoft=0.1, mass_p=8.0)
    st = synth.random_state(p, mean_per_cell=6, seed=nc, clump=max(2, nc // 8))
    out = []
    for cufft in (0, 1):
        g = C.CubeGPU(p)
        try:
            g.set_option(C.OPT_CUFFT, cufft)
            g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
            s = np.float32(st["sigma_vi"])
            g.set_sigma(s, s)
            fs = g.fine_forces()
            F = g.get_field(C.FIELD_FORCE_F)
            pm = g.particle_mesh(0.4, 0.02)
            out.append((fs, F, pm, g.download()["vp"]))
        finally:
            g.close()
    (fa, Fa, pa, va), (fb, Fb, pb, vb) = out
    err = rel_l2(Fa, Fb)
    d = np.abs(va.astype(np.int64) - vb.astype(np.int64))
    print("nf %d: own vs cuFFT force rel-L2 %.2e, f2max %.3e / %.3e, codes differing %.2e" %
          (4 * nc, err, fa["f2_max_fine"], fb["f2_max_fine"], (d > 0).mean()))
    assert err < 2e-6
    assert abs(fa["f2_max_fine"] / fb["f2_max_fine"] - 1) < 1e-5
    assert abs(pa["f2_max_fine"] / pb["f2_max_fine"] - 1) < 1e-5
    assert d.max() <= 2 and (d > 0).mean() < 1e-3
