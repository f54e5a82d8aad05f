"""The FP64 error of the FP32 force path, on the CPU.

The GPU's fine force is checked against the oracle's FP32 path at 1e-5
relative L2 (tests/test_gpu_parity.py).  Here the oracle's FP32 fine force
is compared with the same oracle evaluated in FP64 (kernel and transforms in
double): the reported error bounds how far the FP32 forces of both sides are
from exact arithmetic on the reference's algorithm (FFTW in the reference,
pocketfft here, cuFFT on the GPU).
"""
import numpy as np
import pytest

from cafproject_gb300 import params as P
from cafproject_gb300 import synth
from oracle import cube_oracle as O

FP64_RTOL = 1e-5  # relative L2 of the FP32 force against the FP64 one


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("nnt,seed,clump", [(2, 41, 0), (1, 42, 20)])
def test_fp32_fine_force_against_fp64(nnt, seed, clump):
    p = P.CubeParams(nc=24, nnt=nnt, pp_on=True, rsoft=0.1, mass_p=8.0)
    st = synth.random_state(p, mean_per_cell=6, seed=seed, vsig=0.02, clump=clump)
    forces = []
    for dt in (np.float32, np.float64):
        o = O.OracleImage(p, fft_dtype=dt)
        o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        forces.append(o.global_fine_force()[0])
    err = rel_l2(forces[0], forces[1])
    print("fine force, FP32 vs FP64 oracle: relative L2 %.2e" % err)
    assert err < FP64_RTOL
