"""The initial-condition formulas of the reference, restated in numpy
(oracle/ic_oracle.py), against known answers on the CPU and against the
device's tables on the GPU.

CPU: Dgrow(1) = 1, tophat(0) = 1 and its value at 0.5, vfactor(1) =
H(1) = 2/3 sqrt(1 + omega_l/omega_m) in the reference's units, the sigma_8 sum
of the normalised table equal to s8^2 Dgrow^2, and the corrected potential
kernel's real-space values (-1/r inside 8 cells, -2.5 at the origin).
GPU: the device's initial-condition filter (Wiener scaling times the corrected
kernel, cube_ic_filter through cube_dpm_tables) and its a^2 H equal the
restatement's.
"""
import numpy as np
import pytest

from oracle import ic_oracle as I


def test_growth_and_window_known_answers():
    assert abs(float(I.dgrow(1.0, 0.3, 0.7)) - 1.0) < 1e-6
    assert I.tophat(0.0) == 1.0
    x = 0.5  # the window against its double-precision value (default real cancels near 0)
    assert abs(float(I.tophat(x)) - 3 * (np.sin(x) - np.cos(x) * x) / x ** 3) < 1e-5
    # linear growth is close to a at early times in a matter-dominated universe
    assert abs(float(I.dgrow(0.02, 0.3, 0.7)) / 0.02 / 1.28 - 1) < 0.01
    h1 = 2.0 / 3.0 * np.sqrt(1 + 0.7 / 0.3)
    assert abs(float(I.vfactor(1.0, 0.3, 0.7)) - h1) < 1e-6 * h1


def test_sigma8_normalisation():
    # the table sum the reference normalises with, evaluated on the result
    box, nf, a = 600.0, 1024, 1.0 / 50.0
    k, d2 = I.delta2_table(box, nf, a)
    dk = np.empty_like(k)
    dk[0], dk[1:-1], dk[-1] = k[1] / 2, (k[2:] - k[:-2]) / 2, k[-1] - k[-2]
    kmax = 2 * np.pi * np.sqrt(3.0) * (nf // 2) / box
    sel = k <= kmax
    v8 = sum(d2[i] * float(I.tophat(k[i] * 8)) ** 2 * dk[i] / k[i] for i in np.nonzero(sel)[0])
    g = float(I.dgrow(a, 0.3, 0.7))
    assert abs(v8 / (0.8 ** 2 * g * g) - 1) < 1e-9


def test_corrected_kernel_real_space_values():
    nf = 32
    r3 = np.fft.irfftn(I.corrected_kernel(nf), s=(nf, nf, nf), axes=(0, 1, 2))
    assert abs(r3[0, 0, 0] + 2.5) < 1e-9
    assert abs(r3[0, 0, 1] + 1.0) < 1e-9
    assert abs(r3[0, 3, 4] + 1.0 / 5.0) < 1e-9
    assert abs(r3[8, 0, 0] + 1.0 / 8.0) < 1e-9


@pytest.mark.gpu
@pytest.mark.parametrize("npd,box,z", [(32, 64.0, 9.0), (64, 256.0, 49.0)])
def test_device_filter_matches_restatement(npd, box, z):
    from cafproject_gb300.dpm import DiffPM
    sim = DiffPM(2 * npd, npd, z, 0.0, 2, ckpt_every=1, box=box, omega_b=0.045)
    try:
        filt, _ = sim.tables()
        vf = sim.info()["vf"]
    finally:
        sim.close()
    ref = I.filter_table(npd, box, 1.0 / (1.0 + z), ob=0.045)
    err = np.linalg.norm(filt - ref) / np.linalg.norm(ref)
    print("IC filter vs restatement (npd %d, box %g, z %g): rel-L2 %.2e" % (npd, box, z, err))
    assert err < 1e-5
    vref = float(I.vfactor(1.0 / (1.0 + z), 0.3, 0.7))
    assert abs(vf / vref - 1) < 1e-6
