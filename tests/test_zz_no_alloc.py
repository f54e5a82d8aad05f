"""The codec check whose device scratch is a fixed file-scope array.

Collected last (file name) so it also runs after every other GPU test in the
same process; it passes alone as well.  The reference has no counterpart: it is
the allocation-free form of cube_codec_check, and must give the same codes.
"""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P

pytestmark = pytest.mark.gpu


def _velocities(rng, n, sigma):
    # typical values, the tails and exact zeros
    v = rng.normal(0.0, 3.0 * sigma, n)
    v[: n // 16] = rng.normal(0.0, 40.0 * sigma, n // 16)
    v[n // 16: n // 16 + 8] = 0.0
    return v


def test_static_scratch_codec_check_matches_allocating_entry_point():
    p = P.CubeParams(nc=24, nnt=2, pp_on=True)
    g = C.CubeGPU(p)
    rng = np.random.default_rng(5)
    try:
        # two calls in a row on the shared array, different sizes and sigmas
        for n, sigma in ((C.CODEC_STATIC_MAX, np.float32(0.013)), (3001, np.float32(0.021))):
            v = _velocities(rng, n, sigma)
            d_ref, t_ref = g.codec_check(sigma, v)
            d, t = g.codec_check_static(sigma, v)
            np.testing.assert_array_equal(d, d_ref)
            np.testing.assert_array_equal(t, t_ref)
            np.testing.assert_array_equal(t, d)
    finally:
        g.close()


def test_static_scratch_codec_check_allocates_nothing():
    # after one warm call (the array's address, the kernels' first loads),
    # calls of several sizes and sigmas leave the device's free memory as it was
    torch = pytest.importorskip("torch")
    p = P.CubeParams(nc=24, nnt=2, pp_on=True)
    g = C.CubeGPU(p)
    rng = np.random.default_rng(7)
    try:
        g.codec_check_static(np.float32(0.02), _velocities(rng, 64, 0.02))
        g.synchronize()
        free0 = torch.cuda.mem_get_info(0)[0]
        for n, sigma in ((1, 0.011), (C.CODEC_STATIC_MAX, 0.017), (777, 0.029), (C.CODEC_STATIC_MAX // 2, 0.017)):
            s = np.float32(sigma)
            d, t = g.codec_check_static(s, _velocities(rng, n, s))
            np.testing.assert_array_equal(t, d)
        g.synchronize()
        assert torch.cuda.mem_get_info(0)[0] == free0
    finally:
        g.close()


def test_static_scratch_codec_check_rejects_oversize():
    p = P.CubeParams(nc=24, nnt=2, pp_on=True)
    g = C.CubeGPU(p)
    try:
        v = np.zeros(C.CODEC_STATIC_MAX + 1)
        with pytest.raises(C.CubeError) as e:
            g.codec_check_static(np.float32(0.02), v)
        assert "static scratch maximum" in str(e.value)
        # the context stays usable after the rejection
        d, t = g.codec_check_static(np.float32(0.02), v[:10])
        assert np.all(d == 0) and np.all(t == 0)
    finally:
        g.close()
