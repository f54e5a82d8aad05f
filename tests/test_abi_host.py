"""CPU-only checks of the C ABI library and the host-side logic."""
import ctypes
import os
import re

import numpy as np
import pytest

from cafproject_gb300 import cosmology, params as P

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    src = open(os.path.join(ROOT, "include", "cube_gpu.h")).read()
    return sorted(set(re.findall(r"^\s*(?:int|int64_t|const char\*|void\*)\s+(cube_\w+)\s*\(", src, re.M)))


def test_library_exports_every_declared_symbol(built_lib):
    lib = ctypes.CDLL(built_lib)
    names = declared_symbols()
    assert len(names) >= 20
    for n in names:
        assert hasattr(lib, n), n
    from cafproject_gb300 import cube
    assert set(cube.EXPORTS) == set(names)


def test_params_struct_matches_header():
    c = P.cdm512().to_c()
    assert ctypes.sizeof(c) == 4 * 12 + 8 + 4 * 8
    assert c.nc == 256 and c.nnt == 2 and c.pp_on == 1 and abs(c.rsoft - 0.1) < 1e-7


def test_stats_struct_layout():
    from cafproject_gb300.cube import CubeStats
    # field offsets follow the C struct in include/cube_gpu.h (all naturally aligned)
    assert CubeStats.sigma_vi_new.offset == 7 * 8
    assert CubeStats.npairs.offset % 8 == 0 and CubeStats.testrhof.offset % 8 == 0


@pytest.mark.parametrize("nc,msg", [(14, b"at least 16"), (32768, b"at most 16384")])
def test_cube_create_rejects_bad_sizes(built_lib, nc, msg):
    from cafproject_gb300 import cube
    L = cube.load_library()
    bad = P.CubeParams(nc=nc, nnt=1).to_c()
    fine, coarse = cube.force_tables()
    h = ctypes.c_void_p()
    rc = L.cube_create(ctypes.byref(bad), fine.ctypes.data_as(ctypes.c_void_p),
                       coarse.ctypes.data_as(ctypes.c_void_p), 0, ctypes.byref(h))
    assert rc == 1  # CUBE_ERR_ARG before any device call
    assert msg in L.cube_last_error(h)
    L.cube_destroy(h)


def test_expansion_advances_scale_factor():
    a = np.float32(0.02)
    d1, d2 = cosmology.expansion(a, np.float32(0.1), 0.3, 0.7)
    assert d1 > 0 and d2 > d1 * 0.99
    # matter era: da ~ adot*dt, adot = sqrt(4/9 a^3 (1 + ...)) / ... grows with a
    d1b, _ = cosmology.expansion(np.float32(0.5), np.float32(0.1), 0.3, 0.7)
    assert d1b > d1


def test_timestep_respects_ra_max_and_constraints():
    ts = cosmology.TimeState(a=np.float32(0.02), z_checkpoints=[0.0])
    dt, a_mid = ts.timestep()
    assert ts.da / (ts.a) <= np.float32(0.2) * 1.0001
    assert ts.a > 0.02 and a_mid < ts.a
    ts2 = cosmology.TimeState(a=np.float32(0.02), z_checkpoints=[0.0])
    ts2.dt_pp = np.float32(dt / 10)
    dt2, _ = ts2.timestep()
    assert dt2 == np.float32(dt / 10)


def test_timestep_lands_on_checkpoint():
    ts = cosmology.TimeState(a=np.float32(0.95), z_checkpoints=[0.0])
    for _ in range(50):
        ts.timestep()
        if ts.checkpoint_step:
            break
    assert ts.checkpoint_step and ts.final_step
    assert abs(float(ts.a) - 1.0) < 2e-6


def test_constrain_from_device_maxima():
    ts = cosmology.TimeState(a=np.float32(0.5))
    ts.a_mid = np.float32(0.5)
    ts.constrain({"f2_max_fine": 4.0, "f2_max_coarse": 16.0, "vmax": [1.0, 2.0, 3.0]}, {"f2_max_pp": 9.0})
    GG = cosmology.GG
    assert ts.dt_fine == np.float32(np.sqrt(np.float32(1) / (np.float32(2) * np.float32(0.5) * GG)))
    assert ts.dt_vmax == np.float32(np.float32(18) / np.float32(3))
    assert ts.vz_max == np.float32(3.0)


def test_fast_division_is_exact():
    # the magic-number division used by the kernels (Granlund & Montgomery
    # round-up multiplier), emulated exactly in Python
    rng = np.random.default_rng(0)

    def magic(d):
        l = 0
        while (1 << l) < d:
            l += 1
        return ((((1 << l) - d) << 32) // d + 1) & 0xFFFFFFFF, l

    def fdiv(n, d, m, l):
        if d <= 1:
            return n
        t = (n * m) >> 32
        return (t + ((n - t) >> 1)) >> (l - 1)

    for d in list(range(1, 300)) + [1 << k for k in range(1, 31)] + list(rng.integers(2, 1 << 31, 200)):
        d = int(d)
        m, l = magic(d)
        ns = [0, 1, d - 1, d, d + 1, 2 * d - 1, (1 << 32) - 1, (1 << 31) - 1] + list(rng.integers(0, 1 << 32, 300))
        for n in ns:
            n = int(n)
            assert fdiv(n, d, m, l) == n // d, (n, d)


def test_sim_header_matches_reference_layout():
    # sim_header (parameters.f90:136-160) in Fortran stream I/O: 17 int64 then 22 real(4)
    from cafproject_gb300.cube import SimHeader
    assert ctypes.sizeof(SimHeader) == 17 * 8 + 22 * 4 == 224
    assert SimHeader.a.offset == 136 and SimHeader.vz_max.offset == 220
    assert SimHeader.sigma_vi.offset == 136 + 4 * 17


def test_neutrino_switch_on_checkpoints():
    # initialize.f90:90-136
    f = cosmology.neutrino_checkpoints
    assert f([10.0, 5.0, 0.0], 49.0, 49.0) == ([10.0, 5.0, 0.0], 0, True)
    assert f([10.0, 5.0, 0.0], 49.0, 5.0) == ([10.0, 5.0, 0.0], 2, False)       # already a checkpoint
    assert f([10.0, 2.0, 0.0], 49.0, 5.0) == ([10.0, 5.0, 2.0, 0.0], 2, False)  # inserted
    assert f([10.0, 8.0], 49.0, 5.0) == ([10.0, 8.0, 5.0], 3, False)            # appended after the last
    with pytest.raises(ValueError):
        f([0.0], 10.0, 20.0)
