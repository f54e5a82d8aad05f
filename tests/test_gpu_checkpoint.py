"""Checkpoints in the reference's file format (checkpoint.f90,
particle_initialization.f90): file names, raw layouts, header round trip and
an exact restart."""
import os

import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

A_MID, DT = 0.4, 0.02


def _ctx(p, st):
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    g.set_sigma(st["sigma_vi"], st["sigma_vi"])
    return g


def _step(g, vz):
    g.update_x(np.float32(20.0), np.float32(30.0), vz)
    g.ext_pp_force(A_MID, DT)
    g.particle_mesh(A_MID, DT)


def test_checkpoint_files_have_the_reference_layout(tmp_path):
    p = P.CubeParams(nc=24, nnt=2, pp_on=True, box=75.0)
    st = synth.random_state(p, seed=51)
    g = _ctx(p, st)
    try:
        g.checkpoint_write(str(tmp_path), 49.0, image=1, a=0.02, box=75.0, omega_m=0.3, timestep=7)
        ref = g.download()
    finally:
        g.close()
    n = ref["xp"].shape[0]
    names = sorted(os.listdir(tmp_path))
    assert names == sorted("49.000_%s_1.bin" % w for w in ("info", "xp", "vp", "np", "vc", "id"))
    raw = lambda w, dt: np.fromfile(tmp_path / ("49.000_%s_1.bin" % w), dt)
    np.testing.assert_array_equal(raw("xp", np.int8).reshape(n, 3), ref["xp"].reshape(n, 3))
    np.testing.assert_array_equal(raw("vp", np.int16).reshape(n, 3), ref["vp"].reshape(n, 3))
    np.testing.assert_array_equal(raw("np", np.int32), ref["rhoc"].ravel())
    np.testing.assert_array_equal(raw("vc", np.float32), ref["vfield"].ravel())
    np.testing.assert_array_equal(raw("id", np.int32), ref["pid"].ravel())
    info = raw("info", np.uint8)
    assert info.size == 224
    ints = info[:136].view(np.int64)
    assert ints[0] == n and ints[4] == 1 and ints[5] == 2 and ints[14] == 7   # nplocal, izipx, izipv, timestep
    reals = info[136:].view(np.float32)
    assert reals[0] == np.float32(0.02) and reals[10] == np.float32(75.0)     # a, box
    assert reals[17] == np.float32(st["sigma_vi"])                            # sigma_vi


def test_restart_from_checkpoint_is_exact(tmp_path):
    p = P.CubeParams(nc=24, nnt=2, pp_on=True, box=75.0)
    st = synth.random_state(p, seed=52, clump=8)
    g = _ctx(p, st)
    try:
        _step(g, st["vz_max"])
        g.checkpoint_write(str(tmp_path), 5.25, image=3, a=0.16)
        _step(g, st["vz_max"])
        cont = g.download()
        sig = g.get_sigma()
    finally:
        g.close()
    h = C.CubeGPU(p)
    try:
        hdr = h.checkpoint_read(str(tmp_path), 5.25, image=3)
        assert hdr["image"] == 3 and abs(hdr["a"] - 0.16) < 1e-7
        s_vi = np.float32(hdr["sigma_vi"])
        h.set_sigma(s_vi, s_vi)
        _step(h, st["vz_max"])
        again = h.download()
        assert h.get_sigma()[0] == sig[0]
    finally:
        h.close()
    for k in ("xp", "vp", "pid", "rhoc"):
        np.testing.assert_array_equal(again[k], cont[k])
    np.testing.assert_array_equal(again["vfield"].view(np.uint32), cont["vfield"].view(np.uint32))


def test_checkpoint_read_rejects_a_different_zip_format(tmp_path):
    p = P.CubeParams(nc=24, nnt=2, pp_on=True)
    st = synth.random_state(p, seed=53)
    g = _ctx(p, st)
    try:
        g.checkpoint_write(str(tmp_path), 0.0)
    finally:
        g.close()
    q = P.CubeParams(nc=24, nnt=2, pp_on=True, izipx=2)
    h = C.CubeGPU(q)
    try:
        with pytest.raises(C.CubeError) as e:
            h.checkpoint_read(str(tmp_path), 0.0)
        assert "zip format" in str(e.value)
    finally:
        h.close()
