"""The compiled caller: host/cube_main.cpp runs CUBE's step loop
(main.f90:88-145, with timestep.f90's scalar logic restated in C++) through
the C ABI from a separate process.  The same loop driven from Python through
ctypes (TimeState of cosmology.py, the checkpoint half drift of
main.f90:121-123) must write byte-identical checkpoint files: the linked
library, the C++ and Python timestep restatements and the call sequence agree.
"""
import os
import subprocess

import numpy as np
import pytest

from cafproject_gb300 import build as B
from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300.cosmology import TimeState

pytestmark = pytest.mark.gpu

Z_INIT, Z_OUT, SEED = 49.0, (30.0, 20.0), 11


def _python_run(p, out):
    g = C.CubeGPU(p)
    try:
        sigma, vm = g.ic_zeldovich(Z_INIT, SEED)
        ts = TimeState(a=np.float32(1.0 / (1.0 + Z_INIT)), omega_m=p.omega_m, omega_l=p.omega_l,
                       z_checkpoints=list(Z_OUT))
        ts.vz_max = np.float32(vm[2])
        ts.dt_vmax = np.float32(np.float32(18.0) / np.float32(max(vm)))
        steps = 0
        while True:
            dt, a_mid = ts.timestep()
            g.update_x(ts.dt_old, dt, ts.vz_max)
            g.buffer_grid()
            g.buffer_x()
            if p.pp_on:
                pps, pms = g.pp_particle_mesh(a_mid, dt)
            else:
                pps, pms = None, g.particle_mesh(a_mid, dt)
            g.buffer_v()
            ts.constrain(pms, pps, p.ncell)
            steps += 1
            if ts.checkpoint_step:
                ts.dt_old = np.float32(0)
                g.update_x(ts.dt_old, ts.dt, ts.vz_max)
                z = Z_OUT[ts.cur_checkpoint]
                g.checkpoint_write(out, z)
                ts.cur_checkpoint += 1
                if ts.final_step:
                    break
                ts.dt = np.float32(0)
        return steps
    finally:
        g.close()


@pytest.mark.parametrize("pp", [0, 1])
def test_compiled_driver_matches_python_driver(tmp_path, pp):
    B.build()
    p = P.CubeParams(nc=32, nnt=2, pp_on=bool(pp), rsoft=0.1, box=100.0, np_nc=2)
    dc, dp = tmp_path / "cpp", tmp_path / "py"
    dc.mkdir()
    dp.mkdir()
    r = subprocess.run([B.DRIVER, "--out", str(dc), "--nc", "32", "--nnt", "2", "--np-nc", "2", "--box", "100",
                        "--pp", str(pp), "--z-init", str(Z_INIT), "--z", ",".join(str(z) for z in Z_OUT),
                        "--seed", str(SEED)], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout[-2000:] + r.stderr[-2000:]
    lines = [ln for ln in r.stdout.splitlines() if ln.startswith("step ")]
    steps = _python_run(p, str(dp))
    print("compiled driver: %d steps to z=%g, last: %s" % (len(lines), Z_OUT[-1], lines[-1]))
    assert len(lines) == steps
    for z in Z_OUT:
        for what in ("xp", "vp", "np", "vc", "id"):
            name = "%.3f_%s_1.bin" % (z, what)
            a, b = (dc / name).read_bytes(), (dp / name).read_bytes()
            assert a == b, name
        # the header: same state counts and the same scale factor
        ha = np.fromfile(dc / ("%.3f_info_1.bin" % z), np.uint8)
        hb = np.fromfile(dp / ("%.3f_info_1.bin" % z), np.uint8)
        assert ha.size == hb.size == 224
        assert np.array_equal(ha[:8], hb[:8])  # nplocal
