"""Generate the golden fixtures of the CPU oracle (test infrastructure).

The reference ships no golden vectors for this path, so these pin the oracle
itself: a seeded 20^3-cell state (one tile, PP on) and the oracle's results of
update_x, ext_pp_force and particle_mesh applied in sequence
(oracle_step_nc20.npz); and a 24^3-cell state over 2^3 tiles re-sorted by a
step that moves particles several cells (oracle_resort_nc24.npz: the
reference's layered visit order beyond neighbouring cells).  The CPU tests
require the oracle to reproduce them exactly; the GPU tests compare the CUDA
path with the first.  Run from the repository root:

    python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

from cafproject_gb300 import params as P, synth  # noqa: E402
from oracle import cube_oracle as O  # noqa: E402

A_MID, DT = 0.4, 0.02
DT_OLD, DT_STEP = 28.0, 40.0


def golden_params():
    return P.CubeParams(nc=20, nnt=1, ncb=6, pp_on=True, rsoft=0.1, mass_p=8.0, box=62.5)


def make():
    p = golden_params()
    st = synth.random_state(p, mean_per_cell=1.0, seed=2024, vsig=0.03, clump=3, clump_mult=10)
    o = O.OracleImage(p)
    o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    o.sigma_vi = s
    o.sigma_vi_new = s
    out = {"in_" + k: np.asarray(v) for k, v in st.items() if k in ("xp", "vp", "pid", "rhoc", "vfield")}
    out["sigma_vi"] = np.float32(s)
    out["vz_max"] = np.float32(st["vz_max"])
    u = o.update_x(np.float32(DT_OLD), np.float32(DT_STEP), st["vz_max"])
    for k, v in o.state().items():
        out["upd_" + k] = v
    out["upd_sigma_vi_new"] = np.float32(u["sigma_vi_new"])
    out["upd_sum_r"] = np.float64(u["sum_r"])
    pp = o.pp_force(A_MID, DT)
    out["pp_vp"] = o.state()["vp"]
    out["pp_npairs"] = np.int64(pp["npairs"])
    out["pp_f2_max"] = np.float32(pp["f2_max_pp"])
    pm = o.particle_mesh(A_MID, DT)
    out["pm_vp"] = o.state()["vp"]
    out["pm_vmax"] = np.asarray(pm["vmax"], np.float32)
    out["pm_f2_max_fine"] = np.float32(pm["f2_max_fine"])
    out["pm_f2_max_coarse"] = np.float32(pm["f2_max_coarse"])
    xi = O.power_spectrum(p, out["upd_xp"], out["upd_rhoc"], 2 * p.nc, p.box)
    out["pk_xi"] = xi
    return out


RESORT_DT_OLD, RESORT_DT = 105.0, 150.0


def resort_params():
    return P.CubeParams(nc=24, nnt=2, ncb=6, pp_on=False, mass_p=8.0, box=75.0)


def make_resort():
    p = resort_params()
    st = synth.random_state(p, mean_per_cell=1.5, seed=2025, vsig=0.03, clump=4)
    o = O.OracleImage(p)
    o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    o.sigma_vi = s
    o.sigma_vi_new = s
    out = {"in_" + k: np.asarray(v) for k, v in st.items() if k in ("xp", "vp", "pid", "rhoc", "vfield")}
    out["sigma_vi"] = np.float32(s)
    out["vz_max"] = np.float32(st["vz_max"])
    u = o.update_x(np.float32(RESORT_DT_OLD), np.float32(RESORT_DT), st["vz_max"])
    for k, v in o.state().items():
        out["upd_" + k] = v
    out["upd_nlayer"] = np.int32(u["nlayer"])
    out["upd_sum_r"] = np.float64(u["sum_r"])
    return out


if __name__ == "__main__":
    np.savez_compressed(os.path.join(HERE, "oracle_step_nc20.npz"), **make())
    print("wrote", os.path.join(HERE, "oracle_step_nc20.npz"))
    np.savez_compressed(os.path.join(HERE, "oracle_resort_nc24.npz"), **make_resort())
    print("wrote", os.path.join(HERE, "oracle_resort_nc24.npz"))
