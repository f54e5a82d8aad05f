"""cube_pp_particle_mesh (PP on a second stream beside the PM force chain)
gives bit for bit the state and stats of cube_pp_force followed by
cube_particle_mesh."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_fused_pp_and_pm_match_the_two_calls():
    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300 import synth
    p = P.small(nc=24, nnt=2, pp_on=True)
    st = synth.random_state(p, mean_per_cell=8, seed=11, vsig=0.03, clump=10)
    outs = []
    for fused in (False, True):
        g = C.CubeGPU(p)
        try:
            g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
            s = np.float32(st["sigma_vi"])
            g.set_sigma(s, s)
            stats = []
            for k in range(3):
                u = g.update_x(np.float32(20.0), np.float32(30.0), st["vz_max"])
                if fused:
                    pp, pm = g.pp_particle_mesh(np.float32(0.4), np.float32(0.02))
                else:
                    pp = g.ext_pp_force(np.float32(0.4), np.float32(0.02))
                    pm = g.particle_mesh(np.float32(0.4), np.float32(0.02))
                stats.append((u["sigma_vi_new"], pp["f2_max_pp"], pp["npairs"], pp["itest1"], pm["f2_max_fine"],
                              pm["f2_max_coarse"], tuple(pm["vmax"])))
            outs.append((g.download(), stats))
        finally:
            g.close()
    (sa, ta), (sb, tb) = outs
    assert ta == tb
    for key in ("xp", "vp", "pid", "rhoc", "vfield"):
        assert np.array_equal(sa[key], sb[key]), key
    assert ta[-1][2] > 0  # pairs were found
