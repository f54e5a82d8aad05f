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


def test_upload_rejects_inconsistent_counts():
    # the counts are checked on the device after the copies: a sum that is
    # not nplocal, or a negative count, is an error and leaves no state; a
    # consistent upload afterwards works
    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300 import synth
    p = P.small(nc=24, nnt=2, pp_on=False)
    st = synth.random_state(p, mean_per_cell=4, seed=3)
    g = C.CubeGPU(p)
    try:
        bad = st["rhoc"].copy()
        bad[5] += 1
        with pytest.raises(C.CubeError) as e:
            g.upload(st["xp"], st["vp"], st["pid"], bad, st["vfield"])
        assert e.value.code == 6
        neg = st["rhoc"].copy()
        neg[7] -= neg[7] + 1
        neg[8] += st["rhoc"][7] + 1
        with pytest.raises(C.CubeError) as e:
            g.upload(st["xp"], st["vp"], st["pid"], neg, st["vfield"])
        assert e.value.code == 1
        with pytest.raises(C.CubeError):
            g.update_x(np.float32(1.0), np.float32(1.0), np.float32(0.1))  # no state
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        assert g.nplocal() == st["xp"].shape[0]
        assert np.array_equal(g.download()["rhoc"], st["rhoc"])
    finally:
        g.close()


def test_split_download_matches_download():
    # xp, pid, rhoc and vfield copied beside PP+PM (cube_download_begin right
    # after update_x), vp behind the coarse kick's pieces: the same arrays as a
    # download at the end of the step; an update_x issued before the finish is
    # ordered after the copies, so the arrays hold the state of the step that
    # began them; with no kick before the finish, the finish copies vp
    import torch
    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300 import synth
    p = P.small(nc=24, nnt=2, pp_on=True)
    st = synth.random_state(p, mean_per_cell=8, seed=12, vsig=0.03, clump=4)
    g = C.CubeGPU(p)
    try:
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        s = np.float32(st["sigma_vi"])
        g.set_sigma(s, s)
        out = {k: torch.from_numpy(np.empty_like(st[k])).pin_memory().numpy()
               for k in ("xp", "vp", "pid", "rhoc", "vfield")}
        for _ in range(2):
            g.update_x(np.float32(20.0), np.float32(30.0), st["vz_max"])
            g.download_begin(out)
            g.pp_particle_mesh(np.float32(0.4), np.float32(0.02))
            got = {k: v.copy() for k, v in g.download_finish().items()}
            ref = g.download()
            for key in ("xp", "vp", "pid", "rhoc", "vfield"):
                assert np.array_equal(got[key], ref[key]), key
        ref = g.download()
        g.download_begin(out)
        g.update_x(np.float32(20.0), np.float32(30.0), st["vz_max"])
        got = g.download_finish()
        for key in ("xp", "pid", "rhoc", "vfield"):
            assert np.array_equal(got[key], ref[key]), key
        assert np.array_equal(got["vp"], g.download()["vp"])
    finally:
        g.close()


@pytest.mark.parametrize("first", ["update_x", "particle_mesh"])
def test_overlapped_upload_matches_upload(first):
    # xp and vp in pieces beside the re-sort's first pass, pid beside the rest
    # (cube_upload_begin): the steps give bit for bit the state of a plain
    # upload, and the host arrays may change once update_x has returned; a
    # call other than update_x first waits for the whole upload
    import torch
    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300 import synth
    p = P.small(nc=24, nnt=2, pp_on=True)
    st = synth.random_state(p, mean_per_cell=8, seed=13, vsig=0.03, clump=4)
    outs = []
    for overlap in (False, True):
        g = C.CubeGPU(p)
        try:
            pin = {k: torch.from_numpy(np.ascontiguousarray(st[k])).pin_memory().numpy()
                   for k in ("xp", "vp", "pid", "rhoc", "vfield")}
            (g.upload_begin if overlap else g.upload)(pin["xp"], pin["vp"], pin["pid"], pin["rhoc"], pin["vfield"])
            s = np.float32(st["sigma_vi"])
            g.set_sigma(s, s)
            if first == "particle_mesh":
                g.pp_particle_mesh(np.float32(0.4), np.float32(0.02))
            for _ in range(2):
                g.update_x(np.float32(20.0), np.float32(30.0), st["vz_max"])
                for k in ("pid", "xp", "vp"):
                    pin[k][:] = -7
                g.pp_particle_mesh(np.float32(0.4), np.float32(0.02))
            outs.append(g.download())
        finally:
            g.close()
    for key in ("xp", "vp", "pid", "rhoc", "vfield"):
        assert np.array_equal(outs[0][key], outs[1][key]), key
    assert (outs[1]["pid"] != -7).all()
