"""GPU parity: the CUDA path through the C ABI against the CPU oracle.

Integer state (xp, vp, pid, rhoc, cell order) must be bit-exact given
identical inputs (and identical force fields for the kicks); float fields are
compared with the tolerances written in each test.
"""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.cube_oracle")

FORCE_RTOL = 1e-5   # relative L2 of a force field vs the oracle's FP32 path
RHO_RTOL = 1e-6     # relative L2 of the CIC density (FP32 sum order only)
# kick scale a_mid*dt for the synthetic states: a velocity change of order
# sigma_v per step, as the reference's dt constraints produce (pm.f90:395-398)
A_MID, DT = 0.4, 0.02
# velocity codes after a kick from a recomputed force: differ by at most one,
# and only where the pre-rounding value is within the force error of a half integer
MAX_CODE_DIFF, MAX_DIFF_FRAC = 1, 1e-3


def rel_l2(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_pair(p, st, sigma=None):
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"] if sigma is None else sigma)
    g.set_sigma(s, s)
    o = O.OracleImage(p)
    o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    o.sigma_vi = s
    o.sigma_vi_new = s
    return g, o


CASES = [
    ("nnt2_x1v2", dict(nc=24, nnt=2, izipx=1, izipv=2), dict(mean_per_cell=6, seed=1, vsig=0.02)),
    ("nnt1_x1v2", dict(nc=32, nnt=1, izipx=1, izipv=2), dict(mean_per_cell=4, seed=2, vsig=0.02)),
    ("nnt2_x2v1", dict(nc=24, nnt=2, izipx=2, izipv=1), dict(mean_per_cell=5, seed=3, vsig=0.02)),
    ("nnt3_clump", dict(nc=36, nnt=3, izipx=1, izipv=2), dict(mean_per_cell=3, seed=4, vsig=0.03, clump=30)),
    # three cells of ~600 particles: their new velocity means go through the
    # warp-per-cell pass
    ("nnt2_dense", dict(nc=24, nnt=2, izipx=1, izipv=2), dict(mean_per_cell=4, seed=5, vsig=0.02, clump=3,
                                                             clump_mult=150)),
    # three source cells of ~3200 particles: the counting path ranks them (and
    # every cell over 128) a block per cell (k_rank_dense), not the sort
    ("nnt2_rankdense", dict(nc=24, nnt=2, izipx=1, izipv=2), dict(mean_per_cell=4, seed=6, vsig=0.02, clump=3,
                                                                 clump_mult=800)),
]


def _params(kw):
    return P.CubeParams(pp_on=True, rsoft=0.1, mass_p=8.0, **kw)


@pytest.mark.parametrize("name,pk,sk", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("dt", [0.0, 40.0, 150.0])
def test_update_x_bitexact(name, pk, sk, dt):
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    dt_old = np.float32(dt * 0.7)
    a = g.update_x(dt_old, dt, st["vz_max"])
    b = o.update_x(dt_old, dt, st["vz_max"])
    sg = g.download()
    so = o.state()
    assert a["nplocal"] == b["nplocal"]
    assert a["nlayer"] == b["nlayer"]
    np.testing.assert_array_equal(sg["rhoc"], so["rhoc"])
    np.testing.assert_array_equal(sg["xp"], so["xp"])
    np.testing.assert_array_equal(sg["pid"], so["pid"])
    np.testing.assert_array_equal(sg["vfield"].view(np.uint32), so["vfield"].view(np.uint32))
    np.testing.assert_array_equal(sg["vp"], so["vp"])
    assert abs(a["sum_r"] - b["sum_r"]) <= 1e-12 * max(abs(b["sum_r"]), 1)
    assert abs(float(a["sigma_vi_new"]) - float(b["sigma_vi_new"])) <= 1e-6 * float(b["sigma_vi_new"])
    g.close()


@pytest.mark.parametrize("name,pk,sk", CASES, ids=[c[0] for c in CASES])
@pytest.mark.parametrize("dt", [20.0, 40.0, 90.0, 150.0])
def test_update_rank_paths_agree_bitwise(name, pk, sk, dt):
    # the three rank paths -- counting (every particle moved at most one cell,
    # one frame), the visit-order walker, the sort of all landings -- give the
    # same state and statistics; the default takes the sort when counting does
    # not apply
    p = _params(pk)
    st = synth.random_state(p, **sk)
    outs = []
    for path in (0, 1, 2):
        g = C.CubeGPU(p)
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        g.set_sigma(st["sigma_vi"], st["sigma_vi"])
        g.set_option(C.OPT_RANK_WALK, path)
        s = g.update_x(np.float32(dt * 0.7), np.float32(dt), st["vz_max"])
        outs.append((s, g.download()))
        g.close()
    (sa, da) = outs[0]
    assert outs[1][0]["rank_walked"] == 1 and outs[2][0]["rank_walked"] == 2
    if sa["max_disp"] <= 1 and sa["ndup"] == 0:
        assert sa["rank_walked"] == 0
    else:
        assert sa["rank_walked"] == 2
    for sb, db in outs[1:]:
        for k in ("xp", "vp", "pid", "rhoc"):
            np.testing.assert_array_equal(da[k], db[k])
        np.testing.assert_array_equal(da["vfield"].view(np.uint32), db["vfield"].view(np.uint32))
        assert sa["sum_r"] == sb["sum_r"] and sa["nplocal"] == sb["nplocal"] and sa["ndup"] == sb["ndup"]


def test_upload_download_roundtrip():
    p = _params(dict(nc=24, nnt=2))
    st = synth.random_state(p, seed=7)
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = g.download()
    for k in ("xp", "vp", "pid", "rhoc", "vfield"):
        np.testing.assert_array_equal(s[k], np.asarray(st[k]).reshape(s[k].shape))
    g.close()


@pytest.mark.parametrize("name,pk,sk", CASES[:3], ids=[c[0] for c in CASES[:3]])
def test_fine_density_and_force(name, pk, sk):
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    ds = g.fine_density()
    Rg = g.get_field(C.FIELD_RHO_F)
    gs = g.fine_forces()
    Fo, Ro = o.global_fine_force()
    Fg = g.get_field(C.FIELD_FORCE_F)
    assert rel_l2(Rg, Ro) < RHO_RTOL
    assert abs(ds["testrhof"] - gs["testrhof"]) <= 1e-9 * abs(gs["testrhof"])
    assert rel_l2(Fg, Fo) < FORCE_RTOL
    assert abs(gs["testrhof"] - float(np.sum(Ro, dtype=np.float64))) < 1e-6 * float(np.sum(Ro, dtype=np.float64))
    f2 = ((Fo[0] * Fo[0] + Fo[1] * Fo[1]) + Fo[2] * Fo[2]).max()
    assert abs(gs["f2_max_fine"] - f2) <= 1e-5 * f2
    g.close()


@pytest.mark.parametrize("name,pk,sk", CASES, ids=[c[0] for c in CASES])
def test_fine_kick_bitexact_given_force(name, pk, sk):
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    o.sigma_vi_new = np.float32(st["sigma_vi"] * 1.1)
    g.set_sigma(st["sigma_vi"], o.sigma_vi_new)
    g.fine_forces()
    F = g.get_field(C.FIELD_FORCE_F)
    g.fine_kick(A_MID, DT)
    o.fine_kick_global(F, A_MID, DT)
    np.testing.assert_array_equal(g.download()["vp"], o.state()["vp"])
    g.close()


@pytest.mark.parametrize("name,pk,sk", CASES, ids=[c[0] for c in CASES])
def test_coarse_force_and_kick(name, pk, sk):
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    g.coarse_density()
    rg = g.get_field(C.FIELD_RHO_C)
    gs = g.coarse_forces()
    r3 = o.coarse_density()
    assert rel_l2(rg, r3) < RHO_RTOL
    fo = o.coarse_force(r3)
    fg = g.get_field(C.FIELD_FORCE_C)
    assert rel_l2(fg, fo) < FORCE_RTOL
    # kick with the GPU's own force field on both sides: bit-exact vp and vmax
    ks = g.coarse_kick(A_MID, DT)
    vmax = o.coarse_kick(fg, A_MID, DT)
    np.testing.assert_array_equal(g.download()["vp"], o.state()["vp"])
    np.testing.assert_array_equal(np.asarray(ks["vmax"], np.float32), vmax)
    f2 = np.float32(((fo[0] * fo[0] + fo[1] * fo[1]) + fo[2] * fo[2]).max())
    assert abs(gs["f2_max_coarse"] - f2) <= 1e-5 * f2
    g.close()


def test_kernels_match_oracle():
    p = _params(dict(nc=24, nnt=2))
    g = C.CubeGPU(p)
    kc = g.get_field(C.FIELD_KERN_C)
    ko = O.kernel_c(p.nc, p.ncell)
    assert rel_l2(kc, ko) < 1e-5
    kf = g.get_field(C.FIELD_KERN_F)
    kfo = O.kernel_f(p.nf, p.nf_cutoff, p.pp_on, p.pp_range)
    assert rel_l2(kf, kfo) < 1e-5
    g.close()


@pytest.mark.parametrize("name,pk,sk", [CASES[0], CASES[3]], ids=[CASES[0][0], CASES[3][0]])
def test_pp_force(name, pk, sk):
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    a = g.ext_pp_force(A_MID, DT)
    b = o.pp_force(A_MID, DT)
    assert a["npairs"] == b["npairs"]
    assert a["itest1"] == b["itest1"] == st["xp"].shape[0]
    assert abs(a["f2_max_pp"] - b["f2_max_pp"]) <= 1e-5 * b["f2_max_pp"]
    vg = g.download()["vp"].astype(np.int64)
    vo = o.state()["vp"].astype(np.int64)
    d = np.abs(vg - vo)
    # FP32 pair sums vs the reference's FP64: codes may differ by one where the
    # pre-rounding value sits within the force tolerance of a half integer
    assert d.max() <= MAX_CODE_DIFF
    assert (d > 0).mean() < MAX_DIFF_FRAC
    g.close()


def test_pp_dense_bricks_match_oracle():
    # two cells hold ~3000 particles each: their bricks exceed the shared-memory
    # staging capacity and are redone cell by cell, and those cells go through
    # the global-memory kernel
    p = _params(dict(nc=24, nnt=2))
    st = synth.random_state(p, mean_per_cell=3, seed=21, clump=2, clump_mult=1000)
    g, o = make_pair(p, st)
    a = g.ext_pp_force(A_MID, DT)
    b = o.pp_force(A_MID, DT)
    assert a["pp_dense_bricks"] > 0
    assert a["npairs"] == b["npairs"]
    assert a["itest1"] == b["itest1"] == st["xp"].shape[0]
    assert abs(a["f2_max_pp"] - b["f2_max_pp"]) <= 1e-5 * b["f2_max_pp"]
    d = np.abs(g.download()["vp"].astype(np.int64) - o.state()["vp"].astype(np.int64))
    assert d.max() <= MAX_CODE_DIFF and (d > 0).mean() < MAX_DIFF_FRAC
    g.close()


@pytest.mark.parametrize("clump", [0, 2])
def test_pp_levels_agree_bitwise(clump):
    # every kernel (staged brick, staged cell, global-memory staging) sums a
    # particle's pairs in the same order (neighbour fine cells row by row,
    # each cell's particles by index), so the result does not depend on
    # which one handles it
    p = _params(dict(nc=24, nnt=2))
    st = synth.random_state(p, mean_per_cell=6, seed=22, clump=clump, clump_mult=600)
    # forced levels 1, 3 and 4 take every item in three parts; heavy = 1 walks
    # every particle of a crowded block with a warp (chunk sums folded in
    # order), heavy = 0 keeps the default threshold
    outs = []
    for level, heavy in ((0, 0), (1, 0), (2, 0), (3, 0), (4, 0), (5, 0), (0, 1), (3, 1), (4, 1)):
        g = C.CubeGPU(p)
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        s = np.float32(st["sigma_vi"])
        g.set_sigma(s, s)
        g.set_option(C.OPT_PP_LEVEL, level)
        g.set_option(C.OPT_PP_HEAVY, heavy)
        outs.append((g.ext_pp_force(A_MID, DT), g.download()["vp"]))
        g.close()
    if clump:
        assert outs[0][0]["pp_dense_bricks"] > 0
    for sb, vb in outs[1:]:
        assert np.array_equal(outs[0][1], vb)
        assert sb["npairs"] == outs[0][0]["npairs"] and sb["f2_max_pp"] == outs[0][0]["f2_max_pp"]


def test_particle_mesh_step_matches_oracle():
    p = _params(dict(nc=24, nnt=2))
    st = synth.random_state(p, seed=11, clump=10)
    g, o = make_pair(p, st)
    a = g.particle_mesh(A_MID, DT)
    b = o.particle_mesh(A_MID, DT)
    assert abs(a["f2_max_fine"] - b["f2_max_fine"]) <= 1e-5 * b["f2_max_fine"]
    assert abs(a["f2_max_coarse"] - b["f2_max_coarse"]) <= 1e-5 * b["f2_max_coarse"]
    vg = g.download()["vp"].astype(np.int64)
    vo = o.state()["vp"].astype(np.int64)
    d = np.abs(vg - vo)
    # two chained kicks (fine, then coarse from the re-decoded code), each from a
    # force recomputed by a different FFT: a one-code difference after the first
    # can round to two after the second, and the near-tie fraction doubles
    assert d.max() <= 2 * MAX_CODE_DIFF and (d > 0).mean() < 5 * MAX_DIFF_FRAC
    g.close()


def test_full_step_is_bitwise_deterministic():
    # two contexts, same input: every array and every statistic identical
    p = _params(dict(nc=48, nnt=2))
    st = synth.random_state(p, seed=21, clump=40)
    outs = []
    for _ in range(2):
        g = C.CubeGPU(p)
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        s = np.float32(st["sigma_vi"])
        g.set_sigma(s, s)
        stats = []
        for k in range(2):
            stats.append(g.update_x(np.float32(20.0), np.float32(30.0), st["vz_max"]))
            stats.append(g.ext_pp_force(A_MID, DT))
            stats.append(g.particle_mesh(A_MID, DT))
        outs.append((g.download(), stats))
        g.close()
    (a, sa), (b, sb) = outs
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    assert sa == sb


PP_FORCE_RTOL = 1e-5  # relative L2 of the FP32 pair-force sums vs the oracle's FP64 f_tot


@pytest.mark.parametrize("name,pk,sk", [
    CASES[0], CASES[2], CASES[3],
    ("dense_bricks", dict(nc=24, nnt=2, izipx=1, izipv=2), dict(mean_per_cell=3, seed=21, clump=2, clump_mult=1000)),
], ids=["uniform_x1", "uniform_x2", "clumped", "dense_bricks"])
def test_pp_force_vector_matches_fp64(name, pk, sk):
    # f_tot of every particle (ext_pp_force.f90:94-112): the GPU sums FP32
    # FP32 pair forces in a compensated sum, the oracle sums FP64 pair forces
    p = _params(pk)
    st = synth.random_state(p, **sk)
    g, o = make_pair(p, st)
    a = g.ext_pp_force(A_MID, DT)
    b = o.pp_force(A_MID, DT, want_force=True)
    assert a["npairs"] == b["npairs"]
    Fg = g.get_field(C.FIELD_FORCE_PP).astype(np.float64)
    Fo = b["f_tot"]
    err = rel_l2(Fg, Fo)
    mag = np.sqrt((Fo ** 2).sum(1))
    big = mag > 1e-3 * mag.max()
    worst = float(np.max(np.sqrt(((Fg - Fo) ** 2).sum(1))[big] / mag[big]))
    print("PP force vs FP64 (%s): rel-L2 %.3e, worst particle %.3e" % (name, err, worst))
    assert err < PP_FORCE_RTOL
    assert worst < 1e-4
    g.close()


def test_resort_buffers_after_a_failed_allocation():
    # host-side fault injection: the second of the general re-sort's four
    # buffers reports failure on first use; the step returns CUBE_ERR_NOMEM
    # with nothing launched on the half-made buffers, and the next step makes
    # all four and gives the state of a context that never failed
    p = _params(CASES[0][1])
    st = synth.random_state(p, **CASES[0][2])
    outs = []
    for inject in (False, True):
        g = C.CubeGPU(p)
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        g.set_sigma(st["sigma_vi"], st["sigma_vi"])
        g.set_option(C.OPT_RANK_WALK, 2)
        if inject:
            g.set_option(C.OPT_FAIL_ALLOC, 2)
            with pytest.raises(C.CubeError) as e:
                g.update_x(np.float32(28.0), np.float32(40.0), st["vz_max"])
            assert e.value.code == 9  # CUBE_ERR_NOMEM
        s = g.update_x(np.float32(28.0), np.float32(40.0), st["vz_max"])
        assert s["rank_walked"] == 2
        outs.append(g.download())
        g.close()
    for k in ("xp", "vp", "pid", "rhoc", "vfield"):
        np.testing.assert_array_equal(outs[0][k], outs[1][k])
