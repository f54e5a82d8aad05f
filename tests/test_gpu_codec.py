"""The kernels' velocity encode (boundary table + FP32 estimate) must equal the
reference's FP64 formula nint((nvbin-1)*atan(vcoef*v)/pi) bit for bit."""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

PI_F = np.float32(4.0) * np.arctan(np.float32(1.0))


def probe_values(sigma, izipv, rng):
    nvm1 = (1 << (8 * izipv)) - 1
    nmax = nvm1 // 2
    c = synth.vcoef(sigma)
    n = np.arange(1, nmax + 1, dtype=np.float64)
    # near every bin edge: the analytic edge and +-4 ulps around it
    edge = np.tan((n - 0.5) * np.float64(PI_F) / nvm1) / c
    vals = [edge]
    for k in range(1, 5):
        vals.append(np.nextafter(edge, np.inf) if k == 1 else np.nextafter(vals[-1], np.inf))
    lo = edge.copy()
    for k in range(4):
        lo = np.nextafter(lo, -np.inf)
        vals.append(lo.copy())
    v = np.concatenate(vals)
    v = v[np.isfinite(v)]
    rand = np.concatenate([rng.normal(0, s, 200000) for s in (sigma, 10 * sigma, 1000 * sigma)])
    special = np.array([0.0, -0.0, 1e-300, -1e-300, 5e-324, 1e300, -1e300, np.inf, -np.inf])
    v = np.concatenate([v, -v, rand, special])
    return v


@pytest.mark.parametrize("izipv", [1, 2])
@pytest.mark.parametrize("sigma", [0.003, 0.05, 2.0])
def test_table_encode_equals_fp64_formula(izipv, sigma):
    p = P.CubeParams(nc=24, nnt=2, izipv=izipv)
    g = C.CubeGPU(p)
    rng = np.random.default_rng(7)
    v = probe_values(np.float32(sigma), izipv, rng)
    direct, table = g.codec_check(np.float32(sigma), v)
    bad = np.nonzero(direct != table)[0]
    assert bad.size == 0, (v[bad[:5]], direct[bad[:5]], table[bad[:5]])
    # against the host FP64 formula: differences only where the pre-rounding
    # value is within 1e-9 of a half integer (different atan implementations)
    fin = np.isfinite(v)
    ref = synth.encode(v[fin], np.float32(sigma), izipv)
    d = np.nonzero(ref != direct[fin])[0]
    if d.size:
        nvm1 = (1 << (8 * izipv)) - 1
        u = nvm1 * np.arctan(synth.vcoef(np.float32(sigma)) * v[fin][d]) / np.float64(PI_F)
        assert np.all(np.abs(np.abs(u - np.trunc(u)) - 0.5) < 1e-9)
    # away from the probed edges (the random draws) the two formulas agree
    nrand = 600000
    r0 = v.size - 9 - nrand
    rr = np.arange(r0, r0 + nrand)
    assert np.array_equal(synth.encode(v[rr], np.float32(sigma), izipv), direct[rr])
    g.close()


def _kick_pair(exact, seed, nsteps=2):
    p = P.CubeParams(nc=96, nnt=2, pp_on=False, mass_p=8.0)
    st = synth.random_state(p, mean_per_cell=6, seed=seed, vsig=0.02, clump=200)
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    g.set_sigma(s, np.float32(s * 1.05))
    g.set_option(C.OPT_EXACT_KICKS, int(exact))
    vmax = []
    for _ in range(nsteps):
        g.fine_forces()
        g.fine_kick(0.4, 0.02)
        g.set_sigma(np.float32(s * 1.05), np.float32(s * 1.05))
        g.coarse_forces()
        vmax.append(g.coarse_kick(0.4, 0.02)["vmax"])
    out = g.download()["vp"]
    g.close()
    return out, vmax


def test_certified_kicks_equal_exact_chain():
    # 5M particles, two fine+coarse kicks each (the second coarse kick uses the
    # vmax threshold of the first): the certified fast path must reproduce the
    # full FP64 chain on every velocity code and every vmax bit
    for seed in (1, 2):
        a, va = _kick_pair(False, seed)
        b, vb = _kick_pair(True, seed)
        np.testing.assert_array_equal(a, b)
        np.testing.assert_array_equal(np.asarray(va, np.float32), np.asarray(vb, np.float32))


def _full_steps(exact, seed):
    p = P.CubeParams(nc=72, nnt=2, pp_on=True, rsoft=0.1, mass_p=8.0)
    st = synth.random_state(p, mean_per_cell=5, seed=seed, vsig=0.02, clump=100)
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    g.set_sigma(s, s)
    g.set_option(C.OPT_EXACT_KICKS, int(exact))
    stats = []
    for _ in range(3):
        stats.append(g.update_x(np.float32(30.0), np.float32(40.0), st["vz_max"]))
        stats.append(g.ext_pp_force(0.4, 0.02))
        stats.append(g.particle_mesh(0.4, 0.02))
    out = g.download()
    g.close()
    return out, stats


def test_fast_paths_equal_fp64_expressions_over_full_steps():
    # three full steps (re-sort with multi-cell drifts, PP, fine and coarse
    # kicks) with every certified fast path on, and with FP64 everywhere
    a, sa = _full_steps(False, 3)
    b, sb = _full_steps(True, 3)
    for k in a:
        np.testing.assert_array_equal(a[k], b[k])
    for x, y in zip(sa, sb):
        for k in ("nplocal", "nlost", "ndup", "nlayer", "npairs", "f2_max_fine", "f2_max_coarse", "vmax",
                  "sigma_vi_new"):
            assert x[k] == y[k], k


def test_kick_division_by_constant_is_ieee_for_every_float():
    # the kick terms' /6 and /pi use an FMA-corrected reciprocal product
    g = C.CubeGPU(P.CubeParams(nc=24, nnt=2, pp_on=True))
    try:
        assert g.arith_check() == (0, 0)
    finally:
        g.close()
