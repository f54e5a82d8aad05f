"""PP's prefilter against the unfiltered staging.

A particle whose 27 neighbouring fine cells hold no other particle has the
one list entry of itself and a zero pair force (ext_pp_force.f90:94-112);
the prefilter finds those particles from per-cell occupancy masks and stages
only the others, whose lists it leaves unchanged.  With the filter on, off and
automatic the pair forces, pair counts, force maxima and velocity codes must
be bitwise equal, in the plain and the fused PP+PM call and at every staging
level; on a Zel'dovich lattice (almost every particle alone) the filtered
call is also checked against the oracle.
"""
import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

O = pytest.importorskip("oracle.cube_oracle")

A_MID, DT = 0.4, 0.02
OFF, ON = 1, 2


def _params(nc=24, nnt=2, izipx=1, izipv=2):
    return P.CubeParams(nc=nc, nnt=nnt, izipx=izipx, izipv=izipv, pp_on=True, rsoft=0.1, mass_p=8.0,
                        box=100.0 * nc / 32)


def _lattice_state(p, z=49.0, seed=3):
    g = C.CubeGPU(p)
    try:
        sigma, _ = g.ic_zeldovich(z, seed)
        st = dict(g.download())
        st["sigma_vi"] = np.float32(sigma)
    finally:
        g.close()
    return st


def _pp(p, st, mode, level=0, fused=False):
    g = C.CubeGPU(p)
    try:
        g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        s = np.float32(st["sigma_vi"])
        g.set_sigma(s, s)
        g.set_option(C.OPT_PP_FILTER, mode)
        g.set_option(C.OPT_PP_LEVEL, level)
        if fused:
            stats, _ = g.pp_particle_mesh(A_MID, DT)
            F = None
        else:
            stats = g.ext_pp_force(A_MID, DT)
            F = g.get_field(C.FIELD_FORCE_PP)
        return stats, F, g.download()["vp"].copy()
    finally:
        g.close()


def _same(a, b):
    sa, Fa, va = a
    sb, Fb, vb = b
    assert sa["npairs"] == sb["npairs"] and sa["itest1"] == sb["itest1"]
    assert sa["f2_max_pp"] == sb["f2_max_pp"]
    if Fa is not None:
        assert np.array_equal(Fa.view(np.uint32), Fb.view(np.uint32))
    assert np.array_equal(va, vb)


STATES = [
    # Zel'dovich lattice at z = 49: nearly every particle alone in its fine-cell neighbourhood
    ("lattice", lambda p: _lattice_state(p)),
    # one particle per coarse cell on average: about a third have a neighbour
    ("sparse", lambda p: synth.random_state(p, mean_per_cell=1.0, seed=31)),
    # six per cell: nearly all have one
    ("uniform", lambda p: synth.random_state(p, mean_per_cell=6.0, seed=32)),
    # dense cells beside sparse ones: listed bricks and cells, global staging
    ("clumped", lambda p: synth.random_state(p, mean_per_cell=1.0, seed=33, clump=2, clump_mult=1500)),
]


@pytest.mark.parametrize("name,make", STATES, ids=[s[0] for s in STATES])
def test_filter_on_off_auto_bitwise(name, make):
    p = _params()
    st = make(p)
    off = _pp(p, st, OFF)
    _same(off, _pp(p, st, ON))
    _same(off, _pp(p, st, 0))
    _same(_pp(p, st, OFF, fused=True), _pp(p, st, ON, fused=True))


@pytest.mark.parametrize("level", [1, 2, 3, 4, 5])
def test_filter_agrees_at_every_level(level):
    p = _params()
    st = synth.random_state(p, mean_per_cell=1.0, seed=34, clump=3, clump_mult=400)
    _same(_pp(p, st, OFF), _pp(p, st, ON, level=level))


def test_filtered_lattice_matches_oracle():
    p = _params(nc=32, nnt=2)
    st = _lattice_state(p, seed=5)
    g = C.CubeGPU(p)
    g.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    g.set_sigma(s, s)
    g.set_option(C.OPT_PP_FILTER, ON)
    o = O.OracleImage(p)
    o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    o.sigma_vi = o.sigma_vi_new = s
    a = g.ext_pp_force(A_MID, DT)
    b = o.pp_force(A_MID, DT, want_force=True)
    n = st["xp"].shape[0]
    assert a["npairs"] == b["npairs"] and a["itest1"] == b["itest1"] == n
    # most particles have the one entry of themselves
    assert a["npairs"] < 1.5 * n
    Fg = g.get_field(C.FIELD_FORCE_PP).astype(np.float64)
    Fo = b["f_tot"]
    alone = ~np.any(Fo != 0.0, axis=1)
    assert alone.mean() > 0.5
    assert np.all(Fg[alone] == 0.0)
    err = float(np.linalg.norm(Fg - Fo) / max(np.linalg.norm(Fo), 1e-300))
    assert err < 1e-5
    d = np.abs(g.download()["vp"].astype(np.int64) - o.state()["vp"].astype(np.int64))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3
    g.close()
