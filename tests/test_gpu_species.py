"""Two particle species (CUBEnu): a linked context shares the owner's meshes.
Splitting one species' particles between the two must leave the physics
unchanged: the same forces (up to the order of the density sums) and so the
same kicks."""
import os

import numpy as np
import pytest

from cafproject_gb300 import cube as C
from cafproject_gb300 import params as P
from cafproject_gb300 import synth

pytestmark = pytest.mark.gpu

A_MID, DT = 0.4, 0.02


def _split(st):
    """Per cell, the first half of its particles and the rest, as two states."""
    cnt = st["rhoc"].astype(np.int64)
    start = np.concatenate([[0], np.cumsum(cnt)[:-1]])
    na = (cnt + 1) // 2
    rank = np.arange(cnt.sum()) - np.repeat(start, cnt)
    in_a = rank < np.repeat(na, cnt)
    mk = lambda m, c: dict(xp=st["xp"][m], vp=st["vp"][m], pid=st["pid"][m], rhoc=c.astype(np.int32),
                           vfield=st["vfield"])
    return mk(in_a, na), mk(~in_a, cnt - na), in_a


def test_split_species_match_single_species():
    p = P.CubeParams(nc=24, nnt=2, pp_on=False, box=75.0)
    st = synth.random_state(p, mean_per_cell=6, seed=61, clump=8)
    s = np.float32(st["sigma_vi"])
    one = C.CubeGPU(p)
    try:
        one.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        one.set_sigma(s, s)
        r1 = one.particle_mesh(A_MID, DT)
        v1 = one.download()["vp"].reshape(-1, 3)
    finally:
        one.close()
    sa, sb, in_a = _split(st)
    a = C.CubeGPU(p)
    b = C.CubeGPU(P.CubeParams(nc=24, nnt=2, pp_on=False, box=75.0), owner=a)
    try:
        for g, x in ((a, sa), (b, sb)):
            g.upload(x["xp"], x["vp"], x["pid"], x["rhoc"], x["vfield"])
            g.set_sigma(s, s)
        ra, rb = a.particle_mesh2(b, A_MID, DT)
        va = a.download()["vp"].reshape(-1, 3)
        vb = b.download()["vp"].reshape(-1, 3)
    finally:
        b.close()
        a.close()
    d = np.abs(np.concatenate([va, vb]).astype(np.int64) - np.concatenate([v1[in_a], v1[~in_a]]).astype(np.int64))
    assert d.max() <= 1 and (d > 0).mean() < 1e-3
    assert abs(ra["f2_max_fine"] - r1["f2_max_fine"]) <= 1e-5 * r1["f2_max_fine"]
    vm = np.maximum(np.asarray(ra["vmax"]), np.asarray(rb["vmax"]))
    np.testing.assert_allclose(vm, r1["vmax"], rtol=1e-5)


def test_linked_species_checkpoint_files(tmp_path):
    p = P.CubeParams(nc=24, nnt=2, pp_on=True, box=75.0)
    q = P.CubeParams(nc=24, nnt=2, pp_on=False, izipx=2, izipv=2, mass_p=1.0, box=75.0)
    st = synth.random_state(p, seed=62)
    nu = synth.random_state(q, seed=63, mean_per_cell=3)
    a = C.CubeGPU(p)
    b = C.CubeGPU(q, owner=a)
    try:
        a.upload(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
        a.set_sigma(st["sigma_vi"], st["sigma_vi"])
        b.upload(nu["xp"], nu["vp"], nu["pid"], nu["rhoc"], nu["vfield"])
        b.set_sigma(nu["sigma_vi"], nu["sigma_vi"])
        n_nu = nu["xp"].shape[0]
        a.checkpoint_write(str(tmp_path), 5.0, nplocal_nu=n_nu, izipx_nu=2, izipv_nu=2,
                           sigma_vi_nu=float(nu["sigma_vi"]))
        b.checkpoint_write(str(tmp_path), 5.0)
        names = sorted(os.listdir(tmp_path))
        assert "5.000_xp_nu_1.bin" in names and "5.000_vc_nu_1.bin" in names and "5.000_info_1.bin" in names
        raw = np.fromfile(tmp_path / "5.000_xp_nu_1.bin", np.int16).reshape(-1, 3)
        np.testing.assert_array_equal(raw, nu["xp"].reshape(-1, 3))
        c = C.CubeGPU(p)
        d = C.CubeGPU(q, owner=c)
        try:
            c.checkpoint_read(str(tmp_path), 5.0)
            hdr = d.checkpoint_read(str(tmp_path), 5.0)
            assert hdr["nplocal_nu"] == n_nu
            back = d.download()
            for k in ("xp", "vp", "pid", "rhoc"):
                np.testing.assert_array_equal(back[k].reshape(nu[k].shape), nu[k])
            assert d.get_sigma()[0] == np.float32(nu["sigma_vi"])
        finally:
            d.close()
            c.close()
    finally:
        b.close()
        a.close()


def test_linked_species_needs_the_owner_geometry():
    p = P.CubeParams(nc=24, nnt=2, pp_on=True)
    a = C.CubeGPU(p)
    try:
        with pytest.raises(C.CubeError):
            C.CubeGPU(P.CubeParams(nc=32, nnt=2, pp_on=False), owner=a)
        with pytest.raises(C.CubeError):
            C.CubeGPU(P.CubeParams(nc=24, nnt=2, pp_on=True), owner=a)
    finally:
        a.close()
