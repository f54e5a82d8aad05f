"""The key the re-sort's general path sorts landings by reproduces the
reference's rank order, checked on the CPU oracle.

update_particle.f90:97-126 visits the source cells of each tile's extended
region in the order (layer, k, j, i) with layer = (k + ncb - 1) mod nlayer
(k, j, i local to the tile, 1 - ncb .. nt + ncb) and each cell's particles
in storage order; a particle's rank in its destination cell is its place in
that visit.  The CUDA path (cube_update.cu, k_sort_keys) sorts every
landing by (destination cell, layer of the source's z in the destination
tile's frame, source offsets z, y, x from the destination, index in the
source cell).  Here the oracle's new order is checked to be that key's
order, destination cell by destination cell, for steps that move particles
several cells (the case the counting path does not cover).
"""
import numpy as np
import pytest

from cafproject_gb300 import params as P
from cafproject_gb300 import synth
from oracle import cube_oracle as O


def coords(p, cid):
    nt, nnt = p.nt, p.nnt
    ix, iy, iz = cid % nt, (cid // nt) % nt, (cid // nt ** 2) % nt
    tile = cid // nt ** 3
    tx, ty, tz = tile % nnt, (tile // nnt) % nnt, tile // nnt ** 2
    return np.stack([tx * nt + ix, ty * nt + iy, tz * nt + iz], axis=1)


@pytest.mark.parametrize("nnt,nc,seed", [(2, 24, 31), (1, 24, 32), (2, 32, 33)])
def test_oracle_order_is_the_sort_key_order(nnt, nc, seed):
    p = P.CubeParams(nc=nc, nnt=nnt, pp_on=False, mass_p=8.0, izipx=1, izipv=2)
    st = synth.random_state(p, mean_per_cell=3, seed=seed, vsig=0.03, clump=4)
    o = O.OracleImage(p)
    o.load(st["xp"], st["vp"], st["pid"], st["rhoc"], st["vfield"])
    s = np.float32(st["sigma_vi"])
    o.sigma_vi = o.sigma_vi_new = s
    dt = np.float32(150.0)
    stats = o.update_x(np.float32(dt * 0.7), dt, st["vz_max"])
    new = o.state()
    nlayer = stats["nlayer"]
    n_old = st["xp"].shape[0]
    ncells = p.nc ** 3
    # old: each particle's source cell and index in it (pid = old index + 1)
    cs_old = np.concatenate([[0], np.cumsum(st["rhoc"].astype(np.int64))])
    cell_old = np.repeat(np.arange(ncells), st["rhoc"])
    l_old = np.arange(n_old) - cs_old[cell_old]
    # new: destination cell of each new index, the particle that landed there
    cell_new = np.repeat(np.arange(ncells), new["rhoc"])
    src = new["pid"].astype(np.int64) - 1
    sg = coords(p, cell_old[src])
    dg = coords(p, cell_new)
    off = (sg - dg + p.nc // 2) % p.nc - p.nc // 2  # nearest image: the frame the landing came from
    disp = np.abs(off).max()
    assert disp > 1  # beyond the counting path
    dl_z = dg[:, 2] - (dg[:, 2] // p.nt) * p.nt + 1
    ls_z = dl_z + off[:, 2]  # the source's z in the destination tile's frame
    assert ls_z.min() >= 1 - p.ncb and ls_z.max() <= p.nt + p.ncb
    layer = (ls_z + p.ncb - 1) % nlayer
    key = np.stack([cell_new, layer, off[:, 2], off[:, 1], off[:, 0], l_old[src]], axis=1)
    # within each destination cell the new order is the key's, strictly
    same = cell_new[1:] == cell_new[:-1]
    a, b = key[:-1][same], key[1:][same]
    diff = b - a
    first = np.argmax(diff != 0, axis=1)
    assert np.all(diff[np.arange(diff.shape[0]), first] > 0)
    if nnt == 1:
        assert new["pid"].shape[0] >= n_old  # periodic copies may land twice
