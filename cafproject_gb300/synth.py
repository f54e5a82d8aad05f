"""Random but valid compressed states for parity tests and quick runs.

A state is the reference's disjoint checkpoint layout (rhoc per cell in tile
order, particles sorted by cell): Poisson counts per coarse cell, uniform
in-cell offsets, Gaussian residual velocities stored with the atan code of
update_particle.f90:117, and a Gaussian coarse velocity field.  ``clump``
adds dense cells so PP pairs, multi-particle cells and large ranks appear.
"""
import numpy as np

PI_F = np.float32(4.0) * np.arctan(np.float32(1.0))


def vcoef(sigma):
    s = np.float32(np.sqrt(np.float32(PI_F / np.float32(2.0))))
    return np.float64(s) / (np.float64(np.float32(sigma)) * 2.5)


def encode(v, sigma, izipv):
    nvm1 = float((1 << (8 * izipv)) - 1)
    u = (nvm1 * np.arctan(vcoef(sigma) * v)) / np.float64(PI_F)
    return (np.sign(u) * np.floor(np.abs(u) + 0.5)).astype(np.int64)


def random_state(p, mean_per_cell=8.0, seed=0, vsig=0.02, clump=0, clump_mult=40):
    rng = np.random.default_rng(seed)
    ncells = p.nc ** 3
    lam = np.full(ncells, mean_per_cell)
    if clump:
        hot = rng.choice(ncells, size=clump, replace=False)
        lam[hot] *= clump_mult
    counts = rng.poisson(lam).astype(np.int32)
    n = int(counts.sum())
    hx = 1 << (8 * p.izipx - 1)
    xp = rng.integers(-hx, hx, size=(n, 3)).astype(p.xdtype)
    sigma = np.float32(vsig / 3.0)
    res = rng.normal(0.0, float(sigma), size=(n, 3))
    vp = encode(res, sigma, p.izipv).astype(p.vdtype)
    vfield = rng.normal(0.0, vsig, size=(ncells, 3)).astype(np.float32)
    pid = np.arange(1, n + 1, dtype=np.int32)
    return dict(xp=xp, vp=vp, pid=pid, rhoc=counts, vfield=vfield, sigma_vi=sigma,
                vz_max=float(np.abs(vfield[:, 2]).max() + 6 * sigma))
