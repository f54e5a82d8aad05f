"""The bit rule of PP's prefilter neighbour mask (k_pp_nbmask in
cafproject_gb300/csrc/cube_pp.cu), restated on the host and checked against a
brute-force search over fine cells on a small periodic mesh.

A coarse cell's 64 fine sub-cells are bits x + 4y + 16z.  A sub-cell "has a
neighbour" when one of its 26 neighbouring fine cells (periodic, across coarse
cells) holds a particle, or it holds two itself: a particle there has a PP
list longer than itself (ext_pp_force.f90:94-96).
"""
import random

M64 = (1 << 64) - 1
LAY0 = [0x1111111111111111, 0x000F000F000F000F, 0x000000000000FFFF]
STRIDE = [1, 4, 16]


def up(m, d):
    return ((m << STRIDE[d]) & M64) & ~LAY0[d] & M64


def down(m, d):
    return (m >> STRIDE[d]) & ~(LAY0[d] << (3 * STRIDE[d])) & M64


def ex(m, d):
    return up(m, d) | down(m, d)


def dil(m, d):
    return m | ex(m, d)


def nbmask(occ, multi, c, nc):
    # the kernel's rule: within the cell a neighbour differs by one in z (any
    # x, y), in y only (any x), or in x only; a surrounding cell contributes
    # its facing layer(s), moved next to this cell and spread in the others
    own = occ[c]
    dxo = dil(own, 0)
    e = ex(dil(dxo, 1), 2) | ex(dxo, 1) | ex(own, 0)
    for k in range(27):
        o = (k % 3 - 1, (k // 3) % 3 - 1, k // 9 - 1)
        if o == (0, 0, 0):
            continue
        l = occ[tuple((c[d] + o[d]) % nc for d in range(3))]
        for d in range(3):
            if o[d] < 0:
                l = (l >> (3 * STRIDE[d])) & LAY0[d]
            elif o[d] > 0:
                l = ((l << (3 * STRIDE[d])) & M64) & (LAY0[d] << (3 * STRIDE[d]))
        for d in range(3):
            if o[d] == 0:
                l = dil(l, d)
        e |= l
    return e | multi[c]


def brute(occ, multi, c, nc):
    a = multi[c]
    for s in range(64):
        f = (4 * c[0] + (s & 3), 4 * c[1] + ((s >> 2) & 3), 4 * c[2] + (s >> 4))
        for dz in (-1, 0, 1):
            for dy in (-1, 0, 1):
                for dx in (-1, 0, 1):
                    if (dx, dy, dz) == (0, 0, 0):
                        continue
                    g = [(f[i] + (dx, dy, dz)[i]) % (4 * nc) for i in range(3)]
                    if occ[(g[0] // 4, g[1] // 4, g[2] // 4)] >> ((g[0] % 4) + 4 * ((g[1] % 4) + 4 * (g[2] % 4))) & 1:
                        a |= 1 << s
    return a


def test_neighbour_mask_matches_brute_force():
    nc = 4
    rng = random.Random(7)
    occ, multi = {}, {}
    for x in range(nc):
        for y in range(nc):
            for z in range(nc):
                o = mu = 0
                for _ in range(rng.choice([0, 0, 1, 2, 3, 8])):
                    b = rng.randrange(64)
                    if o >> b & 1:
                        mu |= 1 << b
                    o |= 1 << b
                occ[(x, y, z)], multi[(x, y, z)] = o, mu
    for c in occ:
        assert nbmask(occ, multi, c, nc) == brute(occ, multi, c, nc), c
