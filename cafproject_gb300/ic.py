"""Synthetic initial conditions in CUBE's compressed checkpoint layout.

Input generator for tests and the benchmark (torch on CPU or GPU; it is not
one of the library's CUDA kernels).  It follows the reference IC program
CUBEnu/work/utilities/initial_conditions.f90 step by step, with two stated
substitutions:

* the CAMB transfer table is replaced by the Eisenstein & Hu (1998) no-wiggle
  fitting formula (their eqs. 26, 28-31), normalised to sigma_8 with the
  reference's top-hat sum (initial_conditions.f90:213-225) and grown with its
  Dgrow (:930-943);
* the gfortran ``random_number`` stream is replaced by a counter-based hash
  (the murmur3 32-bit finaliser applied to seed and cell index), so the noise
  is identical on every device and thread count.

The remaining steps are the reference's: Box-Muller (:292-300), delta(k) scaling
(:306-330), the discrete -4 pi/k^2 potential with the real-space correction
(:433-503), Zel'dovich displacement by central differences of phi
(:702-769), the per-cell mean velocity field and the atan velocity code
(:744-754), and xp = floor(x/x_resolution) wrapped to izipx bytes (:741).
One stated simplification: sigma_vi is the measured rms of the residual
velocities / sqrt(3) (the form update_xp uses every step,
update_particle.f90:224) instead of the reference's sigma_v(a,r) tables.
Particles inside a cell keep their Lagrangian order.
"""
import math

import numpy as np
import torch

PI_F = float(np.float32(4.0) * np.arctan(np.float32(1.0)))


def _fmix32(h):
    h = h & 0xFFFFFFFF
    h = h ^ (h >> 16)
    h = (h * 0x85EBCA6B) & 0xFFFFFFFF
    h = h ^ (h >> 13)
    h = (h * 0xC2B2AE35) & 0xFFFFFFFF
    h = h ^ (h >> 16)
    return h


def uniform_noise(n, seed, device):
    """n^3 uniforms in [0,1) from a counter hash of (seed, linear index)."""
    out = torch.empty(n ** 3, dtype=torch.float32, device=device)
    chunk = 1 << 26
    s = _fmix32(torch.tensor(seed * 0x9E3779B1 + 0x7F4A7C15, dtype=torch.int64)).item()
    for a in range(0, n ** 3, chunk):
        b = min(n ** 3, a + chunk)
        idx = torch.arange(a, b, dtype=torch.int64, device=device)
        h = _fmix32(_fmix32(idx ^ s) + s)
        out[a:b] = (h >> 8).to(torch.float32) * (1.0 / 16777216.0)
    return out.view(n, n, n)


def eh_nowiggle(k, omega_m, h, omega_b=0.045, tcmb=2.7255):
    """Eisenstein & Hu (1998) zero-baryon-oscillation transfer function; k in h/Mpc."""
    theta = tcmb / 2.7
    omh2 = omega_m * h * h
    obh2 = omega_b * h * h
    fb = omega_b / omega_m
    s = 44.5 * np.log(9.83 / omh2) / np.sqrt(1.0 + 10.0 * obh2 ** 0.75)
    alpha = 1.0 - 0.328 * np.log(431.0 * omh2) * fb + 0.38 * np.log(22.3 * omh2) * fb * fb
    kmpc = k * h
    gamma_eff = omega_m * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * kmpc * s) ** 4))
    q = k * theta * theta / gamma_eff
    L0 = np.log(2.0 * math.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def dgrow(a, om, ol):
    """Carroll-Press-Turner growth normalised to a=1 (initial_conditions.f90:930-943)."""
    hsq = om / a ** 3 + (1 - om - ol) / a ** 2 + ol
    oma = om / (a ** 3 * hsq)
    ola = ol / hsq
    g = 2.5 * om / (om ** (4.0 / 7) - ol + (1 + om / 2) * (1 + ol / 70))
    ga = 2.5 * oma / (oma ** (4.0 / 7) - ola + (1 + oma / 2) * (1 + ola / 70))
    return a * ga / g


def vfactor(a, om, ol):
    """a^2 H for the Zel'dovich velocity (initial_conditions.f90:971-982, no neutrinos)."""
    lm = ol / om
    km = (1 - om - ol) / om
    H = 2.0 / (3.0 * math.sqrt(a ** 3)) * math.sqrt(1 + a * km + a ** 3 * lm)
    return a * a * H


def delta2_table(p, a, nk=1000):
    """Delta^2(k) table normalised to sigma_8 at scale factor a."""
    k = np.logspace(-4, 2, nk)
    d2 = eh_nowiggle(k, p.omega_m, p.h0) ** 2 * k ** (3 + p.n_s) / (2 * math.pi ** 2)
    dk = np.empty(nk)
    dk[0] = k[1] / 2
    dk[1:-1] = (k[2:] - k[:-2]) / 2
    dk[-1] = k[-1] - k[-2]
    kmax = 2 * math.pi * math.sqrt(3.0) * (p.nf // 2) / p.box
    x = k * 8
    w = 3 * (np.sin(x) - np.cos(x) * x) / x ** 3
    sel = k <= kmax
    v8 = np.sum((d2 * w * w * dk / k)[sel])
    return k, d2 * (p.s8 ** 2 / v8) * dgrow(a, p.omega_m, p.omega_l) ** 2


def _loglog_interp(lx, xt, yt):
    """exp of the linear interpolation of yt(xt) at lx, on lx's device (as interp_tf,
    initial_conditions.f90:895-916, in log-log)."""
    xt_t = torch.tensor(xt, dtype=torch.float32, device=lx.device)
    yt_t = torch.tensor(yt, dtype=torch.float32, device=lx.device)
    lx = lx.clamp(float(xt[0]), float(xt[-1]))
    i = torch.searchsorted(xt_t, lx.contiguous()).clamp(1, len(xt) - 1)
    x0, x1 = xt_t[i - 1], xt_t[i]
    y0, y1 = yt_t[i - 1], yt_t[i]
    return torch.exp(y0 + (y1 - y0) * (lx - x0) / (x1 - x0))


def _kgrid(n, device, dtype=torch.float64):
    f = torch.fft.fftfreq(n, d=1.0 / n, device=device).to(dtype)
    fr = torch.arange(n // 2 + 1, device=device, dtype=dtype)
    return f.view(n, 1, 1), f.view(1, n, 1), fr.view(1, 1, n // 2 + 1)


def potential(p, a, seed, device="cpu"):
    """phi on the fine grid (nf^3, [z,y,x]) following initial_conditions.f90:250-541."""
    nf = p.nf
    r3 = uniform_noise(nf, seed, device)
    # Box-Muller on pairs along x (initial_conditions.f90:292-300)
    u1 = r3[:, :, 0::2]
    u2 = r3[:, :, 1::2]
    rr = torch.sqrt(-2.0 * torch.log(1.0 - u2))
    th = 2.0 * PI_F * u1
    g = torch.empty_like(r3)
    g[:, :, 0::2] = rr * torch.cos(th)
    g[:, :, 1::2] = rr * torch.sin(th)
    del r3, u1, u2, rr, th
    ck = torch.fft.rfftn(g)
    del g
    kz, ky, kx = _kgrid(nf, device, torch.float32)
    kr = torch.sqrt(kx * kx + ky * ky + kz * kz).clamp_min(1.0)
    ktab, d2tab = delta2_table(p, a)
    d2 = _loglog_interp(torch.log((2 * math.pi / p.box) * kr), np.log(ktab), np.log(d2tab))
    ck *= torch.sqrt(d2 / (4 * math.pi) * (nf / kr)) * (nf / kr)
    del d2
    ck[0, 0, 0] = 0
    # potential kernel -4 pi / khat^2 (initial_conditions.f90:433-460)
    sx = 2 * torch.sin(math.pi * kx / nf)
    sy = 2 * torch.sin(math.pi * ky / nf)
    sz = 2 * torch.sin(math.pi * kz / nf)
    ks = (sx * sx + sy * sy + sz * sz).clamp_min(1.0 / nf ** 2)
    kern = (-4 * math.pi / ks).to(torch.complex64)
    kern[0, 0, 0] = 0
    # real-space correction (initial_conditions.f90:462-503)
    rk = torch.fft.irfftn(kern, s=(nf, nf, nf))
    del kern
    phi8 = (rk[0, 0, 8] + rk[0, 8, 0] + rk[8, 0, 0] + rk[0, 0, nf - 8] + rk[0, nf - 8, 0] + rk[nf - 8, 0, 0]) / 6
    c = torch.fft.fftfreq(nf, d=1.0 / nf, device=device).float()
    rr = torch.sqrt(c.view(nf, 1, 1) ** 2 + c.view(1, nf, 1) ** 2 + c.view(1, 1, nf) ** 2)
    rk = torch.where(rr > 8, rk - (phi8 + 1.0 / 8.0), torch.where(rr > 0, -1.0 / rr.clamp_min(1e-30),
                                                                   torch.full_like(rk, -2.5)))
    del rr
    kk = torch.fft.rfftn(rk).real
    del rk
    phi = torch.fft.irfftn(kk * ck, s=(nf, nf, nf))
    return phi


def zeldovich(p, z_init, seed, device="cpu"):
    """Particles in the disjoint checkpoint layout: dict(xp, vp, pid, rhoc, vfield, sigma_vi, a)."""
    a = 1.0 / (1.0 + z_init)
    nf, nc, nt, nnt = p.nf, p.nc, p.nt, p.nnt
    npd = nc * p.np_nc
    step = p.ncell // p.np_nc
    phi = potential(p, a, seed, device)
    vf = vfactor(a, p.omega_m, p.omega_l)
    # Lagrangian grid: particle i sits at fine cell step*i (+1 in 1-based), xq in coarse units
    q1 = torch.arange(npd, device=device, dtype=torch.int64)
    fine = step * q1
    xq1 = q1.double() / p.np_nc + 0.5 / p.ncell
    iz, iy, ix = torch.meshgrid(fine, fine, fine, indexing="ij")
    ip = lambda t: (t + 1) % nf
    im = lambda t: (t - 1) % nf
    gx = (phi[iz, iy, ip(ix)] - phi[iz, iy, im(ix)]).double().reshape(-1)
    gy = (phi[iz, ip(iy), ix] - phi[iz, im(iy), ix]).double().reshape(-1)
    gz = (phi[ip(iz), iy, ix] - phi[im(iz), iy, ix]).double().reshape(-1)
    del phi
    qz, qy, qx = torch.meshgrid(xq1, xq1, xq1, indexing="ij")
    pos = []
    for q, gd in ((qx, gx), (qy, gy), (qz, gz)):
        x = q.reshape(-1) - gd / (8 * PI_F * p.ncell)
        pos.append(torch.remainder(x, float(nc)))
    vel = [-gd / (8 * PI_F) * vf for gd in (gx, gy, gz)]
    del gx, gy, gz, qx, qy, qz
    # cell = ceiling(x) (1-based); in 0-based global coordinates cell-1
    cells = []
    for x in pos:
        c = torch.ceil(x).long() - 1
        c = torch.remainder(c, nc)
        cells.append(c)
    cx, cy, cz = cells
    cid = (cx % nt) + nt * ((cy % nt) + nt * ((cz % nt) + nt * ((cx // nt) + nnt * ((cy // nt) + nnt * (cz // nt)))))
    lag = torch.arange(cid.numel(), device=device, dtype=torch.int64)
    order = torch.argsort(cid * cid.numel() + lag)
    cid = cid[order]
    ncells = nc ** 3
    rhoc = torch.bincount(cid, minlength=ncells).to(torch.int32)
    vfield = torch.zeros(ncells, 3, dtype=torch.float64, device=device)
    for d in range(3):
        vfield[:, d].index_add_(0, cid, vel[d][order])
    vfield = (vfield / rhoc.clamp_min(1).double().unsqueeze(1)).float()
    res = torch.stack([vel[d][order] - vfield[cid, d].double() for d in range(3)], dim=1)
    sigma_vi = float(np.float32(math.sqrt(float((res * res).sum()) / cid.numel()) / math.sqrt(3.0)))
    nvm1 = float((1 << (8 * p.izipv)) - 1)
    coef = float(np.float32(math.sqrt(np.float32(PI_F / 2)))) / (np.float64(np.float32(sigma_vi)) * 2.5)
    u = (nvm1 * torch.atan(coef * res)) / PI_F
    vp = (torch.sign(u) * torch.floor(torch.abs(u) + 0.5)).long()
    xres = 1.0 / (1 << (8 * p.izipx))
    m = 1 << (8 * p.izipx)
    xp = torch.stack([torch.floor(pos[d][order] / xres).long() for d in range(3)], dim=1)
    xp = torch.remainder(xp, m)
    xp = torch.where(xp >= m // 2, xp - m, xp)
    vm = 1 << (8 * p.izipv)
    vp = torch.where(vp >= vm // 2, vp - vm, vp)
    # pid = 1-based Lagrangian fine index (initial_conditions.f90:757-761)
    l = lag[order]
    lx, ly, lz = l % npd, (l // npd) % npd, l // (npd * npd)
    pid = (step * lx + nf * (step * ly) + nf * nf * (step * lz) + 1).to(torch.int32)
    xdt = torch.int8 if p.izipx == 1 else torch.int16
    vdt = torch.int8 if p.izipv == 1 else torch.int16
    return dict(xp=xp.to(xdt), vp=vp.to(vdt), pid=pid, rhoc=rhoc, vfield=vfield, sigma_vi=sigma_vi, a=a,
                vmax=[float(v.abs().max()) for v in vel])


def to_numpy(ic):
    return {k: (v.cpu().numpy() if torch.is_tensor(v) else v) for k, v in ic.items()}
