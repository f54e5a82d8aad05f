"""FP64 reference of the differentiable PM form -- TEST INFRASTRUCTURE ONLY.

The same map as cafproject_gb300/csrc/cube_dpm.cu, written with torch
float64 operations on the CPU so that autograd gives the FP64 reference
gradient and central finite differences can be taken in FP64.  It takes the
two spectral tables (IC filter, Green's function) as inputs, each with the
inverse transform's 1/n^3 folded in, exactly as the device uses them.  The
functions run on the device of their inputs: a float64 noise tensor on a GPU
makes the many forward passes of a finite-difference check affordable at the
workload size (float64 scatters there are summed in varying order, a
rounding of about 1e-16 relative).

The form has no counterpart in the reference (CUBE has no gradients); its
pieces restate the reference's step: the Zel'dovich initial conditions by
central differences of the potential (CUBEnu/work/utilities/
initial_conditions.f90:702-769), the drift by dt_mid
(CUBEnu/work/main/update_particle.f90:66) and the kick by a_mid*dt/(6 pi)
(CUBEnu/work/main/pm.f90:162), on a single cell-centred CIC mesh with the
discrete Green's function -4 pi/khat^2.  Parity unpinned: no reference
output exists for this form.
"""
import math

import numpy as np
import torch

DT = torch.float64


def _irfft3(spec, n):
    return torch.fft.irfftn(spec, s=(n, n, n))


def lattice(npd, step, device=None):
    """(np, 3) integer mesh cell of each particle's lattice point, in the
    order l = x + npd*(y + npd*z); the point itself is that cell's centre."""
    p = torch.arange(npd ** 3, device=device)
    return torch.stack([p % npd, (p // npd) % npd, p // (npd * npd)], 1) * step


def ic(noise, filt, npd, step, vf):
    """noise (npd**3,) -> displacement d and velocity v (np, 3):
    phi = C2R(filt * R2C(noise)), gd = phi(l+e) - phi(l-e),
    d = -step*gd/(8 pi), v = -step*gd*vf/(8 pi)."""
    n3 = float(npd) ** 3
    f = torch.as_tensor(filt, dtype=DT, device=noise.device)
    phi = _irfft3(torch.fft.rfftn(noise.reshape(npd, npd, npd)) * f, npd) * n3
    out_d, out_v = [], []
    for dim in (2, 1, 0):  # x is the last tensor dimension
        gd = (torch.roll(phi, -1, dim) - torch.roll(phi, 1, dim)).reshape(-1)
        s = step * gd / (8 * math.pi)
        out_d.append(-s)
        out_v.append(-s * vf)
    return torch.stack(out_d, 1), torch.stack(out_v, 1)


def _corners(d, ng, npd):
    step = ng // npd
    fl = torch.floor(d).detach()
    f = d - fl
    i0 = lattice(npd, step, d.device) + fl.long()
    for az in (0, 1):
        for ay in (0, 1):
            for ax in (0, 1):
                w = ((f[:, 0] if ax else 1 - f[:, 0]) * (f[:, 1] if ay else 1 - f[:, 1]) *
                     (f[:, 2] if az else 1 - f[:, 2]))
                ix = (i0[:, 0] + ax) % ng
                iy = (i0[:, 1] + ay) % ng
                iz = (i0[:, 2] + az) % ng
                yield (iz * ng + iy) * ng + ix, w


def deposit(d, ng, npd, mass):
    """CIC density on the cell-centred periodic ng^3 mesh, [z, y, x], of the
    particles at their lattice points plus displacements d."""
    rho = torch.zeros(ng ** 3, dtype=d.dtype, device=d.device)
    for idx, w in _corners(d, ng, npd):
        rho = rho.index_add(0, idx, mass * w)
    return rho.reshape(ng, ng, ng)


def potential(rho, green, ng):
    return _irfft3(torch.fft.rfftn(rho) * torch.as_tensor(green, dtype=DT, device=rho.device), ng) * float(ng) ** 3


def force_at(d, phi, ng, npd):
    """CIC interpolation of F = -(phi(c+e) - phi(c-e))/2."""
    comps = []
    for dim in (2, 1, 0):
        comps.append((-(torch.roll(phi, -1, dim) - torch.roll(phi, 1, dim)) / 2).reshape(-1))
    out = torch.zeros(d.shape[0], 3, dtype=d.dtype, device=d.device)
    for idx, w in _corners(d, ng, npd):
        out = out + w[:, None] * torch.stack([c[idx] for c in comps], 1)
    return out


def simulate(noise, filt, green, ng, npd, vf, drift, kick):
    step = ng // npd
    mass = float(ng) ** 3 / float(npd) ** 3
    d, v = ic(noise, filt, npd, step, vf)
    for dr, kk in zip(drift, kick):
        d = d + float(dr) * v
        phi = potential(deposit(d, ng, npd, mass), green, ng)
        v = v + float(kk) * force_at(d, phi, ng, npd)
    return d, v


def loss(noise, target, filt, green, ng, npd, vf, drift, kick):
    """sum over cells of (rho_final - target)^2 (the differentiable workload's loss)."""
    mass = float(ng) ** 3 / float(npd) ** 3
    d, _ = simulate(noise, filt, green, ng, npd, vf, drift, kick)
    return ((deposit(d, ng, npd, mass) - target) ** 2).sum()


def green_table(ng):
    """-4 pi/khat^2 / ng^3 on the half spectrum [z, y, x], 0 at k = 0."""
    k = np.arange(ng)
    s = 2 * np.sin(np.pi * k / ng)
    sx = s[: ng // 2 + 1]
    k2 = sx[None, None, :] ** 2 + s[None, :, None] ** 2 + s[:, None, None] ** 2
    with np.errstate(divide="ignore"):
        g = -4 * np.pi / k2 / float(ng) ** 3
    g[0, 0, 0] = 0.0
    return g
