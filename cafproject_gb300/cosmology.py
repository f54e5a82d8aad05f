"""Host-side time stepping: timestep and expansion (CUBEnu/work/main/timestep.f90).

This scalar logic stays on the CPU in the GB300 design, as in the reference:
it reads the force maxima the device returns and produces dt, a_mid and the
checkpoint flags.  Arithmetic follows the reference's kinds: ``real`` (FP32)
for a, dt, da and the constraints; FP64 inside ``expansion``.  Note the
literal ``4.0/9.0`` is a default-real quotient widened to real(8)
(timestep.f90:145), reproduced here.
"""
from dataclasses import dataclass, field

import numpy as np

f32 = np.float32
PI_F = f32(4.0) * np.arctan(f32(1.0))
GG = f32(1.0) / f32(6.0) / PI_F  # variables.f90:15


def expansion(a0, dt0, omega_m, omega_l, wde=-1.0):
    """Third-order Friedmann step over dt0 in two halves (timestep.f90:133-177)."""
    om, ol, w = f32(omega_m), f32(omega_l), f32(wde)
    dt_x = f32(f32(dt0) / f32(2))
    omhsq = np.float64(f32(4.0) / f32(9.0))
    e3w = np.float64(f32(-3) * w)
    curv = np.float64(f32(f32(1.0) - om) - ol)

    def half(ax):
        ax = np.float64(ax)
        a3rlm = ax ** e3w * np.float64(ol) / np.float64(om)
        arkm = ax * curv / np.float64(om)
        adot = np.sqrt(omhsq * ax ** 3 * (1.0 + arkm + a3rlm))
        addot = ax ** 2 * omhsq * (1.5 + 2.0 * arkm + 1.5 * np.float64(f32(1.0) - w) * a3rlm)
        atdot = ax * adot * omhsq * (3.0 + 6.0 * arkm + 1.5 * np.float64(f32(2.0) - f32(3.0) * w)
                                      * np.float64(f32(1.0) - w) * a3rlm)
        dx = np.float64(dt_x)
        return f32(adot * dx + (addot * dx ** 2) / 2.0 + (atdot * dx ** 3) / 6.0)

    da1 = half(a0)
    da2 = half(f32(f32(a0) + da1))
    return da1, da2


@dataclass
class TimeState:
    """The scalar module state the reference keeps in `variables`/`sim`."""

    a: np.float32
    omega_m: float = 0.3
    omega_l: float = 0.7
    t: np.float32 = f32(0)
    tau: np.float32 = f32(0)
    dt: np.float32 = f32(0)
    dt_old: np.float32 = f32(0)
    da: np.float32 = f32(0)
    a_mid: np.float32 = f32(0)
    istep: int = 0
    dt_fine: np.float32 = f32(1000)
    dt_coarse: np.float32 = f32(1000)
    dt_pp: np.float32 = f32(1000)
    dt_vmax: np.float32 = f32(1000)
    vz_max: np.float32 = f32(0)
    ra_max: float = 0.2
    z_checkpoints: list = field(default_factory=lambda: [0.0])
    cur_checkpoint: int = 0
    checkpoint_step: bool = False
    final_step: bool = False

    def timestep(self):
        """timestep (timestep.f90:1-92) for one image."""
        self.dt_old = self.dt
        self.istep += 1
        a = f32(self.a)
        dt_e = f32(1.0)  # dt_max
        ntry = 0
        while True:
            ntry += 1
            d1, d2 = expansion(a, dt_e, self.omega_m, self.omega_l)
            da = f32(d1 + d2)
            ra = f32(da / f32(a + da))
            if ra > f32(self.ra_max):
                dt_e = f32(dt_e * f32(f32(self.ra_max) / ra))
            else:
                break
            if ntry > 10:
                break
        dt = min(dt_e, self.dt_fine, self.dt_coarse, self.dt_pp, self.dt_vmax, f32(1000.0))
        d1, d2 = expansion(a, dt, self.omega_m, self.omega_l)
        da = f32(d1 + d2)
        self.checkpoint_step = False
        if self.cur_checkpoint < len(self.z_checkpoints):
            z_next = f32(self.z_checkpoints[self.cur_checkpoint])
            a_next = f32(f32(1.0) / f32(f32(1) + z_next))
            if da >= f32(a_next - a):
                self.checkpoint_step = True
                if self.cur_checkpoint == len(self.z_checkpoints) - 1:
                    self.final_step = True
                n = 0
                while abs(f32(f32(a + da) / a_next) - f32(1)) >= f32(1e-6) and n < 100:
                    dt = f32(dt * f32(f32(a_next - a) / da))
                    d1, d2 = expansion(a, dt, self.omega_m, self.omega_l)
                    da = f32(d1 + d2)
                    n += 1
        self.a_mid = f32(a + f32(da / f32(2)))
        self.tau = f32(self.tau + dt)
        self.t = f32(self.t + dt)
        self.a = f32(a + da)
        self.da = da
        self.dt = f32(dt)
        return self.dt, self.a_mid

    def constrain(self, pm_stats, pp_stats=None, ncell=4):
        """dt constraints from the device maxima (pm.f90:395-398, ext_pp_force.f90:141)."""
        am = f32(self.a_mid)
        f2f = f32(pm_stats["f2_max_fine"])
        f2c = f32(pm_stats["f2_max_coarse"])
        if f2f > 0:
            self.dt_fine = f32(np.sqrt(f32(f32(1.0) / f32(f32(np.sqrt(f2f)) * am * GG))))
        if f2c > 0:
            self.dt_coarse = f32(np.sqrt(f32(f32(ncell) / f32(f32(np.sqrt(f2c)) * am * GG))))
        vm = max(f32(v) for v in pm_stats["vmax"])
        if vm > 0:
            self.dt_vmax = f32(f32(f32(0.9) * f32(20)) / vm)
        self.vz_max = f32(pm_stats["vmax"][2])
        if pp_stats is not None and f32(pp_stats["f2_max_pp"]) > 0:
            self.dt_pp = f32(f32(1.0) * f32(np.sqrt(f32(1.0))) /
                             f32(f32(np.sqrt(f32(pp_stats["f2_max_pp"]))) * am * GG))


def fixed_schedule(z_init, z_final, nsteps, omega_m=0.3, omega_l=0.7, spacing="log"):
    """A fixed step schedule from z_init to z_final: nsteps equal steps in
    ln a ("log") or in a ("linear").  Each step's dt is the one whose Friedmann
    step (``expansion``) covers the step's da, found by bisection; a_mid is
    a + da/2 as in ``TimeState.timestep``.  Returns float32 arrays (dt,
    a_mid, a) with a the nsteps+1 scale factors."""
    a0, a1 = 1.0 / (1.0 + z_init), 1.0 / (1.0 + z_final)
    if spacing == "log":
        a = np.exp(np.linspace(np.log(a0), np.log(a1), nsteps + 1)).astype(np.float32)
    else:
        a = np.linspace(a0, a1, nsteps + 1).astype(np.float32)
    dts, amids = np.zeros(nsteps, f32), np.zeros(nsteps, f32)
    for i in range(nsteps):
        target = float(a[i + 1]) - float(a[i])
        lo, hi = 0.0, 1.0
        while sum(float(d) for d in expansion(a[i], hi, omega_m, omega_l)) < target:
            hi *= 2
        for _ in range(60):
            mid = 0.5 * (lo + hi)
            if sum(float(d) for d in expansion(a[i], mid, omega_m, omega_l)) < target:
                lo = mid
            else:
                hi = mid
        dt = f32(hi)
        d1, d2 = expansion(a[i], dt, omega_m, omega_l)
        dts[i] = dt
        amids[i] = f32(a[i] + f32(f32(d1 + d2) / f32(2)))
    return dts, amids, a


def neutrino_checkpoints(z_checkpoint, z_i, z_i_nu):
    """When the second species (neutrinos) switches on (initialize.f90:90-136).

    Returns (checkpoint redshifts, index of the switch-on checkpoint (1-based,
    0 when the species starts with the run), neutrino_flag at the start).
    z_i_nu above z_i is an error; equal means both species start together;
    otherwise z_i_nu becomes a checkpoint (inserted in decreasing order, or
    appended after the last one) and the species is switched on there
    (checkpoint.f90:85-91)."""
    zc = [float(z) for z in z_checkpoint]
    if z_i_nu > z_i:
        raise ValueError("z_i_nu > z_i: neutrinos cannot start before the initial conditions")
    if z_i_nu == z_i:
        return zc, 0, True
    for i, z in enumerate(zc):
        if z == z_i_nu:
            return zc, i + 1, False
    if zc[-1] > z_i_nu:
        return zc + [float(z_i_nu)], len(zc) + 1, False
    for i, z in enumerate(zc):
        if z < z_i_nu:
            return zc[:i] + [float(z_i_nu)] + zc[i:], i + 1, False
    return zc, 0, False
