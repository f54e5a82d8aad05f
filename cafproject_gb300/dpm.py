"""Differentiable PM over the C ABI (``cube_dpm_*``), with a thin
``torch.autograd.Function`` harness for checking gradients.

The simulation and its adjoint are CUDA kernels in ``libcube_gb300.so``; the
autograd functions only hand device pointers across the boundary.  Tensors
are float32 on the context's device: noise ``(npd**3,)`` in lattice order,
displacements from the lattice points and velocities ``(np, 3)`` (mesh
cells), densities ``(ng, ng, ng)`` indexed ``[z, y, x]``.
"""
import ctypes

import numpy as np

from . import cosmology as cm
from .cube import Cosmology, CubeError, load_library


class DpmParams(ctypes.Structure):
    """ctypes image of ``cube_dpm_params``."""

    _fields_ = [("ng", ctypes.c_int32), ("npd", ctypes.c_int32), ("max_steps", ctypes.c_int32),
                ("ckpt_every", ctypes.c_int32), ("z_init", ctypes.c_float)]


def _bind(L):
    if getattr(L, "_dpm_bound", False):
        return L
    P, F, I = ctypes.c_void_p, ctypes.c_float, ctypes.c_int
    L.cube_dpm_create.argtypes = [P, P, I, ctypes.POINTER(P)]
    L.cube_dpm_destroy.argtypes = [P]
    L.cube_dpm_last_error.argtypes = [P]
    L.cube_dpm_last_error.restype = ctypes.c_char_p
    L.cube_dpm_stream.argtypes = [P]
    L.cube_dpm_stream.restype = P
    L.cube_dpm_nparticles.argtypes = [P]
    L.cube_dpm_nparticles.restype = ctypes.c_int64
    L.cube_dpm_set_schedule.argtypes = [P, I, P, P]
    L.cube_dpm_noise.argtypes = [P, ctypes.c_uint32, P]
    L.cube_dpm_forward.argtypes = [P, P, P, P]
    L.cube_dpm_backward.argtypes = [P, P, P, P, P, P]
    L.cube_dpm_density.argtypes = [P, P, P]
    L.cube_dpm_density_adjoint.argtypes = [P, P, P, P]
    L.cube_dpm_tables.argtypes = [P, P, P]
    L.cube_dpm_info.argtypes = [P, P, P, P, P]
    L._dpm_bound = True
    return L


def schedule(z_init, z_final, nsteps, omega_m=0.3, omega_l=0.7):
    """Step coefficients for nsteps equal steps in a from z_init to z_final.

    Each step's dt is the one whose Friedmann step (timestep.f90:133-177,
    ``cosmology.expansion``) covers the step's da (found by bisection); the
    drift is dt_mid = (dt_old + dt)/2 (update_particle.f90:32, dt_old = 0 on
    the first step) and the kick a_mid*dt/(6 pi) (pm.f90:162).
    Returns (drift, kick, a) with a the nsteps+1 scale factors."""
    dts, amids, a = cm.fixed_schedule(z_init, z_final, nsteps, omega_m, omega_l, spacing="linear")
    drift, kick = np.zeros(nsteps, np.float32), np.zeros(nsteps, np.float32)
    dt_old = np.float32(0)
    for i in range(nsteps):
        drift[i] = np.float32((dt_old + dts[i]) / np.float32(2))
        kick[i] = np.float32(amids[i] * dts[i] * cm.GG)
        dt_old = dts[i]
    return drift, kick, a


class DiffPM:
    """One differentiable-PM context (cube_dpm) on one GPU."""

    def __init__(self, ng, npd, z_init, z_final, nsteps, ckpt_every=2, device=0, box=256.0, omega_m=0.3,
                 omega_l=0.7, h0=0.7, s8=0.8, n_s=0.96, omega_b=0.049):
        import torch

        self.torch = torch
        self.L = _bind(load_library())
        self.device = torch.device("cuda", device)
        self.ng, self.npd, self.nsteps = ng, npd, nsteps
        self.np = npd ** 3
        self._p = DpmParams(ng, npd, nsteps, ckpt_every, z_init)
        self._cs = Cosmology(box, omega_m, omega_l, h0, s8, n_s, omega_b, 1)
        h = ctypes.c_void_p()
        rc = self.L.cube_dpm_create(ctypes.byref(self._p), ctypes.byref(self._cs), device, ctypes.byref(h))
        self.h = h
        if rc:
            msg = self.L.cube_dpm_last_error(h).decode() if h.value else ""
            if h.value:
                self.L.cube_dpm_destroy(h)
            self.h = None
            raise CubeError(rc, msg)
        self.drift, self.kick, self.a = schedule(z_init, z_final, nsteps, omega_m, omega_l)
        self._check(self.L.cube_dpm_set_schedule(self.h, nsteps, self.drift.ctypes.data, self.kick.ctypes.data))
        self.forwards = 0

    def _check(self, rc):
        if rc:
            raise CubeError(rc, self.L.cube_dpm_last_error(self.h).decode())

    def close(self):
        if self.h is not None and self.h.value:
            self.L.cube_dpm_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _empty(self, *shape):
        return self.torch.empty(*shape, dtype=self.torch.float32, device=self.device)

    @staticmethod
    def _dev(t):
        assert t.is_cuda and t.dtype.is_floating_point and t.is_contiguous()
        return ctypes.c_void_p(t.data_ptr())

    def _sync(self):
        self.torch.cuda.synchronize(self.device)

    def info(self):
        m, vf, f, b = ctypes.c_float(), ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        self._check(self.L.cube_dpm_info(self.h, ctypes.byref(m), ctypes.byref(vf), ctypes.byref(f), ctypes.byref(b)))
        return {"mass": m.value, "vf": vf.value, "forward_ms": f.value, "backward_ms": b.value}

    def stream(self):
        return self.L.cube_dpm_stream(self.h)

    def noise(self, seed):
        out = self._empty(self.np)
        self._sync()
        self._check(self.L.cube_dpm_noise(self.h, seed, self._dev(out)))
        return out

    def forward(self, noise):
        x, v = self._empty(self.np, 3), self._empty(self.np, 3)
        noise = noise.contiguous().float()
        self._sync()
        self._check(self.L.cube_dpm_forward(self.h, self._dev(noise), self._dev(x), self._dev(v)))
        self.forwards += 1
        return x, v

    def backward(self, gx, gv, initial=False):
        gx, gv = gx.contiguous().float(), gv.contiguous().float()
        gn = self._empty(self.np)
        gx0 = self._empty(self.np, 3) if initial else None
        gv0 = self._empty(self.np, 3) if initial else None
        self._sync()
        self._check(self.L.cube_dpm_backward(self.h, self._dev(gx), self._dev(gv), self._dev(gn),
                                             self._dev(gx0) if initial else None,
                                             self._dev(gv0) if initial else None))
        return (gn, gx0, gv0) if initial else gn

    def density(self, x):
        rho = self._empty(self.ng, self.ng, self.ng)
        x = x.contiguous().float()
        self._sync()
        self._check(self.L.cube_dpm_density(self.h, self._dev(x), self._dev(rho)))
        return rho

    def density_adjoint(self, x, grho):
        gx = self._empty(self.np, 3)
        x, grho = x.contiguous().float(), grho.contiguous().float()
        self._sync()
        self._check(self.L.cube_dpm_density_adjoint(self.h, self._dev(x), self._dev(grho), self._dev(gx)))
        return gx

    def tables(self):
        nh = self.npd // 2 + 1
        filt = np.zeros((self.npd, self.npd, nh), np.float32)
        green = np.zeros((self.ng, self.ng, self.ng // 2 + 1), np.float32)
        self._check(self.L.cube_dpm_tables(self.h, filt.ctypes.data, green.ctypes.data))
        return filt, green


def autograd_functions():
    """The torch.autograd.Function pair over a DiffPM (checking harness):
    Simulate(noise, sim) -> (x, v) and Density(x, sim) -> rho."""
    import torch

    class Simulate(torch.autograd.Function):
        @staticmethod
        def forward(ctx, noise, sim):
            x, v = sim.forward(noise)
            ctx.sim, ctx.tag = sim, sim.forwards
            return x, v

        @staticmethod
        def backward(ctx, gx, gv):
            if ctx.sim.forwards != ctx.tag:
                raise RuntimeError("the checkpoints belong to a later forward pass")
            gx = torch.zeros_like(gv) if gx is None else gx
            gv = torch.zeros_like(gx) if gv is None else gv
            return ctx.sim.backward(gx, gv), None

    class Density(torch.autograd.Function):
        @staticmethod
        def forward(ctx, x, sim):
            ctx.sim = sim
            ctx.save_for_backward(x)
            return sim.density(x)

        @staticmethod
        def backward(ctx, grho):
            (x,) = ctx.saved_tensors
            return ctx.sim.density_adjoint(x, grho), None

    return Simulate, Density
