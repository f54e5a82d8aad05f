"""Batched ensemble over the C ABI (``cube_batch_*``).

Independent boxes -- each a single-tile CUBE image with its own particle
count, cosmology, seed and fixed step schedule -- advanced together.  In graph
mode one captured CUDA graph per step covers every box (the plain path's
kernels, every per-step decision on the device); serial mode runs the same
schedule through the plain entry points, one box after another.
"""
import ctypes

import numpy as np

from . import cosmology as cm
from .cube import Cosmology, CubeError, CubeGPU, force_tables, load_library
from .params import CubeParams, CubeParamsC

GRAPH, SERIAL = 0, 1


class BatchBox(ctypes.Structure):
    """ctypes image of ``cube_batch_box``."""

    _fields_ = [("params", CubeParamsC), ("cosmo", Cosmology), ("z_init", ctypes.c_float),
                ("seed", ctypes.c_uint32)]


class BatchStats(ctypes.Structure):
    """ctypes image of ``cube_batch_stats``."""

    _fields_ = [("sigma_vi_new", ctypes.c_float), ("f2_max_fine", ctypes.c_float),
                ("f2_max_coarse", ctypes.c_float), ("f2_max_pp", ctypes.c_float), ("vmax", ctypes.c_float * 3),
                ("flags", ctypes.c_int32), ("npairs", ctypes.c_int64), ("itest1", ctypes.c_int64),
                ("ndup", ctypes.c_int64), ("sum_r", ctypes.c_double)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_}
        d["vmax"] = list(self.vmax)
        return d


def _bind(L):
    if getattr(L, "_batch_bound", False):
        return L
    P, I = ctypes.c_void_p, ctypes.c_int
    L.cube_batch_create.argtypes = [P, I, P, P, I, I, ctypes.POINTER(P)]
    L.cube_batch_destroy.argtypes = [P]
    L.cube_batch_last_error.argtypes = [P]
    L.cube_batch_last_error.restype = ctypes.c_char_p
    L.cube_batch_set_schedule.argtypes = [P, I, P, P]
    L.cube_batch_autotune.argtypes = [P, P]
    L.cube_batch_step.argtypes = [P, I]
    L.cube_batch_history.argtypes = [P, I, P]
    L.cube_batch_ctx.argtypes = [P, I, ctypes.POINTER(P)]
    L.cube_batch_time.argtypes = [P, P, P, P]
    L.cube_batch_step_times.argtypes = [P, P]
    L._batch_bound = True
    return L


def box_params(npd, box=None, omega_m=0.3, s8=0.8, pp_on=True):
    """A single-tile box of npd^3 particles with a fine mesh of twice the
    particle grid (np_nc = 2: coarse nc = npd/2, fine 4 nc = 2 npd)."""
    assert npd % 2 == 0
    return CubeParams(nc=npd // 2, nnt=1, pp_on=pp_on, rsoft=0.1, box=float(box or 2.0 * npd), omega_m=omega_m,
                      omega_l=1.0 - omega_m, s8=s8, np_nc=2, np_max=npd ** 3)


def ensemble(nbox, base_seed=1, sizes=(32, 48, 64, 96, 128), seed=2024, pp_on=True):
    """The ensemble workload: per box a particle grid drawn uniformly from
    sizes, Omega_m ~ U[0.25, 0.35], sigma_8 ~ U[0.7, 0.9], seed base+box.
    Returns a list of (CubeParams, seed)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(nbox):
        npd = int(rng.choice(sizes))
        om = float(rng.uniform(0.25, 0.35))
        s8 = float(rng.uniform(0.7, 0.9))
        out.append((box_params(npd, omega_m=om, s8=s8, pp_on=pp_on), base_seed + i))
    return out


class Batch:
    """A cube_batch: boxes [(CubeParams, seed)], z_init, mode GRAPH or SERIAL."""

    def __init__(self, boxes, z_init, mode=GRAPH, device=0, omega_b=0.045):
        self.L = _bind(load_library())
        self.params = [p for p, _ in boxes]
        arr = (BatchBox * len(boxes))()
        for i, (p, seed) in enumerate(boxes):
            arr[i].params = p.to_c()
            arr[i].cosmo = Cosmology(box=p.box, omega_m=p.omega_m, omega_l=p.omega_l, h0=p.h0, s8=p.s8, n_s=p.n_s,
                                     omega_b=omega_b, np_nc=p.np_nc)
            arr[i].z_init = float(z_init)
            arr[i].seed = int(seed) & 0xFFFFFFFF
        fine, coarse = force_tables()
        h = ctypes.c_void_p()
        rc = self.L.cube_batch_create(arr, len(boxes), fine.ctypes.data, coarse.ctypes.data, device, mode,
                                      ctypes.byref(h))
        self.h, self.nbox, self.mode, self.z_init = h, len(boxes), mode, z_init
        if rc:
            msg = self.L.cube_batch_last_error(h).decode() if h.value else ""
            if h.value:
                self.L.cube_batch_destroy(h)
            self.h = None
            raise CubeError(rc, msg)
        self.nsteps = 0

    def _check(self, rc):
        if rc:
            raise CubeError(rc, self.L.cube_batch_last_error(self.h).decode())

    def close(self):
        if self.h is not None and self.h.value:
            self.L.cube_batch_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def set_schedule(self, z_final, nsteps, spacing="log"):
        """Each box's fixed schedule from z_init to z_final (its own cosmology)."""
        dt = np.zeros((self.nbox, nsteps), np.float32)
        am = np.zeros((self.nbox, nsteps), np.float32)
        for i, p in enumerate(self.params):
            dt[i], am[i], _ = cm.fixed_schedule(self.z_init, z_final, nsteps, p.omega_m, p.omega_l, spacing)
        self._check(self.L.cube_batch_set_schedule(self.h, nsteps, dt.ctypes.data, am.ctypes.data))
        self.nsteps, self.dt, self.a_mid = nsteps, dt, am
        return dt, am

    def autotune(self):
        """(nbox, 3) int32: PP start level, fine and coarse deposit brick shape per box."""
        ch = np.zeros((self.nbox, 3), np.int32)
        self._check(self.L.cube_batch_autotune(self.h, ch.ctypes.data))
        return ch

    def step(self, n=1):
        self._check(self.L.cube_batch_step(self.h, int(n)))

    def history(self, step):
        out = (BatchStats * self.nbox)()
        self._check(self.L.cube_batch_history(self.h, int(step), out))
        return [o.as_dict() for o in out]

    def time(self):
        ms, dev, n = ctypes.c_float(), ctypes.c_float(), ctypes.c_int64()
        self._check(self.L.cube_batch_time(self.h, ctypes.byref(ms), ctypes.byref(dev), ctypes.byref(n)))
        return {"wall_ms": ms.value, "device_ms": dev.value, "steps_done": n.value}

    def step_times(self):
        """Per step done: ms over all boxes (device time in graph mode)."""
        n = self.time()["steps_done"]
        ms = np.zeros(max(n, 1), np.float32)
        self._check(self.L.cube_batch_step_times(self.h, ms.ctypes.data))
        return ms[:n]

    def box(self, i):
        """The i-th box as a borrowed CubeGPU (download, power spectrum, ...)."""
        h = ctypes.c_void_p()
        self._check(self.L.cube_batch_ctx(self.h, int(i), ctypes.byref(h)))
        return CubeGPU.borrow(h, self.params[i])
