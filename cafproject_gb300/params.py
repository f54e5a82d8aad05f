"""Run-time mirror of CUBE's compile-time parameters.

The reference fixes its mesh, tile, buffer and compression sizes as Fortran
``parameter`` constants (CUBEnu/work/main/parameters.f90:8-123); one binary
serves one configuration.  Here they travel as the ``cube_params`` C struct
(include/cube_gpu.h) so one library serves every configuration.

Named workloads (their sizes, not their provenance):

* ``cdm64``   -- 64^3 particles, 200 Mpc/h, coarse 32^3, fine 128^3, 1 tile, PM only
* ``cdm512``  -- 512^3 particles, 600 Mpc/h, coarse 256^3, fine 1024^3 over 2^3
                 tiles, PP within +-1 fine cell, rsoft 0.1 fine cells
"""
import ctypes
from dataclasses import dataclass, field

import numpy as np


class CubeParamsC(ctypes.Structure):
    """ctypes image of ``cube_params`` (include/cube_gpu.h)."""

    _fields_ = [
        ("nc", ctypes.c_int32),
        ("nnt", ctypes.c_int32),
        ("ncell", ctypes.c_int32),
        ("ncb", ctypes.c_int32),
        ("izipx", ctypes.c_int32),
        ("izipv", ctypes.c_int32),
        ("nf_cutoff", ctypes.c_int32),
        ("pp_range", ctypes.c_int32),
        ("pp_on", ctypes.c_int32),
        ("with_pid", ctypes.c_int32),
        ("rsoft", ctypes.c_float),
        ("mass_p", ctypes.c_float),
        ("np_max", ctypes.c_int64),
        ("reserved", ctypes.c_int32 * 8),
    ]


@dataclass
class CubeParams:
    """Mesh, tiling and compression sizes (parameters.f90:8-65)."""

    nc: int = 32            # coarse cells per dim (nc)
    nnt: int = 1            # tiles per dim (nnt)
    ncell: int = 4          # fine cells per coarse cell per dim (ncell)
    ncb: int = 6            # buffer depth in coarse cells (ncb)
    izipx: int = 1          # bytes per stored position component
    izipv: int = 2          # bytes per stored velocity component
    nf_cutoff: int = 16     # fine force kernel extent
    pp_range: int = 1       # PP neighbourhood in fine cells
    pp_on: bool = False     # Extended_pp_force
    with_pid: bool = True   # -DPID
    rsoft: float = 0.1      # PP hard cut, fine cells
    mass_p: float = 8.0     # sim%mass_p_cdm
    np_max: int = 0         # device particle capacity (0: derive)
    # cosmology / box (used by the host driver and the input generator)
    box: float = 200.0
    omega_m: float = 0.3
    omega_l: float = 0.7
    h0: float = 0.7
    s8: float = 0.8
    n_s: float = 0.96
    np_nc: int = 2          # particles per coarse cell per dim

    @property
    def nt(self):
        return self.nc // self.nnt

    @property
    def nf(self):
        return self.nc * self.ncell

    @property
    def nft(self):
        return self.nt * self.ncell

    @property
    def nfb(self):
        return self.ncb * self.ncell

    @property
    def nfe(self):
        return self.nft + 2 * self.nfb

    @property
    def npglobal(self):
        return (self.nc * self.np_nc) ** 3

    @property
    def xdtype(self):
        return np.int8 if self.izipx == 1 else np.int16

    @property
    def vdtype(self):
        return np.int8 if self.izipv == 1 else np.int16

    def validate(self):
        assert self.nc % self.nnt == 0, "nc must be a multiple of nnt"
        assert self.nt >= 2 * self.ncb, "tiles must be at least twice the buffer depth"
        assert self.izipx in (1, 2) and self.izipv in (1, 2)
        assert self.ncell == 4, "the fine/coarse ratio is fixed at 4 (ext_pp_force.f90:91)"
        assert self.nf_cutoff < self.nfb, "fine kernel must fit inside the tile buffer"

    def capacity(self):
        if self.np_max:
            return int(self.np_max)
        # generous margin over the mean count; the reference sizes its image
        # array with image_buffer=1.5 over the buffered count (variables.f90:9)
        return int(self.npglobal * 1.25) + 4096

    def to_c(self):
        self.validate()
        c = CubeParamsC()
        c.nc, c.nnt, c.ncell, c.ncb = self.nc, self.nnt, self.ncell, self.ncb
        c.izipx, c.izipv = self.izipx, self.izipv
        c.nf_cutoff, c.pp_range = self.nf_cutoff, self.pp_range
        c.pp_on, c.with_pid = int(bool(self.pp_on)), int(bool(self.with_pid))
        c.rsoft, c.mass_p = float(self.rsoft), float(self.mass_p)
        c.np_max = self.capacity()
        return c


def cdm64():
    """64^3 particles, 200 Mpc/h, coarse 32^3, fine 128^3 in one tile, PM only."""
    return CubeParams(nc=32, nnt=1, pp_on=False, box=200.0)


def cdm512():
    """512^3 particles, 600 Mpc/h, fine 1024^3 over 2^3 tiles, PP +-1 cell, rsoft 0.1."""
    return CubeParams(nc=256, nnt=2, pp_on=True, rsoft=0.1, box=600.0)


def cdm256():
    """256^3 particles, 300 Mpc/h, coarse 128^3, fine 512^3 over 2^3 tiles, PP: the
    cdm512 workload at 1/8 the volume, for profiling captures of a few GB."""
    return CubeParams(nc=128, nnt=2, pp_on=True, rsoft=0.1, box=300.0)


def small(nc=24, nnt=2, pp_on=True, izipx=1, izipv=2):
    """A small multi-tile case for parity tests (nt = nc/nnt >= 12)."""
    return CubeParams(nc=nc, nnt=nnt, pp_on=pp_on, izipx=izipx, izipv=izipv, box=100.0 * nc / 32)


WORKLOADS = {"cdm64": cdm64, "cdm256": cdm256, "cdm512": cdm512}
