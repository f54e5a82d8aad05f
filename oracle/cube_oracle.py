"""Oracle driver: CPU restatement of CUBE's per-step path (TEST INFRASTRUCTURE).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg may
import this module, and only as the checker or the timed CPU reference.  The
product (``cafproject_gb300``) never calls it.

PARITY UNPINNED: the reference (Coarray Fortran + FFTW3f) cannot be built
where this oracle runs and ships no golden vectors for this path; the loops in
cube_oracle.c restate the reference statement by statement and are pinned by
analytic known-answer tests.  The FFTs here are scipy's pocketfft in single
precision, standing in for FFTW3f (sfftw_*, CUBEnu/work/main/cubefft.f90:24-25,
pencil_fft.f90:165-176); no reference test fixes FFT output bits, so forces are
compared with a tolerance.
"""
import ctypes
import os
import subprocess

import numpy as np
import scipy.fft as sfft

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libcube_oracle.so")
PI_F = np.float32(4.0) * np.arctan(np.float32(1.0))  # parameters.f90:67


def build(force=False):
    """Compile cube_oracle.c (gcc -O3, no FMA contraction, no fast-math, OpenMP)."""
    src = os.path.join(HERE, "cube_oracle.c")
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) >= os.path.getmtime(src):
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    tmp = LIB + ".tmp%d" % os.getpid()
    subprocess.check_call(["gcc", "-O3", "-ffp-contract=off", "-fno-fast-math", "-fopenmp", "-fPIC",
                           "-shared", "-o", tmp, src, "-lm"])
    os.replace(tmp, LIB)
    return LIB


class OrcParams(ctypes.Structure):
    _fields_ = [("nc", ctypes.c_int64), ("nnt", ctypes.c_int64), ("nt", ctypes.c_int64),
                ("ncell", ctypes.c_int64), ("ncb", ctypes.c_int64), ("izipx", ctypes.c_int64),
                ("izipv", ctypes.c_int64), ("nf_cutoff", ctypes.c_int64), ("pp_range", ctypes.c_int64),
                ("rsoft", ctypes.c_float), ("mass_p", ctypes.c_float), ("nthreads", ctypes.c_int32),
                ("tile_sel", ctypes.c_int32)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        _lib = ctypes.CDLL(build())
        P = ctypes.c_void_p
        _lib.orc_buffer_count.restype = ctypes.c_int64
        _lib.orc_buffer_count.argtypes = [P, P]
        _lib.orc_buffer.argtypes = [P] * 12
        _lib.orc_unbuffer.argtypes = [P] * 9
        _lib.orc_update_xp.restype = ctypes.c_int64
        _lib.orc_update_xp.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_float] + [P] * 13
        _lib.orc_sigma_sums.argtypes = [P, ctypes.c_float, P, P, P, P]
        _lib.orc_fine_deposit.argtypes = [P, ctypes.c_int64, P, P, P, P, P, P, P, P]
        _lib.orc_fine_kick.argtypes = [P, ctypes.c_int64, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                                       ctypes.c_float, P, P, P, P, P]
        _lib.orc_coarse_deposit.argtypes = [P, P, P, P, P, P, P, P, P]
        _lib.orc_coarse_kick.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_float] + [P] * 8
        _lib.orc_pp_force.argtypes = [P, ctypes.c_float, ctypes.c_float, ctypes.c_float] + [P] * 6
    return _lib


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def fine_table():
    """fk_table(i,j,k,d) as a (3,16,16,16) array indexed [d,k,j,i]."""
    path = os.path.join(HERE, "..", "cafproject_gb300", "data", "fine_force_table.f32")
    return np.fromfile(path, "<f4").reshape(3, 16, 16, 16)


def coarse_table():
    """ck_table(d,i,j,k) as a (4,4,4,3) array indexed [k,j,i,d]."""
    path = os.path.join(HERE, "..", "cafproject_gb300", "data", "coarse_force_table.f32")
    return np.fromfile(path, "<f4").reshape(4, 4, 4, 3)


# --------------------------------------------------------------- kernels


def kernel_f(n, nf_cutoff=16, pp_on=False, pp_range=1, table=None, dtype=np.float32):
    """Fine force kernel on an n^3 box (kernel_f.f90:25-37).

    Returns kern (3, n, n, n//2+1) indexed [d, kz, ky, kx] = Im FFT of the
    odd-mirrored table.  The reference builds it on the tile box n = nfe.
    """
    tab = fine_table() if table is None else table
    kern = np.zeros((3, n, n, n // 2 + 1), dtype=dtype)
    nfc = nf_cutoff
    for d in range(3):
        box = np.zeros((n, n, n), dtype=dtype)  # [k, j, i]
        box[:nfc, :nfc, :nfc] = tab[d]
        if pp_on:
            box[:pp_range + 1, :pp_range + 1, :pp_range + 1] = 0
        mf = [1, 1, 1]
        mf[d] = -1
        # rho_f(nfe-nf_cutoff+2:nfe,:,:)=mfactor(1)*rho_f(nf_cutoff:2:-1,:,:) etc.
        box[:, :, n - nfc + 1:] = mf[0] * box[:, :, nfc - 1:0:-1]
        box[:, n - nfc + 1:, :] = mf[1] * box[:, nfc - 1:0:-1, :]
        box[n - nfc + 1:, :, :] = mf[2] * box[nfc - 1:0:-1, :, :]
        kern[d] = np.imag(sfft.rfftn(box, workers=-1)).astype(dtype)
    return kern


def _coarse_raw(nc, ncell):
    """-r/r^3 on the periodic coarse grid, r in fine cells (kernel_c.f90:16-28)."""
    g = np.arange(1, nc + 1, dtype=np.int64)
    rx1 = (ncell * (np.mod(g + nc // 2 - 1, nc) - nc // 2)).astype(np.float32)
    rz, ry, rx = np.meshgrid(rx1, rx1, rx1, indexing="ij")
    r = np.sqrt(rx * rx + ry * ry + rz * rz).astype(np.float32)
    r3 = (r * r) * r
    ck = np.zeros((3, nc, nc, nc), dtype=np.float32)
    with np.errstate(divide="ignore", invalid="ignore"):
        for d, comp in enumerate((rx, ry, rz)):
            ck[d] = np.where(r == 0, np.float32(0), -comp / r3)
    return ck


def kernel_c(nc, ncell=4, table=None):
    """Coarse force kernel with the near-field table and LRCKCORR
    (kernel_c.f90:16-117, nn=1 so all eight octant copies apply).

    Returns kern (3, nc, nc, nc//2+1) indexed [d, kz, ky, kx]."""
    ct = coarse_table() if table is None else table  # [k, j, i, d]
    ck = _coarse_raw(nc, ncell)  # [d, k, j, i]
    T = np.transpose(ct, (3, 0, 1, 2))  # [d, k, j, i] with k,j,i in 0..3
    rev = slice(3, 0, -1)  # Fortran 4:2:-1
    hi = slice(nc - 3, nc)  # Fortran nc-2:nc
    lo = slice(0, 4)
    # 1
    ck[:, lo, lo, lo] = T
    # 5 x
    ck[0, lo, lo, hi] = -T[0][:, :, rev]
    ck[1:3, lo, lo, hi] = T[1:3][:, :, :, rev]
    # 3 y
    ck[0::2, lo, hi, lo] = T[0::2][:, :, rev, :]
    ck[1, lo, hi, lo] = -T[1][:, rev, :]
    # 2 z
    ck[0:2, hi, lo, lo] = T[0:2][:, rev, :, :]
    ck[2, hi, lo, lo] = -T[2][rev, :, :]
    # 4 yz
    ck[0, hi, hi, lo] = T[0][rev, rev, :]
    ck[1:3, hi, hi, lo] = -T[1:3][:, rev, rev, :]
    # 6 xz
    ck[0::2, hi, lo, hi] = -T[0::2][:, rev, :, rev]
    ck[1, hi, lo, hi] = T[1][rev, :, rev]
    # 7 xy
    ck[0:2, lo, hi, hi] = -T[0:2][:, :, rev, rev]
    ck[2, lo, hi, hi] = T[2][:, rev, rev]
    # 8 xyz
    ck[:, hi, hi, hi] = -T[:, rev, rev, rev]

    raw = _coarse_raw(nc, ncell)
    kern = np.zeros((3, nc, nc, nc // 2 + 1), dtype=np.float32)
    k1 = (np.mod(np.arange(1, nc + 1) + nc // 2 - 1, nc) - nc // 2).astype(np.float32)
    kxh = k1[: nc // 2 + 1].copy()
    kxh[nc // 2] = k1[nc // 2]  # ig = nc/2+1 maps to -nc/2
    kz, ky, kx = np.meshgrid(k1, k1, kxh, indexing="ij")
    kr = np.sqrt(kx * kx + ky * ky + kz * kz).astype(np.float32)
    s = [np.float32(2) * np.sin(PI_F * c / np.float32(nc)).astype(np.float32) for c in (kx, ky, kz)]
    ssum = ((s[0] * s[0] + s[1] * s[1]) + s[2] * s[2]).astype(np.float32)
    for d in range(3):
        kd = np.imag(sfft.rfftn(ck[d], workers=-1)).astype(np.float32)
        im_raw = np.imag(sfft.rfftn(raw[d], workers=-1)).astype(np.float32)
        comp = (kx, ky, kz)[d]
        with np.errstate(divide="ignore", invalid="ignore"):
            corr = ((((kd * np.float32(0.25)) * PI_F) * s[d]) / ssum) / im_raw
        keep = (kr > np.float32(8.0)) | (comp == 0)
        kern[d] = np.where(keep, kd, corr).astype(np.float32)
    return kern


# ------------------------------------------------------------------ image


class OracleImage:
    """One coarray image (nn=1) of the reference state, on the CPU."""

    def __init__(self, params, nthreads=1, fft_dtype=np.float32):
        self.p = params
        self.op = OrcParams(nc=params.nc, nnt=params.nnt, nt=params.nt, ncell=params.ncell, ncb=params.ncb,
                            izipx=params.izipx, izipv=params.izipv, nf_cutoff=params.nf_cutoff,
                            pp_range=params.pp_range, rsoft=params.rsoft, mass_p=params.mass_p,
                            nthreads=nthreads, tile_sel=-1)
        self.fft_dtype = fft_dtype
        self._kf = None
        self._kc = None
        self.sigma_vi = np.float32(0)
        self.sigma_vi_new = np.float32(0)
        self.last = {}

    # ---- state
    def load(self, xp, vp, pid, rhoc, vfield):
        p = self.p
        self.np = int(xp.shape[0])
        self.xp = np.ascontiguousarray(xp, dtype=p.xdtype).reshape(-1, 3)
        self.vp = np.ascontiguousarray(vp, dtype=p.vdtype).reshape(-1, 3)
        self.pid = np.ascontiguousarray(pid, dtype=np.int32) if pid is not None else np.zeros(self.np, np.int32)
        self.rhoc = np.ascontiguousarray(rhoc, dtype=np.int32).reshape(-1)
        self.vfield = np.ascontiguousarray(vfield, dtype=np.float32).reshape(-1, 3)
        self._buffer()

    def _buffer(self):
        p = self.p
        L = lib()
        nte = p.nt + 2 * p.ncb
        next_ = nte ** 3 * p.nnt ** 3
        nb = L.orc_buffer_count(ctypes.byref(self.op), _p(self.rhoc))
        self.brhoc = np.zeros(next_, np.int32)
        self.bvfield = np.zeros((next_, 3), np.float32)
        self.bstart = np.zeros(next_, np.int64)
        self.bxp = np.zeros((max(nb, 1), 3), p.xdtype)
        self.bvp = np.zeros((max(nb, 1), 3), p.vdtype)
        self.bpid = np.zeros(max(nb, 1), np.int32)
        L.orc_buffer(ctypes.byref(self.op), _p(self.xp), _p(self.vp), _p(self.pid), _p(self.rhoc),
                     _p(self.vfield), _p(self.brhoc), _p(self.bvfield), _p(self.bstart), _p(self.bxp),
                     _p(self.bvp), _p(self.bpid))

    def _unbuffer(self):
        L = lib()
        L.orc_unbuffer(ctypes.byref(self.op), _p(self.brhoc), _p(self.bstart), _p(self.bxp), _p(self.bvp),
                       _p(self.bpid), _p(self.xp), _p(self.vp), _p(self.pid))

    def buffer_v(self):
        """buffer_v (buffer_particle.f90:5-25; main.f90:118): refresh the buffer
        copies from the kicked physical particles.  PP and PM kick only the
        physical particles of each tile; the next update_x reads the buffer
        regions too."""
        self._unbuffer()
        self._buffer()

    def state(self):
        """Disjoint state (checkpoint layout) after the last call."""
        self._unbuffer()
        return dict(xp=self.xp.copy(), vp=self.vp.copy(), pid=self.pid.copy(), rhoc=self.rhoc.copy(),
                    vfield=self.vfield.copy())

    # ---- update_x
    def update_x(self, dt_old, dt, vz_max):
        """update_xp (update_particle.f90:16-256) followed by buffer_grid/x/v."""
        p = self.p
        L = lib()
        dt_mid = np.float32((np.float32(dt_old) + np.float32(dt)) / np.float32(2))
        cap = int(self.brhoc.sum()) + 16
        xo = np.zeros((cap, 3), p.xdtype)
        vo = np.zeros((cap, 3), p.vdtype)
        po = np.zeros(cap, np.int32)
        ro = np.zeros(p.nc ** 3, np.int32)
        fo = np.zeros((p.nc ** 3, 3), np.float32)
        mx = ctypes.c_int64(0)
        fl = ctypes.c_int32(0)
        n = L.orc_update_xp(ctypes.byref(self.op), float(dt_mid), float(np.float32(vz_max)),
                            float(self.sigma_vi), _p(self.brhoc), _p(self.bstart), _p(self.bvfield),
                            _p(self.bxp), _p(self.bvp), _p(self.bpid), _p(xo), _p(vo), _p(po), _p(ro), _p(fo),
                            ctypes.byref(mx), ctypes.byref(fl))
        self.np = int(n)
        self.xp, self.vp, self.pid = xo[:n].copy(), vo[:n].copy(), po[:n].copy()
        self.rhoc, self.vfield = ro, fo
        sums = np.zeros(3, np.float64)
        L.orc_sigma_sums(ctypes.byref(self.op), float(self.sigma_vi), _p(self.vp), _p(self.rhoc),
                         _p(self.vfield), _p(sums))
        npg = self.np
        std_vsim = np.sqrt(sums[2] / npg)
        std_c = np.sqrt(sums[0] / p.nc / p.nc / p.nc)
        std_res = np.sqrt(sums[1] / npg)
        # sigma_vi_new=std_vsim_res/sqrt(3.) (update_particle.f90:224)
        self.sigma_vi_new = np.float32(std_res / np.float64(np.sqrt(np.float32(3.0))))
        self._buffer()
        q = np.float32(np.float32(dt_mid * np.float32(vz_max)) / np.float32(p.ncell))
        self.last = dict(nplocal=self.np, max_tile_np=int(mx.value), flags=int(fl.value), sum_c=sums[0],
                         sum_r=sums[1], sum_s=sums[2], std_vsim=std_vsim, std_vsim_c=std_c,
                         std_vsim_res=std_res, sigma_vi_new=self.sigma_vi_new,
                         nlayer=2 * int(np.ceil(q)) + 1)
        return self.last

    def physical_slots(self):
        """Buffered index of every particle of the disjoint state, in storage
        order (the walk of orc_unbuffer: tile, cell x fastest, rank)."""
        p = self.p
        nt, ncb, nte = p.nt, p.ncb, p.nt + 2 * p.ncb
        t = np.arange(p.nnt ** 3)
        c = np.arange(nt)
        T, K, J, I = np.meshgrid(t, c, c, c, indexing="ij")
        e = ((I + ncb) + nte * ((J + ncb) + nte * ((K + ncb) + nte * T))).ravel()
        cnt = self.brhoc[e].astype(np.int64)
        first = np.repeat(self.bstart[e] - np.cumsum(cnt) + cnt, cnt)
        return first + np.arange(int(cnt.sum()))

    # ---- PP
    def pp_force(self, a_mid, dt, want_force=False):
        """ext_pp_force (ext_pp_force.f90:10-162), FP64 pair sums.  With
        want_force the result carries f_tot of every particle, (np, 3) float64
        in storage order, under "f_tot"."""
        out = np.zeros(3, np.float64)
        fb = np.zeros((self.bxp.shape[0], 3), np.float64) if want_force else None
        lib().orc_pp_force(ctypes.byref(self.op), float(np.float32(a_mid)), float(np.float32(dt)),
                           float(self.sigma_vi), _p(self.brhoc), _p(self.bstart), _p(self.bxp), _p(self.bvp),
                           _p(out), _p(fb))
        r = dict(f2_max_pp=np.float32(out[0]), npairs=int(out[1]), itest1=int(out[2]))
        if want_force:
            r["f_tot"] = fb[self.physical_slots()]
        return r

    # ---- PM
    def kern_f(self):
        if self._kf is None:
            p = self.p
            self._kf = kernel_f(p.nfe, p.nf_cutoff, p.pp_on, p.pp_range, dtype=self.fft_dtype)
        return self._kf

    def kern_c(self):
        if self._kc is None:
            self._kc = kernel_c(self.p.nc, self.p.ncell)
        return self._kc

    def fine_density(self, tile, nu=None):
        """Fine CIC density of one tile's nfe^3 box; nu (an OracleImage of
        the second species, same geometry) deposits each cell's neutrinos
        after its CDM particles into the same box (pm.f90:52-107)."""
        p = self.p
        rho = np.zeros((p.nfe, p.nfe, p.nfe), np.float32)  # [k, j, i]
        q = (ctypes.byref(nu.op), _p(nu.brhoc), _p(nu.bstart), _p(nu.bxp)) if nu is not None else (None,) * 4
        lib().orc_fine_deposit(ctypes.byref(self.op), tile, _p(self.brhoc), _p(self.bstart), _p(self.bxp),
                               _p(rho), *q)
        return rho

    def fine_force(self, rho):
        """force_f(d, nfb:nfe-nfb+1)^3 of one tile (pm.f90:112-126): returns
        (3, m, m, m) indexed [d, k, j, i] with m = nft+2."""
        p = self.p
        n, nfb = p.nfe, p.nfb
        kern = self.kern_f()
        dt = self.fft_dtype
        ck = sfft.rfftn(rho.astype(dt), workers=-1)
        out = np.zeros((3, p.nft + 2, p.nft + 2, p.nft + 2), np.float32)
        nn = dt(n)
        for d in range(3):
            prod = ck * (1j * kern[d])  # (re,im) -> (-im*K, re*K)
            f = sfft.irfftn(prod, s=(n, n, n), norm="forward", workers=-1).astype(dt)
            f = ((f / nn) / nn) / nn
            out[d] = f[nfb - 1:n - nfb + 1, nfb - 1:n - nfb + 1, nfb - 1:n - nfb + 1]
        return out

    def fine_kick(self, tile, force, a_mid, dt):
        fk = np.ascontiguousarray(np.transpose(force, (1, 2, 3, 0)))  # (m,m,m,3) -> Fortran (3,m,m,m)
        lib().orc_fine_kick(ctypes.byref(self.op), tile, float(np.float32(a_mid)), float(np.float32(dt)),
                            float(self.sigma_vi), float(self.sigma_vi_new), _p(self.brhoc), _p(self.bstart),
                            _p(self.bxp), _p(self.bvp), _p(fk))

    def tile_box(self, field_global, t):
        """Cut tile t's force box force_f(:,nfb:nfe-nfb+1)^3 out of a periodic
        global fine field (3,nf,nf,nf): box position q <-> global cell origin+q-1."""
        p = self.p
        m, nf, nft, nnt = p.nft + 2, p.nf, p.nft, p.nnt
        tx, ty, tz = t % nnt, (t // nnt) % nnt, t // (nnt * nnt)
        iz = (tz * nft - 1 + np.arange(m)) % nf
        iy = (ty * nft - 1 + np.arange(m)) % nf
        ix = (tx * nft - 1 + np.arange(m)) % nf
        return np.ascontiguousarray(field_global[:, iz][:, :, iy][:, :, :, ix])

    def fine_kick_global(self, field_global, a_mid, dt):
        """Fine kick of every tile reading a given periodic global force field."""
        for t in range(self.p.nnt ** 3):
            self.fine_kick(t, self.tile_box(field_global, t), a_mid, dt)

    def global_fine_force(self, nu=None):
        """Physical regions of every tile's force box assembled on the global
        periodic fine mesh (3,nf,nf,nf), plus the fine density; nu adds the
        second species' mass (fine_density)."""
        p = self.p
        nf, nft, nnt, nfb = p.nf, p.nft, p.nnt, p.nfb
        F = np.zeros((3, nf, nf, nf), np.float32)
        R = np.zeros((nf, nf, nf), np.float32)
        for t in range(nnt ** 3):
            tx, ty, tz = t % nnt, (t // nnt) % nnt, t // (nnt * nnt)
            rho = self.fine_density(t, nu)
            box = self.fine_force(rho)
            F[:, tz * nft:(tz + 1) * nft, ty * nft:(ty + 1) * nft, tx * nft:(tx + 1) * nft] = \
                box[:, 1:nft + 1, 1:nft + 1, 1:nft + 1]
            R[tz * nft:(tz + 1) * nft, ty * nft:(ty + 1) * nft, tx * nft:(tx + 1) * nft] = \
                rho[nfb:nfb + nft, nfb:nfb + nft, nfb:nfb + nft]
        return F, R

    def coarse_density(self, nu=None):
        """Coarse CIC density of the image; nu as in fine_density
        (pm.f90:205-267)."""
        p = self.p
        r3 = np.zeros((p.nc, p.nc, p.nc), np.float32)
        q = (ctypes.byref(nu.op), _p(nu.brhoc), _p(nu.bstart), _p(nu.bxp)) if nu is not None else (None,) * 4
        lib().orc_coarse_deposit(ctypes.byref(self.op), _p(self.brhoc), _p(self.bstart), _p(self.bxp), _p(r3), *q)
        return r3

    def coarse_force(self, r3):
        """force_c(d,1:nc)^3 (pm.f90:275-287): (3,nc,nc,nc) indexed [d,k,j,i]."""
        nc = self.p.nc
        kern = self.kern_c()
        ck = sfft.rfftn(r3.astype(np.float32), workers=-1)
        out = np.zeros((3, nc, nc, nc), np.float32)
        for d in range(3):
            f = sfft.irfftn(ck * (1j * kern[d]), s=(nc, nc, nc), norm="forward", workers=-1).astype(np.float32)
            out[d] = ((f / np.float32(nc)) / np.float32(nc)) / np.float32(nc)
        return out

    def coarse_kick(self, force_c, a_mid, dt, signed=False):
        """Coarse kick; returns vmax(3) = max|v + vfield| per component, and
        with signed=True also the neutrino loop's signed statistic
        max(maxval(v + vfield)) (pm.f90:349, 377)."""
        fc = np.ascontiguousarray(np.transpose(force_c, (1, 2, 3, 0)))
        vmax = np.zeros(3, np.float32)
        vs = np.zeros(1, np.float64)
        lib().orc_coarse_kick(ctypes.byref(self.op), float(np.float32(a_mid)), float(np.float32(dt)),
                              float(self.sigma_vi), _p(self.brhoc), _p(self.bstart), _p(self.bvfield),
                              _p(self.bxp), _p(self.bvp), _p(fc), _p(vmax), _p(vs))
        return (vmax, float(vs[0])) if signed else vmax

    def particle_mesh(self, a_mid, dt, keep_fields=False):
        """particle_mesh (pm.f90:2-415) without the dt bookkeeping."""
        p = self.p
        f2f = np.float32(0)
        testrhof = 0.0
        fields = {}
        nfb, nft = p.nfb, p.nft
        for t in range(p.nnt ** 3):
            rho = self.fine_density(t)
            testrhof += float(np.sum(rho[nfb:nft + nfb, nfb:nft + nfb, nfb:nft + nfb], dtype=np.float64))
            force = self.fine_force(rho)
            f2 = ((force[0] * force[0] + force[1] * force[1]) + force[2] * force[2]).max()
            f2f = max(f2f, np.float32(f2))
            if keep_fields:
                fields[("rho_f", t)] = rho
                fields[("force_f", t)] = force
            self.fine_kick(t, force, a_mid, dt)
        self.sigma_vi = self.sigma_vi_new  # pm.f90:193
        r3 = self.coarse_density()
        testrhoc = float(np.sum(r3, dtype=np.float64))
        fc = self.coarse_force(r3)
        f2c = np.float32(((fc[0] * fc[0] + fc[1] * fc[1]) + fc[2] * fc[2]).max())
        vmax = self.coarse_kick(fc, a_mid, dt)
        if keep_fields:
            fields["rho_c"] = r3
            fields["force_c"] = fc
        self.fields = fields
        self.buffer_v()
        return dict(f2_max_fine=f2f, f2_max_coarse=f2c, vmax=vmax, testrhof=testrhof, testrhoc=testrhoc)

    def particle_mesh2(self, nu, a_mid, dt, keep_fields=False):
        """particle_mesh (pm.f90:2-415) with CUBEnu's second species: nu (an
        OracleImage with its own izipx/izipv, mass and sigma) deposits into the
        same fine and coarse meshes, both species are kicked by the same
        forces with their own codes.  Returns (stats, nu stats); the nu
        stats carry vmax per component and the reference's signed
        vmax_nu (pm.f90:377)."""
        p = self.p
        f2f = np.float32(0)
        testrhof = 0.0
        fields = {}
        nfb, nft = p.nfb, p.nft
        for t in range(p.nnt ** 3):
            rho = self.fine_density(t, nu)
            testrhof += float(np.sum(rho[nfb:nft + nfb, nfb:nft + nfb, nfb:nft + nfb], dtype=np.float64))
            force = self.fine_force(rho)
            f2 = ((force[0] * force[0] + force[1] * force[1]) + force[2] * force[2]).max()
            f2f = max(f2f, np.float32(f2))
            if keep_fields:
                fields[("rho_f", t)] = rho
                fields[("force_f", t)] = force
            self.fine_kick(t, force, a_mid, dt)
            nu.fine_kick(t, force, a_mid, dt)
        self.sigma_vi = self.sigma_vi_new  # pm.f90:193-194
        nu.sigma_vi = nu.sigma_vi_new
        r3 = self.coarse_density(nu)
        testrhoc = float(np.sum(r3, dtype=np.float64))
        fc = self.coarse_force(r3)
        f2c = np.float32(((fc[0] * fc[0] + fc[1] * fc[1]) + fc[2] * fc[2]).max())
        vmax = self.coarse_kick(fc, a_mid, dt)
        vmax_nu, vsigned = nu.coarse_kick(fc, a_mid, dt, signed=True)
        if keep_fields:
            fields["rho_c"] = r3
            fields["force_c"] = fc
        self.fields = fields
        self.buffer_v()
        nu.buffer_v()
        return (dict(f2_max_fine=f2f, f2_max_coarse=f2c, vmax=vmax, testrhof=testrhof, testrhoc=testrhoc),
                dict(vmax=vmax_nu, vmax_signed=vsigned))


def time_sample(params, state, sigma, a_mid, dt, dt_old, vz_max, tile=0, nthreads=0):
    """Time the reference's step on one tile of the given state (CPU baseline).

    The reference processes tiles one after another, each with all OpenMP
    threads (update_particle.f90:40-150, ext_pp_force.f90:36-136,
    pm.f90:45-192); the image-wide parts (buffering, coarse PM) run once.  The
    step time is therefore estimated as nnt^3 x (one tile of update_xp + PP +
    fine PM) + buffering + coarse PM, each timed here on the host cores.
    Kernel construction (initialisation in the reference) is not timed.
    """
    import time

    img = OracleImage(params, nthreads=nthreads)
    img.kern_f()
    img.kern_c()
    t0 = time.perf_counter()
    img.load(state["xp"], state["vp"], state["pid"], state["rhoc"], state["vfield"])
    t_buf = time.perf_counter() - t0
    img.sigma_vi = img.sigma_vi_new = np.float32(sigma)
    L = lib()
    img.op.tile_sel = tile
    # update_xp of one tile (outputs discarded)
    p = params
    dt_mid = np.float32((np.float32(dt_old) + np.float32(dt)) / np.float32(2))
    cap = int(img.brhoc.sum()) + 16
    xo = np.zeros((cap, 3), p.xdtype)
    vo = np.zeros((cap, 3), p.vdtype)
    po = np.zeros(cap, np.int32)
    ro = np.zeros(p.nc ** 3, np.int32)
    fo = np.zeros((p.nc ** 3, 3), np.float32)
    mx, fl = ctypes.c_int64(0), ctypes.c_int32(0)
    t0 = time.perf_counter()
    L.orc_update_xp(ctypes.byref(img.op), float(dt_mid), float(np.float32(vz_max)), float(img.sigma_vi),
                    _p(img.brhoc), _p(img.bstart), _p(img.bvfield), _p(img.bxp), _p(img.bvp), _p(img.bpid),
                    _p(xo), _p(vo), _p(po), _p(ro), _p(fo), ctypes.byref(mx), ctypes.byref(fl))
    t_upd = time.perf_counter() - t0
    del xo, vo, po
    t0 = time.perf_counter()
    if p.pp_on:
        img.pp_force(a_mid, dt)
    t_pp = time.perf_counter() - t0
    t0 = time.perf_counter()
    rho = img.fine_density(tile)
    force = img.fine_force(rho)
    img.fine_kick(tile, force, a_mid, dt)
    t_fine = time.perf_counter() - t0
    del rho, force
    img.op.tile_sel = -1
    t0 = time.perf_counter()
    r3 = img.coarse_density()
    fc = img.coarse_force(r3)
    img.coarse_kick(fc, a_mid, dt)
    t_coarse = time.perf_counter() - t0
    nt3 = p.nnt ** 3
    est = nt3 * (t_upd + t_pp + t_fine) + t_buf + t_coarse
    return dict(t_update_tile=t_upd, t_pp_tile=t_pp, t_fine_tile=t_fine, t_buffer=t_buf, t_coarse=t_coarse,
                step_estimate=est, sampled=t_upd + t_pp + t_fine + t_buf + t_coarse)


def particle_cells(params, rhoc):
    """Global coarse-cell coordinates (x, y, z) of every particle in storage
    order: tile (x fastest), cell inside the tile (x fastest), rank
    (update_particle.f90:132-142)."""
    nt, nnt = params.nt, params.nnt
    t = np.arange(nnt)
    c = np.arange(nt)
    # index order of rhoc(nt,nt,nt,nnt,nnt,nnt): i, j, k, itx, ity, itz (i fastest)
    tz, ty, tx, k, j, i = np.meshgrid(t, t, t, c, c, c, indexing="ij")
    gx = (tx * nt + i).ravel()
    gy = (ty * nt + j).ravel()
    gz = (tz * nt + k).ravel()
    cnt = np.asarray(rhoc).ravel().astype(np.int64)
    return np.stack([np.repeat(gx, cnt), np.repeat(gy, cnt), np.repeat(gz, cnt)], axis=1)


def cic_density(params, xp, rhoc, ng):
    """Density contrast of mass-1 particles deposited by CIC at
    (cell + frac)*ng/nc - 0.5 in real(4) (cicpower.f90:100-133, 171-176);
    an (ng, ng, ng) float32 array indexed [z, y, x], summed in float64."""
    nc = params.nc
    xres = np.float32(1.0 / 256.0) if params.izipx == 1 else np.float32(1.0 / 65536.0)
    mask = (1 << (8 * params.izipx)) - 1
    gc = particle_cells(params, rhoc)
    frac = ((np.asarray(xp).reshape(-1, 3).astype(np.int64) & mask).astype(np.float32) + np.float32(0.5)) * xres
    pos = gc.astype(np.float32) + frac
    pos = (pos * np.float32(ng)) / np.float32(nc) - np.float32(0.5)
    fl = np.floor(pos)
    d1 = (fl + np.float32(1.0)) - pos
    d2 = np.float32(1.0) - d1
    i1 = fl.astype(np.int64) % ng
    i2 = (i1 + 1) % ng
    rho = np.zeros((ng, ng, ng), np.float64)  # [z, y, x]
    for oz in (0, 1):
        for oy in (0, 1):
            for ox in (0, 1):
                w = ((d2[:, 0] if ox else d1[:, 0]) * (d2[:, 1] if oy else d1[:, 1])) * (d2[:, 2] if oz else d1[:, 2])
                np.add.at(rho, ((i2 if oz else i1)[:, 2], (i2 if oy else i1)[:, 1], (i2 if ox else i1)[:, 0]),
                          w.astype(np.float64))
    mean = rho.sum() / float(ng) ** 3
    return (rho / mean - 1.0).astype(np.float32)


def binned_power(delta1, delta2, ng, box):
    """cross_power of powerspectrum.f90:21-135 for two density contrasts
    ([z, y, x] arrays; delta2 None for the auto power): forward FFT / ng^3,
    linear bins nint(|k|) with the reference's skipped modes, 1/sinc^4 and
    4 pi k^3 weights; returns xi as an (nbin, 10) array (float64 sums)."""
    c1 = np.fft.rfftn(np.asarray(delta1, np.float64).reshape(ng, ng, ng)) / float(ng) ** 3
    if delta2 is None:
        c2 = c1
    else:
        c2 = np.fft.rfftn(np.asarray(delta2, np.float64).reshape(ng, ng, ng)) / float(ng) ** 3
    nyq = ng // 2
    kk = (np.arange(ng) + nyq) % ng - nyq
    kz, ky, kx = np.meshgrid(kk, kk, kk[: nyq + 1], indexing="ij")
    k_i, j_i, i_i = np.meshgrid(np.arange(ng), np.arange(ng), np.arange(nyq + 1), indexing="ij")
    keep = ~((i_i == 0) & (j_i == 0) & (k_i == 0))
    edge = (i_i == 0) | (i_i == nyq)
    keep &= ~(edge & (j_i > nyq))
    keep &= ~(edge & ((j_i == 0) | (j_i == nyq)) & (k_i > nyq))
    kr = np.sqrt((kx * kx + ky * ky + kz * kz).astype(np.float32))

    def sinc(q):
        a = PI_F * q.astype(np.float32) / np.float32(ng)
        with np.errstate(invalid="ignore", divide="ignore"):
            return np.where(q == 0, np.float32(1.0), np.sin(a) / a).astype(np.float32)

    s = sinc(kx) * sinc(ky) * sinc(kz)
    ibin = np.floor(kr.astype(np.float64) + 0.5).astype(np.int64)  # nint, kr >= 0
    nbin = int(np.floor(np.float32(nyq) * np.sqrt(np.float32(3.0)) + np.float32(0.5)))
    w = 4.0 * np.pi * kr.astype(np.float64) ** 3 / s.astype(np.float64) ** 4
    q = [np.ones_like(kr, np.float64), kr.astype(np.float64), (np.abs(c1) ** 2) * w, (np.abs(c2) ** 2) * w,
         (c1 * np.conj(c2)).real * w, 1.0 / s.astype(np.float64) ** 2, 1.0 / s.astype(np.float64) ** 4]
    b = ibin[keep]
    sums = np.stack([np.bincount(b, weights=v[keep], minlength=nbin + 1)[1: nbin + 1] for v in q], axis=1)
    xi = np.zeros((nbin, 10))
    with np.errstate(invalid="ignore", divide="ignore"):
        xi[:, 0] = sums[:, 0]
        xi[:, 1] = sums[:, 1] / sums[:, 0] * (2 * float(PI_F)) / box
        for t in range(2, 7):
            xi[:, t] = sums[:, t] / sums[:, 0]
        xi[:, 7] = xi[:, 4] / np.sqrt(xi[:, 2] * xi[:, 3])
        xi[:, 8] = np.sqrt(xi[:, 3] / xi[:, 2])
        xi[:, 9] = xi[:, 7] ** 4 / xi[:, 8] ** 2 * xi[:, 3]
    return xi


def power_spectrum(params, xp, rhoc, ng, box, delta2=None):
    """cicpower.f90 + powerspectrum.f90: xi of the particles' CIC density
    (crossed with delta2 when given)."""
    return binned_power(cic_density(params, xp, rhoc, ng), delta2, ng, box)
