"""Host-side mirror of CUBE's per-step subroutine surface over the C ABI.

``CubeGPU`` exposes the reference's call surface -- ``update_x``,
``buffer_grid``, ``buffer_x``, ``ext_pp_force``, ``particle_mesh``,
``buffer_v`` (CUBEnu/work/main/main.f90:102-118) -- with the same argument
meaning, on a device-resident state.  It loads ``libcube_gb300.so`` built from
this tree and raises if the library or a GPU is missing: there is no CPU
fallback.  Errors come back as ``CubeError`` carrying the C status code (each
replaces one of the reference's ``stop`` statements).
"""
import ctypes
import os

import numpy as np

from .params import CubeParams

HERE = os.path.dirname(os.path.abspath(__file__))
LIBPATH = os.path.join(HERE, "_build", "libcube_gb300.so")

FIELD_RHO_F, FIELD_FORCE_F, FIELD_RHO_C, FIELD_FORCE_C, FIELD_KERN_F, FIELD_KERN_C = 1, 2, 3, 4, 5, 6
FIELD_FORCE_PP = 7

STATUS = {0: "CUBE_OK", 1: "CUBE_ERR_ARG", 2: "CUBE_ERR_CUDA", 3: "CUBE_ERR_TILE_OVERFLOW",
          4: "CUBE_ERR_IMAGE_OVERFLOW", 5: "CUBE_ERR_PP_OVERFLOW", 6: "CUBE_ERR_COUNT_MISMATCH",
          7: "CUBE_ERR_NONFINITE", 8: "CUBE_ERR_DISPLACEMENT", 9: "CUBE_ERR_NOMEM", 10: "CUBE_ERR_STATE"}

# every symbol include/cube_gpu.h declares
EXPORTS = ["cube_create", "cube_destroy", "cube_last_error", "cube_upload_state", "cube_download_state",
           "cube_upload_begin", "cube_download_begin", "cube_download_finish",
           "cube_set_sigma", "cube_get_sigma", "cube_update_x", "cube_buffer_grid", "cube_buffer_x",
           "cube_buffer_v", "cube_pp_force", "cube_particle_mesh", "cube_pp_particle_mesh", "cube_pm_fine_density", "cube_pm_coarse_density",
           "cube_pm_fine_forces", "cube_pm_fine_kick",
           "cube_pm_coarse_forces", "cube_pm_coarse_kick", "cube_get_field", "cube_set_field", "cube_nplocal",
           "cube_synchronize", "cube_timing", "cube_timing_read", "cube_phase_name", "cube_stream",
           "cube_codec_check", "cube_codec_check_static", "cube_arith_check", "cube_pk_nbin",
           "cube_power_spectrum", "cube_checkpoint_write", "cube_checkpoint_read", "cube_ic_zeldovich", "cube_ic_zeldovich_nu", "cube_create_linked", "cube_particle_mesh2", "cube_pm_fine_density2", "cube_pm_coarse_density2", "cube_set_option",
           "cube_dpm_create", "cube_dpm_destroy", "cube_dpm_last_error", "cube_dpm_stream", "cube_dpm_nparticles",
           "cube_dpm_set_schedule", "cube_dpm_noise", "cube_dpm_forward", "cube_dpm_backward", "cube_dpm_density",
           "cube_dpm_density_adjoint", "cube_dpm_tables", "cube_dpm_info",
           "cube_batch_create", "cube_batch_destroy", "cube_batch_last_error", "cube_batch_set_schedule",
           "cube_batch_autotune", "cube_batch_step", "cube_batch_history", "cube_batch_ctx", "cube_batch_time",
           "cube_batch_step_times"]
CODEC_STATIC_MAX = 16384
OPT_EXACT_KICKS = 1
OPT_PP_LEVEL = 2
OPT_RANK_WALK = 3
OPT_DEPOSIT_FINE = 4
OPT_DEPOSIT_COARSE = 5
OPT_FAIL_ALLOC = 6
OPT_PP_HEAVY = 7
OPT_PP_PARTS = 8
OPT_PP_FILTER = 9
NPHASE = 16


class CubeError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("%s: %s" % (STATUS.get(code, code), msg))
        self.code = code


class Cosmology(ctypes.Structure):
    """ctypes image of ``cube_cosmology``."""

    _fields_ = [("box", ctypes.c_float), ("omega_m", ctypes.c_float), ("omega_l", ctypes.c_float),
                ("h0", ctypes.c_float), ("s8", ctypes.c_float), ("n_s", ctypes.c_float), ("omega_b", ctypes.c_float),
                ("np_nc", ctypes.c_int32)]


class SimHeader(ctypes.Structure):
    """ctypes image of ``cube_sim_header``: the reference's sim_header
    (parameters.f90:136-160), 224 bytes."""

    _fields_ = ([(n, ctypes.c_int64) for n in (
        "nplocal", "npglobal", "nplocal_nu", "npglobal_nu", "izipx", "izipv", "izipx_nu", "izipv_nu", "image",
        "nn", "nnt", "nt", "ncell", "ncb", "timestep", "cur_checkpoint", "cur_halofind")] +
        [(n, ctypes.c_float) for n in (
            "a", "t", "tau", "dt_pp", "dt_fine", "dt_coarse", "dt_vmax", "dt_vmax_nu", "mass_p_cdm", "mass_p_nu",
            "box", "h0", "omega_m", "omega_l", "s8", "vsim2phys", "sigma_vres", "sigma_vi", "sigma_vi_nu", "z_i",
            "z_i_nu", "vz_max")])

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


class CubeStats(ctypes.Structure):
    """ctypes image of ``cube_stats`` (include/cube_gpu.h)."""

    _fields_ = [("nplocal", ctypes.c_int64), ("max_tile_np", ctypes.c_int64), ("nlost", ctypes.c_int64),
                ("ndup", ctypes.c_int64), ("sum_c", ctypes.c_double), ("sum_r", ctypes.c_double),
                ("sum_s", ctypes.c_double), ("sigma_vi_new", ctypes.c_float), ("nlayer", ctypes.c_int32),
                ("max_disp", ctypes.c_int32), ("rank_walked", ctypes.c_int32), ("f2_max_pp", ctypes.c_float),
                ("pp_dense_bricks", ctypes.c_int32), ("npairs", ctypes.c_int64), ("itest1", ctypes.c_int64),
                ("f2_max_fine", ctypes.c_float), ("f2_max_coarse", ctypes.c_float),
                ("vmax", ctypes.c_float * 3), ("pad2", ctypes.c_int32), ("testrhof", ctypes.c_double),
                ("testrhoc", ctypes.c_double), ("flags", ctypes.c_int32), ("pad3", ctypes.c_int32)]

    def as_dict(self):
        d = {}
        for name, _ in self._fields_:
            if name.startswith("pad"):
                continue
            v = getattr(self, name)
            d[name] = list(v) if name == "vmax" else v
        return d


_lib = None


def load_library(path=None):
    """Load the in-tree library; raise if it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    path = path or LIBPATH
    if not os.path.exists(path):
        raise RuntimeError("libcube_gb300.so is not built (%s); run __graft_entry__.build()" % path)
    L = ctypes.CDLL(path)
    P, I64, F = ctypes.c_void_p, ctypes.c_int64, ctypes.c_float
    L.cube_create.argtypes = [P, P, P, ctypes.c_int, ctypes.POINTER(ctypes.c_void_p)]
    L.cube_destroy.argtypes = [P]
    L.cube_last_error.argtypes = [P]
    L.cube_last_error.restype = ctypes.c_char_p
    L.cube_upload_state.argtypes = [P, I64, P, P, P, P, P]
    L.cube_download_state.argtypes = [P, ctypes.POINTER(I64), P, P, P, P, P]
    L.cube_upload_begin.argtypes = L.cube_upload_state.argtypes
    L.cube_download_begin.argtypes = [P, ctypes.POINTER(I64), P, P, P, P, P]
    L.cube_download_finish.argtypes = [P]
    L.cube_set_sigma.argtypes = [P, F, F]
    L.cube_get_sigma.argtypes = [P, ctypes.POINTER(F), ctypes.POINTER(F)]
    L.cube_update_x.argtypes = [P, F, F, F, P]
    for n in ("cube_buffer_grid", "cube_buffer_x", "cube_buffer_v", "cube_synchronize"):
        getattr(L, n).argtypes = [P]
    L.cube_pp_force.argtypes = [P, F, F, P]
    L.cube_particle_mesh.argtypes = [P, F, F, P]
    L.cube_pp_particle_mesh.argtypes = [P, F, F, P, P]
    L.cube_pm_fine_density.argtypes = [P, P]
    L.cube_pm_coarse_density.argtypes = [P, P]
    L.cube_pm_fine_forces.argtypes = [P, P]
    L.cube_pm_fine_kick.argtypes = [P, F, F]
    L.cube_pm_coarse_forces.argtypes = [P, P]
    L.cube_pm_coarse_kick.argtypes = [P, F, F, P]
    L.cube_get_field.argtypes = [P, ctypes.c_int, P]
    L.cube_set_field.argtypes = [P, ctypes.c_int, P]
    L.cube_nplocal.argtypes = [P]
    L.cube_nplocal.restype = I64
    L.cube_timing.argtypes = [P, ctypes.c_int]
    L.cube_timing_read.argtypes = [P, P, P, ctypes.c_int]
    L.cube_phase_name.argtypes = [ctypes.c_int]
    L.cube_phase_name.restype = ctypes.c_char_p
    L.cube_stream.argtypes = [P]
    L.cube_stream.restype = ctypes.c_void_p
    L.cube_codec_check.argtypes = [P, F, P, I64, P, P]
    L.cube_codec_check_static.argtypes = [P, F, P, I64, P, P]
    L.cube_arith_check.argtypes = [P, P]
    L.cube_pk_nbin.argtypes = [ctypes.c_int]
    L.cube_power_spectrum.argtypes = [P, ctypes.c_int, F, P, P, ctypes.c_int]
    L.cube_checkpoint_write.argtypes = [P, ctypes.c_char_p, F, ctypes.c_int, P]
    L.cube_checkpoint_read.argtypes = [P, ctypes.c_char_p, F, ctypes.c_int, P]
    L.cube_ic_zeldovich.argtypes = [P, P, F, ctypes.c_uint32, P, P]
    L.cube_ic_zeldovich_nu.argtypes = [P, P, F, ctypes.c_uint32, F, ctypes.c_uint32, P, P]
    L.cube_create_linked.argtypes = [P, P, P]
    L.cube_particle_mesh2.argtypes = [P, P, F, F, P, P]
    L.cube_pm_fine_density2.argtypes = [P, P, P]
    L.cube_pm_coarse_density2.argtypes = [P, P, P]
    L.cube_set_option.argtypes = [P, ctypes.c_int, I64]
    _lib = L
    return L


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def force_tables():
    d = os.path.join(HERE, "data")
    fine = np.fromfile(os.path.join(d, "fine_force_table.f32"), "<f4")
    coarse = np.fromfile(os.path.join(d, "coarse_force_table.f32"), "<f4")
    return np.ascontiguousarray(fine), np.ascontiguousarray(coarse)


class CubeGPU:
    """One image of CUBE's state resident on one GPU."""

    def __init__(self, params: CubeParams, device=0, owner=None):
        """owner: a CubeGPU whose meshes this context shares as a second
        particle species (cube_create_linked); close it before the owner."""
        self.p = params
        self.L = load_library()
        self._cp = params.to_c()
        h = ctypes.c_void_p()
        if owner is None:
            fine, coarse = force_tables()
            rc = self.L.cube_create(ctypes.byref(self._cp), _ptr(fine), _ptr(coarse), device, ctypes.byref(h))
        else:
            rc = self.L.cube_create_linked(ctypes.byref(self._cp), owner.h, ctypes.byref(h))
        self.owner = owner
        self.h = h
        if rc:
            msg = self.L.cube_last_error(h).decode() if h.value else ""
            if h.value:
                self.L.cube_destroy(h)
            self.h = None
            raise CubeError(rc, msg)

    @classmethod
    def borrow(cls, handle, params):
        """A view of a context owned elsewhere (a box of a cube_batch): the
        same methods, and close() leaves the context alone."""
        g = cls.__new__(cls)
        g.p, g.L, g._cp, g.owner, g.h, g._borrowed = params, load_library(), params.to_c(), None, handle, True
        return g

    def _check(self, rc):
        if rc:
            raise CubeError(rc, self.L.cube_last_error(self.h).decode())

    def close(self):
        if self.h is not None and self.h.value and not getattr(self, "_borrowed", False):
            self.L.cube_destroy(self.h)
        self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ---- state
    def upload(self, xp, vp, pid, rhoc, vfield):
        p = self.p
        xp = np.ascontiguousarray(xp, dtype=p.xdtype).reshape(-1, 3)
        vp = np.ascontiguousarray(vp, dtype=p.vdtype).reshape(-1, 3)
        pid = None if pid is None else np.ascontiguousarray(pid, dtype=np.int32)
        rhoc = np.ascontiguousarray(rhoc, dtype=np.int32).reshape(-1)
        vfield = np.ascontiguousarray(vfield, dtype=np.float32).reshape(-1, 3)
        self._check(self.L.cube_upload_state(self.h, xp.shape[0], _ptr(xp), _ptr(vp), _ptr(pid), _ptr(rhoc),
                                             _ptr(vfield)))

    def nplocal(self):
        return int(self.L.cube_nplocal(self.h))

    def download(self, out=None):
        """Disjoint state as host arrays; ``out`` may supply (pinned) arrays of
        at least the right size to receive it."""
        p = self.p
        n = self.nplocal()
        if out is not None:
            xp, vp, pid = out["xp"][:n], out["vp"][:n], out["pid"][:n]
            rhoc, vf = out["rhoc"], out["vfield"]
        else:
            xp = np.empty((n, 3), p.xdtype)
            vp = np.empty((n, 3), p.vdtype)
            pid = np.empty(n, np.int32)
            rhoc = np.empty(p.nc ** 3, np.int32)
            vf = np.empty((p.nc ** 3, 3), np.float32)
        nn = ctypes.c_int64()
        self._check(self.L.cube_download_state(self.h, ctypes.byref(nn), _ptr(xp), _ptr(vp), _ptr(pid), _ptr(rhoc),
                                               _ptr(vf)))
        return dict(xp=xp, vp=vp, pid=pid, rhoc=rhoc, vfield=vf)

    def upload_begin(self, xp, vp, pid, rhoc, vfield):
        """``upload`` with xp and vp copied in pieces beside the next
        update_x's first pass and pid beside the rest of it; the arrays must
        be contiguous, of the state's dtypes, and pinned for the overlap, and
        xp, vp and pid unchanged until that update_x returns."""
        for a in (xp, vp, pid, rhoc, vfield):
            assert a is None or a.flags.c_contiguous
        self._check(self.L.cube_upload_begin(self.h, xp.shape[0], _ptr(xp), _ptr(vp), _ptr(pid), _ptr(rhoc),
                                             _ptr(vfield)))

    def download_begin(self, out):
        """Start the download into the (pinned) arrays of ``out``: xp, pid,
        rhoc and vfield now, beside the rest of the step, vp behind the next
        coarse kick.  Call it after update_x and the buffer calls;
        ``download_finish`` waits."""
        n = self.nplocal()
        nn = ctypes.c_int64()
        self._pending = (n, out)
        self._check(self.L.cube_download_begin(self.h, ctypes.byref(nn), _ptr(out["xp"][:n]), _ptr(out["vp"][:n]),
                                               _ptr(out["pid"][:n]), _ptr(out["rhoc"]), _ptr(out["vfield"])))

    def download_finish(self):
        n, out = self._pending
        self._pending = None
        self._check(self.L.cube_download_finish(self.h))
        return dict(xp=out["xp"][:n], vp=out["vp"][:n], pid=out["pid"][:n], rhoc=out["rhoc"], vfield=out["vfield"])

    def set_sigma(self, sigma_vi, sigma_vi_new=None):
        sn = sigma_vi if sigma_vi_new is None else sigma_vi_new
        self._check(self.L.cube_set_sigma(self.h, float(sigma_vi), float(sn)))

    def get_sigma(self):
        a, b = ctypes.c_float(), ctypes.c_float()
        self._check(self.L.cube_get_sigma(self.h, ctypes.byref(a), ctypes.byref(b)))
        return np.float32(a.value), np.float32(b.value)

    # ---- the reference's per-step call surface
    def update_x(self, dt_old, dt, vz_max):
        st = CubeStats()
        self._check(self.L.cube_update_x(self.h, float(dt_old), float(dt), float(vz_max), ctypes.byref(st)))
        return st.as_dict()

    def buffer_grid(self):
        self._check(self.L.cube_buffer_grid(self.h))

    def buffer_x(self):
        self._check(self.L.cube_buffer_x(self.h))

    def buffer_v(self):
        self._check(self.L.cube_buffer_v(self.h))

    def ext_pp_force(self, a_mid, dt):
        st = CubeStats()
        self._check(self.L.cube_pp_force(self.h, float(a_mid), float(dt), ctypes.byref(st)))
        return st.as_dict()

    def particle_mesh2(self, nu, a_mid, dt):
        """particle_mesh of this species and the linked species nu together;
        returns (stats, stats of nu)."""
        st, sn = CubeStats(), CubeStats()
        self._check(self.L.cube_particle_mesh2(self.h, nu.h, float(a_mid), float(dt), ctypes.byref(st),
                                               ctypes.byref(sn)))
        return st.as_dict(), sn.as_dict()

    def pp_particle_mesh(self, a_mid, dt):
        """ext_pp_force then particle_mesh in one call, PP beside the PM
        force chain on a second stream; returns (pp stats, pm stats)."""
        sp, sm = CubeStats(), CubeStats()
        self._check(self.L.cube_pp_particle_mesh(self.h, float(a_mid), float(dt), ctypes.byref(sp), ctypes.byref(sm)))
        return sp.as_dict(), sm.as_dict()

    def particle_mesh(self, a_mid, dt):
        st = CubeStats()
        self._check(self.L.cube_particle_mesh(self.h, float(a_mid), float(dt), ctypes.byref(st)))
        return st.as_dict()

    # ---- stages (parity tests)
    def fine_density(self):
        st = CubeStats()
        self._check(self.L.cube_pm_fine_density(self.h, ctypes.byref(st)))
        return st.as_dict()

    def coarse_density(self):
        st = CubeStats()
        self._check(self.L.cube_pm_coarse_density(self.h, ctypes.byref(st)))
        return st.as_dict()

    def fine_density2(self, nu):
        """Fine density of this species and the linked species nu together."""
        st = CubeStats()
        self._check(self.L.cube_pm_fine_density2(self.h, nu.h, ctypes.byref(st)))
        return st.as_dict()

    def coarse_density2(self, nu):
        st = CubeStats()
        self._check(self.L.cube_pm_coarse_density2(self.h, nu.h, ctypes.byref(st)))
        return st.as_dict()

    def fine_forces(self):
        st = CubeStats()
        self._check(self.L.cube_pm_fine_forces(self.h, ctypes.byref(st)))
        return st.as_dict()

    def fine_kick(self, a_mid, dt):
        self._check(self.L.cube_pm_fine_kick(self.h, float(a_mid), float(dt)))

    def coarse_forces(self):
        st = CubeStats()
        self._check(self.L.cube_pm_coarse_forces(self.h, ctypes.byref(st)))
        return st.as_dict()

    def coarse_kick(self, a_mid, dt):
        st = CubeStats()
        self._check(self.L.cube_pm_coarse_kick(self.h, float(a_mid), float(dt), ctypes.byref(st)))
        return st.as_dict()

    def synchronize(self):
        self._check(self.L.cube_synchronize(self.h))

    def stream(self):
        """The cudaStream_t (as an int) every call of this context runs on."""
        return int(self.L.cube_stream(self.h) or 0)

    def set_option(self, option, value):
        self._check(self.L.cube_set_option(self.h, int(option), int(value)))

    def codec_check(self, sigma, v):
        """(direct FP64 codes, table codes) of the doubles v under sigma."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        a = np.empty(v.size, np.int32)
        b = np.empty(v.size, np.int32)
        self._check(self.L.cube_codec_check(self.h, float(sigma), _ptr(v), v.size, _ptr(a), _ptr(b)))
        return a, b

    def ic_zeldovich(self, z_init, seed, omega_b=0.045):
        """Zel'dovich initial conditions generated on the device into this
        context (cosmology and particle grid from the context's parameters);
        returns (sigma_vi, vmax[3])."""
        p = self.p
        cs = Cosmology(box=p.box, omega_m=p.omega_m, omega_l=p.omega_l, h0=p.h0, s8=p.s8, n_s=p.n_s,
                       omega_b=omega_b, np_nc=p.np_nc)
        sig = ctypes.c_float()
        vm = (ctypes.c_float * 3)()
        self._check(self.L.cube_ic_zeldovich(self.h, ctypes.byref(cs), float(z_init), int(seed) & 0xFFFFFFFF,
                                             ctypes.byref(sig), vm))
        return np.float32(sig.value), [float(v) for v in vm]

    def ic_zeldovich_nu(self, z_init, seed, m_nu_ev, thermal_seed, omega_b=0.045):
        """Neutrino initial conditions: the Zel'dovich state of seed's field
        plus Fermi-Dirac thermal velocities for m_nu_ev; returns (sigma_vi, vmax[3])."""
        p = self.p
        cs = Cosmology(box=p.box, omega_m=p.omega_m, omega_l=p.omega_l, h0=p.h0, s8=p.s8, n_s=p.n_s,
                       omega_b=omega_b, np_nc=p.np_nc)
        sig = ctypes.c_float()
        vm = (ctypes.c_float * 3)()
        self._check(self.L.cube_ic_zeldovich_nu(self.h, ctypes.byref(cs), float(z_init), int(seed) & 0xFFFFFFFF,
                                                float(m_nu_ev), int(thermal_seed) & 0xFFFFFFFF, ctypes.byref(sig),
                                                vm))
        return np.float32(sig.value), [float(v) for v in vm]

    def checkpoint_write(self, directory, z, image=1, **header):
        """checkpoint (checkpoint.f90): the reference's files for this image;
        header fields (a, t, tau, box, omega_m, ...) as keyword arguments."""
        h = SimHeader()
        for k, v in header.items():
            setattr(h, k, v)
        self._check(self.L.cube_checkpoint_write(self.h, os.fsencode(directory), float(z), int(image),
                                                 ctypes.byref(h)))

    def checkpoint_read(self, directory, z, image=1):
        """particle_initialization's restart read; returns the header dict."""
        h = SimHeader()
        self._check(self.L.cube_checkpoint_read(self.h, os.fsencode(directory), float(z), int(image),
                                                ctypes.byref(h)))
        return h.as_dict()

    def power_spectrum(self, ng, box, delta2=None):
        """xi(10, nbin) of cross_power (powerspectrum.f90) for the particles'
        CIC density on an ng^3 mesh, as an (nbin, 10) array; delta2 (ng^3,
        Fortran order) gives the cross power, None the auto power."""
        nbin = int(self.L.cube_pk_nbin(int(ng)))
        xi = np.zeros((nbin, 10), np.float64)
        d2 = None
        if delta2 is not None:
            d2 = np.ascontiguousarray(np.asarray(delta2, np.float32).reshape(ng, ng, ng))
        self._check(self.L.cube_power_spectrum(self.h, int(ng), float(box), _ptr(d2) if d2 is not None else None,
                                               _ptr(xi), nbin))
        return xi

    def arith_check(self):
        """Mismatches of the fast division by 6 and by pi_f against the IEEE
        division over every float (expected (0, 0))."""
        m = np.zeros(2, np.int64)
        self._check(self.L.cube_arith_check(self.h, _ptr(m)))
        return int(m[0]), int(m[1])

    def codec_check_static(self, sigma, v):
        """codec_check through the entry point whose device scratch is a fixed
        array (at most CODEC_STATIC_MAX values, no device allocation)."""
        v = np.ascontiguousarray(v, dtype=np.float64)
        a = np.empty(v.size, np.int32)
        b = np.empty(v.size, np.int32)
        self._check(self.L.cube_codec_check_static(self.h, float(sigma), _ptr(v), v.size, _ptr(a), _ptr(b)))
        return a, b

    def timing(self, enable):
        self._check(self.L.cube_timing(self.h, int(bool(enable))))

    def timing_read(self):
        """{phase: (total ms, launches)} accumulated since timing(True)."""
        ms = (ctypes.c_double * NPHASE)()
        cnt = (ctypes.c_int64 * NPHASE)()
        self._check(self.L.cube_timing_read(self.h, ms, cnt, NPHASE))
        return {self.L.cube_phase_name(i).decode(): (ms[i], int(cnt[i])) for i in range(NPHASE)}

    def _field_shape(self, which):
        nf, nc = self.p.nf, self.p.nc
        return {FIELD_RHO_F: (nf, nf, nf), FIELD_FORCE_F: (3, nf, nf, nf), FIELD_RHO_C: (nc, nc, nc),
                FIELD_FORCE_C: (3, nc, nc, nc), FIELD_KERN_F: (3, nf, nf, nf // 2 + 1),
                FIELD_KERN_C: (3, nc, nc, nc // 2 + 1), FIELD_FORCE_PP: (self.nplocal(), 3)}[which]

    def get_field(self, which):
        """Fields as numpy arrays indexed [.., z, y, x] (Fortran order of the reference)."""
        a = np.empty(self._field_shape(which), np.float32)
        self._check(self.L.cube_get_field(self.h, int(which), _ptr(a)))
        return a

    def set_field(self, which, arr):
        a = np.ascontiguousarray(arr, dtype=np.float32).reshape(self._field_shape(which))
        self._check(self.L.cube_set_field(self.h, int(which), _ptr(a)))
