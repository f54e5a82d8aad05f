"""CPU restatement of the reference's initial-condition formulas -- TEST
INFRASTRUCTURE ONLY (the checker of the device's initial conditions; nothing
in cafproject_gb300 imports it).

Follows CUBEnu/work/utilities/initial_conditions.f90:
  * the sigma_8 normalisation: v8 = sum Delta^2(k) W_th(8k)^2 dk/k over the
    table up to kmax = 2 pi sqrt(3) nyquist / box, with the table's dk rule
    (dk(1) = k(2)/2, central differences, backward at the end), then
    Delta^2 *= s8^2/v8 * Dgrow(a)^2 (:209-225);
  * the top-hat window (tophat, :942-951) and the growth factor Dgrow
    (:953-966), both in default real (float32) as the reference declares them;
  * the Zel'dovich velocity factor vfactor = a^2 H (:994-1004; no neutrinos,
    so its exponent np is 1);
  * the Wiener scaling of the noise spectrum,
    sqrt(interp_tf(2 pi kr/box)/(4 pi) * (nf/kr)) * (nf/kr) with kr =
    max(|k|, 1) in grid units (:326-343) and interp_tf the log-log linear
    interpolation of the table (:917-939);
  * the discrete potential kernel -4 pi/khat^2, khat = 2 sin(pi k/nf), with
    max(khat^2, 1/nf^2) and a zero DC mode (:433-460), and its real-space
    correction (correct_kernel, :462-503): phi8 the mean of the kernel at the
    six points 8 cells from the origin along the axes, then -1/r inside 8
    cells, -2.5 at the origin, the kernel minus (phi8 + 1/8) beyond;
  * phi(k) = Re(corrected kernel(k)) * delta(k) (:505-507).
One stated substitution, the same as the device's: the CAMB transfer table
becomes the Eisenstein & Hu (1998) no-wiggle fit (their eqs. 26, 28-31)
sampled on 1000 log-spaced k from 1e-4 to 1e2 h/Mpc.

PARITY UNPINNED: the reference cannot run here; these are the formulas as
written in its source, evaluated in numpy.
"""
import numpy as np

f32 = np.float32


def eh_nowiggle(k, om, h, ob):
    """Eisenstein & Hu (1998) zero-baryon-oscillation transfer function; k in h/Mpc."""
    theta = 2.7255 / 2.7
    omh2, obh2, fb = om * h * h, ob * h * h, ob / om
    s = 44.5 * np.log(9.83 / omh2) / np.sqrt(1.0 + 10.0 * obh2 ** 0.75)
    alpha = 1.0 - 0.328 * np.log(431.0 * omh2) * fb + 0.38 * np.log(22.3 * omh2) * fb * fb
    gamma_eff = om * h * (alpha + (1.0 - alpha) / (1.0 + (0.43 * k * h * s) ** 4))
    q = k * theta * theta / gamma_eff
    L0 = np.log(2.0 * np.e + 1.8 * q)
    C0 = 14.2 + 731.0 / (1.0 + 62.5 * q)
    return L0 / (L0 + C0 * q * q)


def tophat(x):
    """tophat (initial_conditions.f90:942-951), default real."""
    x = f32(x)
    if x == 0:
        return f32(1.0)
    return f32(f32(3) * (np.sin(x) - np.cos(x) * x) / x ** 3)


def dgrow(a, om, ol):
    """Dgrow (initial_conditions.f90:953-966), default real arithmetic."""
    a, om, ol = f32(a), f32(om), f32(ol)
    hsq = om / a ** 3 + (f32(1) - om - ol) / a ** 2 + ol
    oma = om / (a ** 3 * hsq)
    ola = ol / hsq
    g = f32(2.5) * om / (om ** f32(4.0 / 7) - ol + (f32(1) + om / f32(2)) * (f32(1) + ol / f32(70)))
    ga = f32(2.5) * oma / (oma ** f32(4.0 / 7) - ola + (f32(1) + oma / f32(2)) * (f32(1) + ola / f32(70)))
    return f32(a * ga / g)


def vfactor(a, om, ol):
    """vfactor (initial_conditions.f90:994-1004) without neutrinos: a^2 H."""
    a, om, ol = f32(a), f32(om), f32(ol)
    lm = ol / om
    km = (f32(1) - om - ol) / om
    H = f32(2) / (f32(3) * np.sqrt(a ** 3)) * np.sqrt(f32(1) + a * km + a ** 3 * lm)
    return f32(a ** 2 * H)


def delta2_table(box, nf, a, om=0.3, ol=0.7, h=0.7, s8=0.8, n_s=0.96, ob=0.045, nk=1000):
    """(k, Delta^2(k) at a) of the sigma_8-normalised no-wiggle spectrum."""
    k = 10.0 ** (-4.0 + 6.0 * np.arange(nk) / (nk - 1))
    t = eh_nowiggle(k, om, h, ob)
    d2 = t * t * k ** (3 + n_s) / (2 * np.pi ** 2)
    dk = np.empty(nk)
    dk[0] = k[1] / 2
    dk[1:-1] = (k[2:] - k[:-2]) / 2
    dk[-1] = k[-1] - k[-2]
    kmax = 2 * np.pi * np.sqrt(3.0) * (nf // 2) / box
    v8 = 0.0
    for i in range(nk):
        if k[i] > kmax:
            break
        v8 += d2[i] * float(tophat(k[i] * 8)) ** 2 * dk[i] / k[i]
    g = float(dgrow(a, om, ol))
    return k, d2 * (s8 * s8 / v8) * g * g


def interp_tf(kr, k, d2):
    """interp_tf (initial_conditions.f90:917-939): log-log linear between the
    bracketing table points (clamped to the table's ends)."""
    lk, ld = np.log(k), np.log(d2)
    x = np.clip(np.log(kr), lk[0], lk[-1])
    i = np.clip(np.searchsorted(lk, x, side="right") - 1, 0, len(lk) - 2)
    t = (x - lk[i]) / (lk[i + 1] - lk[i])
    return np.exp(ld[i] + (ld[i + 1] - ld[i]) * t)


def _freq(n):
    return (np.arange(n) + n // 2) % n - n // 2


def corrected_kernel(nf):
    """Re of the corrected discrete potential kernel's spectrum, (nf, nf,
    nf//2+1) indexed [z, y, x] (initial_conditions.f90:433-507)."""
    ky = _freq(nf)
    kx = np.arange(nf // 2 + 1)
    sx = 2 * np.sin(np.pi * kx / nf)
    sy = 2 * np.sin(np.pi * ky / nf)
    ks = sx[None, None, :] ** 2 + sy[None, :, None] ** 2 + sy[:, None, None] ** 2
    ks = np.maximum(ks, 1.0 / nf ** 2)
    kern = -4 * np.pi / ks
    kern[0, 0, 0] = 0.0
    r3 = np.fft.irfftn(kern, s=(nf, nf, nf), axes=(0, 1, 2))  # normalised inverse (pencil_fft_backward divides by nf^3)
    phi8 = (r3[0, 0, 8] + r3[0, 8, 0] + r3[8, 0, 0] + r3[0, 0, nf - 8] + r3[0, nf - 8, 0] + r3[nf - 8, 0, 0]) / 6
    c = _freq(nf)
    rr = np.sqrt(c[:, None, None] ** 2 + c[None, :, None] ** 2 + c[None, None, :] ** 2)
    r3 = np.where(rr > 8, r3 - (phi8 + 1 / 8.0), np.where(rr > 0, -1.0 / np.where(rr > 0, rr, 1), -2.5))
    return np.fft.rfftn(r3).real


def filter_table(nf, box, a, **cosmo):
    """The real factor taking the noise spectrum to phi's spectrum on an nf^3
    grid, with the inverse transform's 1/nf^3 folded in, [z, y, x] half
    spectrum (the device's cube_ic_filter output)."""
    k, d2 = delta2_table(box, nf, a, **cosmo)
    kz = _freq(nf)
    kx = np.arange(nf // 2 + 1)
    kr = np.sqrt(kx[None, None, :] ** 2 + kz[None, :, None] ** 2 + kz[:, None, None] ** 2).astype(np.float64)
    kr = np.maximum(kr, 1.0)
    w = np.sqrt(interp_tf(2 * np.pi * kr / box, k, d2) / (4 * np.pi) * (nf / kr)) * (nf / kr)
    f = w * corrected_kernel(nf) / float(nf) ** 3
    f[0, 0, 0] = 0.0
    return f
