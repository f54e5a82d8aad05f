"""CPU checks of the differentiable form's host logic and of its FP64 oracle."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")

from cafproject_gb300 import dpm  # noqa: E402
from oracle import dpm_oracle as orc  # noqa: E402


def test_schedule_covers_the_redshift_range():
    drift, kick, a = dpm.schedule(9.0, 0.0, 10)
    assert a[0] == np.float32(0.1) and a[-1] == np.float32(1.0)
    assert np.all(drift > 0) and np.all(kick > 0)
    # the first drift is dt/2 (dt_old = 0), later drifts average two steps;
    # each step's Friedmann expansion lands on the next scale factor
    from cafproject_gb300 import cosmology as cm
    dts = [2 * drift[0]]
    for i in range(1, 10):
        dts.append(2 * drift[i] - dts[-1])
    for i in range(10):
        da = sum(float(d) for d in cm.expansion(a[i], np.float32(dts[i]), 0.3, 0.7))
        assert abs(a[i] + da - a[i + 1]) < 2e-5


def _tables(ng, npd, seed=0):
    rng = np.random.default_rng(seed)
    k = np.sqrt(np.add.outer(np.add.outer(np.fft.fftfreq(npd) ** 2, np.fft.fftfreq(npd) ** 2),
                             np.fft.rfftfreq(npd) ** 2))
    filt = np.exp(-k * 6.0) * 0.3 / float(npd) ** 3  # real, even, smooth
    filt[0, 0, 0] = 0
    return filt, orc.green_table(ng)


def test_oracle_gradient_matches_its_finite_differences():
    ng, npd = 16, 8
    filt, green = _tables(ng, npd)
    drift, kick, _ = dpm.schedule(9.0, 0.0, 4)
    rng = np.random.default_rng(3)
    noise = torch.tensor(rng.standard_normal(npd ** 3), dtype=torch.float64, requires_grad=True)
    target = torch.tensor(1.0 + 0.1 * rng.standard_normal((ng, ng, ng)))
    L = orc.loss(noise, target, filt, green, ng, npd, 1.0, drift, kick)
    L.backward()
    g = noise.grad.numpy()
    eps = 1e-4
    for i in rng.choice(npd ** 3, 8, replace=False):
        e = torch.zeros(npd ** 3, dtype=torch.float64)
        e[i] = eps
        with torch.no_grad():
            lp = orc.loss(noise + e, target, filt, green, ng, npd, 1.0, drift, kick).item()
            lm = orc.loss(noise - e, target, filt, green, ng, npd, 1.0, drift, kick).item()
        fd = (lp - lm) / (2 * eps)
        assert abs(fd - g[i]) <= 1e-6 * max(1.0, abs(fd)), (i, fd, g[i])


def test_spectral_multiply_is_symmetric():
    # C2R o G o R2C is a symmetric operator for real, even G: the Green's
    # multiply is its own adjoint
    ng = 16
    g = orc.green_table(ng)
    rng = np.random.default_rng(1)
    u = torch.tensor(rng.standard_normal((ng, ng, ng)))
    w = torch.tensor(rng.standard_normal((ng, ng, ng)))
    mu = orc.potential(u, g, ng)
    mw = orc.potential(w, g, ng)
    a, b = float((mu * w).sum()), float((u * mw).sum())
    assert abs(a - b) <= 1e-12 * max(abs(a), 1.0)


def test_green_table_is_the_discrete_laplacian_inverse():
    ng = 16
    g = orc.green_table(ng) * float(ng) ** 3
    k = np.arange(ng)
    s = (2 * np.sin(np.pi * k / ng)) ** 2
    k2 = s[: ng // 2 + 1][None, None, :] + s[None, :, None] + s[:, None, None]
    assert np.allclose((g * k2)[k2 > 0], -4 * np.pi)


def test_fixed_log_schedule_and_ensemble():
    from cafproject_gb300 import batch as B
    from cafproject_gb300 import cosmology as cm
    dt, am, a = cm.fixed_schedule(19.0, 0.0, 50, 0.3, 0.7, "log")
    assert abs(a[0] - 0.05) < 1e-7 and abs(a[-1] - 1.0) < 1e-6
    r = a[1:] / a[:-1]
    assert np.allclose(r, r[0], rtol=1e-4)  # equal steps in ln a
    assert np.all((am > a[:-1]) & (am < a[1:]))
    ens = B.ensemble(256)
    sizes = sorted({p.nc * 2 for p, _ in ens})
    assert sizes == [32, 48, 64, 96, 128]
    assert all(0.25 <= p.omega_m <= 0.35 and 0.7 <= p.s8 <= 0.9 for p, _ in ens)
    assert all(p.nf == 4 * p.nc and p.nnt == 1 for p, _ in ens)  # fine mesh: twice the particle grid
    assert [s for _, s in ens] == list(range(1, 257))
