"""The differentiable PM form on the GPU against its FP64 oracle.

Forward state within FP32 rounding of the FP64 map; the loss gradient with
respect to the white noise within 1e-3 (relative L2) of the FP64 autograd
gradient and of FP64 central finite differences (eps = 1e-3) on 64 random
noise points; gradients independent of the checkpoint interval."""
import numpy as np
import pytest

torch = pytest.importorskip("torch")
pytestmark = pytest.mark.gpu

from oracle import dpm_oracle as orc  # noqa: E402

NG, NPD, NSTEPS = 32, 16, 10
BOX = 32.0  # 2 Mpc/h per particle, the spacing of 128^3 particles in 256 Mpc/h


def make(ckpt=2, ng=NG, npd=NPD, box=BOX):
    from cafproject_gb300.dpm import DiffPM
    return DiffPM(ng, npd, 9.0, 0.0, NSTEPS, ckpt_every=ckpt, box=box)


@pytest.fixture(scope="module")
def sim():
    s = make()
    yield s
    s.close()


def oracle_inputs(sim):
    filt, green = sim.tables()
    return filt.astype(np.float64), green.astype(np.float64), sim.info()["vf"]


def gpu_grad(sim, noise, target):
    Simulate, Density = __import__("cafproject_gb300.dpm", fromlist=["x"]).autograd_functions()
    n = noise.clone().requires_grad_(True)
    x, _ = Simulate.apply(n, sim)
    rho = Density.apply(x, sim)
    L = ((rho - target) ** 2).sum()
    L.backward()
    return n.grad.detach(), float(L)


def test_green_table(sim):
    _, green = sim.tables()
    ref = orc.green_table(NG)
    assert np.allclose(green, ref, rtol=1e-5, atol=0)


def test_forward_matches_fp64(sim):
    filt, green, vf = oracle_inputs(sim)
    noise = sim.noise(11)
    x, v = sim.forward(noise)
    with torch.no_grad():
        xo, vo = orc.simulate(noise.double().cpu(), filt, green, NG, NPD, vf, sim.drift, sim.kick)
    dx = x.double().cpu().numpy() - xo.numpy()
    disp = xo.numpy()
    ex = np.linalg.norm(dx) / np.linalg.norm(disp)
    ev = np.linalg.norm(v.double().cpu().numpy() - vo.numpy()) / np.linalg.norm(vo.numpy())
    print("forward rel err: displacement %.3g velocity %.3g" % (ex, ev))
    assert ex < 1e-4 and ev < 1e-4
    assert np.abs(disp).max() > 0.05  # the particles moved


@pytest.fixture(scope="module")
def problem(sim):
    target = sim.density(sim.forward(sim.noise(2))[0]).detach()
    noise = sim.noise(1)
    g, L = gpu_grad(sim, noise, target)
    return noise, target, g, L


def test_gradient_matches_fp64_autograd(sim, problem):
    noise, target, g, L = problem
    filt, green, vf = oracle_inputs(sim)
    n64 = noise.double().cpu().requires_grad_(True)
    Lo = orc.loss(n64, target.double().cpu(), filt, green, NG, NPD, vf, sim.drift, sim.kick)
    Lo.backward()
    go = n64.grad.numpy()
    err = np.linalg.norm(g.double().cpu().numpy() - go) / np.linalg.norm(go)
    print("loss %.6g (fp64 %.6g), gradient rel err vs fp64 %.3g" % (L, float(Lo), err))
    assert abs(L - float(Lo)) <= 1e-4 * abs(float(Lo))
    assert err <= 1e-3


def test_gradient_matches_finite_differences(sim, problem):
    noise, target, g, _ = problem
    filt, green, vf = oracle_inputs(sim)
    n64 = noise.double().cpu()
    t64 = target.double().cpu()
    rng = np.random.default_rng(7)
    idx = rng.choice(NPD ** 3, 64, replace=False)
    eps = 1e-3
    fd = []
    with torch.no_grad():
        for i in idx:
            e = torch.zeros_like(n64)
            e[i] = eps
            lp = orc.loss(n64 + e, t64, filt, green, NG, NPD, vf, sim.drift, sim.kick).item()
            lm = orc.loss(n64 - e, t64, filt, green, NG, NPD, vf, sim.drift, sim.kick).item()
            fd.append((lp - lm) / (2 * eps))
    fd = np.array(fd)
    gi = g.double().cpu().numpy()[idx]
    err = np.linalg.norm(gi - fd) / np.linalg.norm(fd)
    print("gradient rel err vs central differences on 64 points: %.3g" % err)
    assert err <= 1e-3


def test_gradient_does_not_depend_on_checkpoint_interval(problem):
    noise, target, g, _ = problem
    for ck in (1, 3, NSTEPS):
        s = make(ckpt=ck)
        try:
            gk, _ = gpu_grad(s, noise, target)
        finally:
            s.close()
        err = float((gk - g).norm() / g.norm())
        assert err < 1e-5, (ck, err)


def test_initial_state_cotangents_match_fp64(sim):
    # cotangents of the initial (x, v) for a linear functional of the final state
    filt, green, vf = oracle_inputs(sim)
    noise = sim.noise(5)
    sim.forward(noise)
    rng = np.random.default_rng(9)
    wx = torch.tensor(rng.standard_normal((NPD ** 3, 3)), dtype=torch.float32, device=noise.device)
    wv = torch.tensor(rng.standard_normal((NPD ** 3, 3)), dtype=torch.float32, device=noise.device)
    gn, gx0, gv0 = sim.backward(wx, wv, initial=True)
    n64 = noise.double().cpu().requires_grad_(True)
    x0, v0 = orc.ic(n64, filt, NPD, NG // NPD, vf)
    x0r = x0.detach().requires_grad_(True)
    v0r = v0.detach().requires_grad_(True)
    x, v = x0r, v0r
    mass = float(NG) ** 3 / float(NPD) ** 3
    for dr, kk in zip(sim.drift, sim.kick):
        x = x + float(dr) * v
        v = v + float(kk) * orc.force_at(x, orc.potential(orc.deposit(x, NG, NPD, mass), green, NG), NG, NPD)
    L = (x * wx.double().cpu()).sum() + (v * wv.double().cpu()).sum()
    L.backward()
    for got, ref in ((gx0, x0r.grad), (gv0, v0r.grad)):
        err = float((got.double().cpu() - ref).norm() / ref.norm())
        assert err <= 1e-3, err
    # and through the initial conditions to the noise
    (x0 * x0r.grad).sum().add((v0 * v0r.grad).sum()).backward()
    err = float((gn.double().cpu() - n64.grad).norm() / n64.grad.norm())
    assert err <= 1e-3, err


@pytest.fixture(scope="module")
def workload():
    # the differentiable workload itself: 128^3 particles, 256^3 mesh,
    # 256 Mpc/h, 10 steps z=9 -> 0, checkpoint every 2 steps; its FP64
    # gradient by autograd on the GPU in float64
    s = make(ng=256, npd=128, box=256.0)
    try:
        target = s.density(s.forward(s.noise(2))[0]).detach()
        noise = s.noise(1)
        g, L = gpu_grad(s, noise, target)
        g2, _ = gpu_grad(s, noise, target)
        filt, green, vf = oracle_inputs(s)
        drift, kick = s.drift, s.kick
    finally:
        s.close()
    w = dict(noise=noise, target=target, g=g, g2=g2, L=L, filt=filt, green=green, vf=vf, drift=drift, kick=kick)
    n64 = noise.double().requires_grad_(True)
    Lo = orc.loss(n64, target.double(), filt, green, 256, 128, vf, drift, kick)
    Lo.backward()
    w["g64"], w["L64"] = n64.grad.detach(), float(Lo)
    return w


def test_workload_gradient_is_deterministic(workload):
    # fixed-point scatters: two passes give the same gradient bit for bit
    assert torch.equal(workload["g"], workload["g2"])


def test_workload_gradient_matches_fp64(workload):
    # The CIC loss's gradient is piecewise constant in the positions (the
    # weights' slopes jump at cell faces).  FP32 and FP64 trajectories differ
    # by about 1e-6 cells, so a few of the 2M particles sit on different sides
    # of a face, and each such jump reaches every noise point through the
    # adjoint Poisson solves: the error concentrates on a small set of noise
    # points.  Bounds: 1.5e-3 over all points, 1e-3 without the 0.1% largest.
    w = workload
    go = w["g64"].double().cpu().numpy()
    gg = w["g"].double().cpu().numpy()
    err = np.linalg.norm(gg - go) / np.linalg.norm(go)
    dv = np.abs(gg - go)
    keep = dv <= np.quantile(dv, 0.999)
    trimmed = np.linalg.norm((gg - go)[keep]) / np.linalg.norm(go[keep])
    print("workload loss %.6g (fp64 %.6g), gradient rel err vs fp64 %.3g, without the 0.1%% largest %.3g" %
          (w["L"], w["L64"], err, trimmed))
    assert abs(w["L"] - w["L64"]) <= 1e-4 * abs(w["L64"])
    assert err <= 1.5e-3 and trimmed <= 1e-3


def test_workload_gradient_matches_finite_differences(workload):
    # central differences of the FP64 loss on 64 random noise points of the
    # 128^3 lattice.  With eps = 1e-3 a perturbation moves particles by about
    # 1e-4 cells, across the cell faces where the loss's slope jumps, so the
    # differences themselves stray from the exact (FP64) gradient; with
    # eps = 1e-5 they follow it.  The GPU gradient must be as close to the
    # eps = 1e-3 differences as the FP64 gradient is (within 1e-3), and within
    # 1e-3 of the eps = 1e-5 differences.
    w = workload
    n64 = w["noise"].double()
    t64 = w["target"].double()
    rng = np.random.default_rng(17)
    idx = rng.choice(128 ** 3, 64, replace=False)
    args = (w["filt"], w["green"], 256, 128, w["vf"], w["drift"], w["kick"])

    def fd(eps):
        out = []
        with torch.no_grad():
            for i in idx:
                e = torch.zeros_like(n64)
                e[int(i)] = eps
                out.append((orc.loss(n64 + e, t64, *args).item() - orc.loss(n64 - e, t64, *args).item()) / (2 * eps))
        return np.array(out)

    fd3, fd5 = fd(1e-3), fd(1e-5)
    gi = w["g"].double().cpu().numpy()[idx]
    g64 = w["g64"].double().cpu().numpy()[idx]
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))
    print("workload gradient vs central differences on 64 points: GPU %.3g / FP64 %.3g (eps 1e-3), "
          "GPU %.3g / FP64 %.3g (eps 1e-5)" % (rel(gi, fd3), rel(g64, fd3), rel(gi, fd5), rel(g64, fd5)))
    assert rel(gi, fd3) <= rel(g64, fd3) + 1e-3
    assert rel(gi, fd5) <= 1e-3


def test_rejects_bad_geometry():
    from cafproject_gb300.cube import CubeError
    with pytest.raises(CubeError):
        make(ng=48, npd=32)
