#!/usr/bin/env python
"""Particle-steps/s of CUBE's per-step gravity/update path on one GB300.

Workload ``cdm512``: 512^3 CDM particles, 600 Mpc/h, coarse mesh 256^3, fine
mesh 1024^3 (2^3 tiles of the reference), PP within +-1 fine cell with
rsoft=0.1, int8 positions / int16 velocities, Zel'dovich initial conditions at
z=49 from the Eisenstein-Hu no-wiggle spectrum (synthetic, seeded).

One step is the reference's loop body (CUBEnu/work/main/main.f90:102-118):
timestep (host) -> update_x -> buffer_grid -> buffer_x -> ext_pp_force ->
particle_mesh -> buffer_v, every call through the C ABI of libcube_gb300.so
(ext_pp_force and particle_mesh as the one call cube_pp_particle_mesh, which
runs PP beside the PM force chain with the same results).

``value``: N*K / device time of K steps (CUDA events on the library's
stream), state resident in HBM.  ``e2e``: the same metric when every step also
uploads the state from pinned host arrays and downloads it again (what a host
caller holding the reference's arrays pays).  ``--impl reference`` times the
reference's CPU algorithm (the oracle restatement, OpenMP on every host core)
over whole steps of the same workload (at most two, each about half a minute).  ``--gpus N`` runs N independent replicas
(the path does not shard on one-GPU machines); value sums them, time is the max.
"""
import argparse
import copy
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/s at 512^3 PM+PP"
UNIT = "particle-steps/s"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="cdm512")
    ap.add_argument("--z", type=float, default=49.0)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--e2e-steps", type=int, default=0)
    ap.add_argument("--no-adjoint", action="store_true", help="skip the differentiable-form line")
    ap.add_argument("--adjoint-only", action="store_true", help="run only the differentiable-form measurement")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched-ensemble line")
    ap.add_argument("--batched-only", action="store_true", help="run only the batched-ensemble measurement")
    ap.add_argument("--no-two-species", action="store_true", help="skip the two-species line")
    ap.add_argument("--no-redshifts", action="store_true", help="skip the later-redshift steps")
    ap.add_argument("--redshifts", default="5,1",
                    help="redshifts of the evolved run at which to time the step (z=0 takes ~1500 steps)")
    ap.add_argument("--two-species-only", action="store_true", help="run only the two-species measurement")
    ap.add_argument("--boxes", type=int, default=256, help="batched ensemble size")
    ap.add_argument("--profile-range", choices=["step", "z"], default=None,
                    help="bracket the timed steps (step) or the last redshift's timed steps (z) with "
                         "cudaProfilerStart/Stop, for ncu --profile-from-start off")
    return ap.parse_args()


def dist_init():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    lrank = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        # one process per GPU over NCCL; gloo where there is no GPU (host tests)
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    return ws, rank, lrank


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def allreduce_max(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def allreduce_sum(x, ws, device):
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def replica_throughput(units, seconds, ws, device):
    """Whole-job throughput of ws independent replicas (no data-path
    collective): the units all ranks processed over the slowest rank's time."""
    return allreduce_sum(float(units), ws, device) / allreduce_max(float(seconds), ws, device)


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu):
        self.gpu = gpu
        self.f = tempfile.NamedTemporaryFile(mode="w+", suffix=".csv", delete=False)
        self.p = None

    def start(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.Q,
                                       "--format=csv,noheader,nounits", "-lms", "200"],
                                      stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self):
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        self.p.terminate()
        try:
            self.p.wait(timeout=5)
        except Exception:
            self.p.kill()
        self.f.flush()
        rows = [r.split(",") for r in open(self.f.name).read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            r = [x.strip() for x in r]
            if len(r) < 9:
                continue
            try:
                sm.append(float(r[1]))
                smax.append(float(r[2]))
            except ValueError:
                continue
            for n, v in zip(names, r[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ gb300 arm


# DRAM bytes (read + write) per particle of one launch, from the full ncu
# capture of the 256^3 workload (profiles/step_kernels_cdm256.md); meshes and
# particle counts scale together between 256^3 and 512^3, so per-particle
# traffic carries over
TRAFFIC_PER_PARTICLE = {
    # one ncu capture per kernel at 256^3 (profiles/step_kernels_cdm256.md),
    # DRAM read + write per launch over the particles; pp_force: the brick
    # kernel and the neighbour-mask pass that marks the active particles
    # (the prefilter's smaller passes uncaptured)
    "pp_force": (93.1e6 + 34.2e6 + 113.5e6 + 4.5e6) / 16778347,
    "fine_kick": (2194.1e6 + 114.8e6) / 16778347,
    "coarse_kick": (325.2e6 + 89.9e6) / 16778347,
    "fine_deposit": (83.7e6 + 476.4e6) / 16778347,
    "update_dest": (243.8e6 + 77.9e6) / 16778347,
    "update_scatter": (506.5e6 + 257.2e6) / 16778347,
    "fine_green": (1347.5e6 + 1567.8e6) / 16778347,
    "fine_f2max": (1617.1e6 + 1560.4e6) / 16778347,
}


def algorithmic_bytes(p, n):
    """Algorithmic bytes per launch of each phase (each array element read or
    written once; s = 3*izipx+3*izipv bytes of particle code)."""
    nf3, nc3 = p.nf ** 3, p.nc ** 3
    hf = (p.nf // 2 + 1) * p.nf * p.nf
    hc = (p.nc // 2 + 1) * p.nc * p.nc
    s = 3 * p.izipx + 3 * p.izipv
    cell = 4 + 4  # rhoc + cell start (int32 index, int32 count)
    return {
        "update_dest": n * (s + 4) + n * 5,                 # read x,v,cell; write dest+frame
        # counting rank path: local ranks + 27 uint16 counts per cell, then base ranks in place
        "update_rank": n * (4 + 1 + 2) + nc3 * (8 + 3 * 54 + 4),
        "update_place": n * (4 + 4 + 1 + 2 + 2 + 8 + 4 + 4) + n * (4 + 4 + 3 * p.izipv + 12) + nc3 * (4 + 8 + 12 + 12),
        "update_scan": nc3 * (4 + 8),
        "update_scatter": n * (s + 4 + 4 + 4 + 5) + n * (s + 4 + 4),
        "update_sigma": n * (3 * p.izipv + 4) + nc3 * 12,
        "pp_force": n * (3 * p.izipx + 2 * 3 * p.izipv + 4),
        "fine_deposit": n * (3 * p.izipx + 4) + 4 * nf3,
        "fine_r2c": 4 * nf3 + 8 * hf,
        "fine_green": 8 * hf + 12 * hf + 3 * 8 * hf,
        "fine_c2r": 3 * (8 * hf + 4 * nf3),
        "fine_f2max": 12 * nf3 + 12 * nf3,                 # maxima, then the kick factors written back
        "fine_kick": n * (3 * p.izipx + 2 * 3 * p.izipv + 4) + 12 * nf3,
        "coarse_deposit": n * (3 * p.izipx + 4) + 4 * nc3,
        "coarse_fft": (4 * nc3 + 8 * hc) + (8 * hc + 12 * hc + 24 * hc) + 3 * (8 * hc + 4 * nc3) + 24 * nc3,
        "coarse_kick": n * (3 * p.izipx + 2 * 3 * p.izipv + 4 + 12) + 12 * nc3,
    }


def run_redshifts(args, lrank, zs=(5.0, 0.0)):
    """The same 512^3 step at later redshifts of one run evolved on the GPU
    from the initial conditions under the reference's dt constraints
    (timestep.f90, pm.f90:391-407), where clustering makes PP and the
    re-sort dearer: the run stops at each z (the timestep's checkpoint
    landing), then args.warmup + args.steps more steps continue from there
    and the last args.steps are timed (CUDA events on the library stream),
    with the step's PP and PM as one call as in the headline."""
    import torch

    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300.cosmology import TimeState

    torch.cuda.set_device(lrank)
    p = P.WORKLOADS[args.workload]()
    out = {}
    g = C.CubeGPU(p, device=lrank)
    try:
        sigma, vm = g.ic_zeldovich(args.z, args.seed)
        ts = TimeState(a=np.float32(1.0 / (1.0 + args.z)), omega_m=p.omega_m, omega_l=p.omega_l)
        ts.vz_max = np.float32(vm[2])
        ts.dt_vmax = np.float32(np.float32(18.0) / np.float32(max(vm)))
        stream = torch.cuda.ExternalStream(g.stream())
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        nsteps = 0

        def step():
            nonlocal nsteps
            dt, a_mid = ts.timestep()
            g.update_x(ts.dt_old, dt, ts.vz_max)
            pps, pms = g.pp_particle_mesh(a_mid, dt)
            ts.constrain(pms, pps, p.ncell)
            nsteps += 1
            return pps

        t0 = time.perf_counter()
        for z in zs:
            ts.z_checkpoints, ts.cur_checkpoint, ts.final_step = [z], 0, False
            while not ts.final_step and nsteps < 5000:
                step()
            reached = nsteps
            ts.z_checkpoints = []  # the timed steps continue past z
            for _ in range(args.warmup):
                step()
            g.synchronize()
            prof = args.profile_range == "z" and z == zs[-1]
            if prof:
                torch.cuda.profiler.start()
            e0.record(stream)
            for _ in range(args.steps):
                pps = step()
            e1.record(stream)
            g.synchronize()
            if prof:
                torch.cuda.profiler.stop()
            ms = e0.elapsed_time(e1) / args.steps
            out["%g" % z] = {"ms_per_step": round(ms, 2), "value": g.nplocal() / (ms / 1000.0),
                             "pp_pairs_per_step": int(pps["npairs"]), "steps_from_ics": reached,
                             "state": "evolved on the GPU from z=%g" % args.z,
                             "wall_s_since_ics": round(time.perf_counter() - t0, 1)}
    finally:
        g.close()
    return out


def run_gb300(args, ws, rank, lrank):
    import torch

    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300.cosmology import TimeState

    torch.cuda.set_device(lrank)
    dev = torch.device("cuda", lrank)
    p = P.WORKLOADS[args.workload]()
    # initial conditions generated on the device by the library's IC kernels
    t_ic = time.perf_counter()
    g = C.CubeGPU(p, device=lrank)
    sigma, vm = g.ic_zeldovich(args.z, args.seed + rank)
    a0 = 1.0 / (1.0 + args.z)
    t_ic = time.perf_counter() - t_ic
    ts = TimeState(a=np.float32(a0), omega_m=p.omega_m, omega_l=p.omega_l, z_checkpoints=[0.0])
    ts.vz_max = np.float32(vm[2])
    ts.dt_vmax = np.float32(np.float32(18.0) / np.float32(max(vm)))
    stream = torch.cuda.ExternalStream(g.stream())

    def step(fused=True, after_x=None):
        dt, a_mid = ts.timestep()
        g.update_x(ts.dt_old, dt, ts.vz_max)
        g.buffer_grid()
        g.buffer_x()
        if after_x:
            after_x()
        if p.pp_on and fused:  # ext_pp_force + particle_mesh, PP beside the PM force chain
            pps, pms = g.pp_particle_mesh(a_mid, dt)
        elif p.pp_on:
            pps = g.ext_pp_force(a_mid, dt)
            pms = g.particle_mesh(a_mid, dt)
        else:
            pps, pms = None, g.particle_mesh(a_mid, dt)
        g.buffer_v()
        ts.constrain(pms, pps, p.ncell)
        return pms

    for _ in range(args.warmup):
        step()
    g.synchronize()
    n0 = g.nplocal()
    clocks = ClockSampler(lrank)
    barrier(ws)
    clocks.start()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    g.synchronize()
    torch.cuda.synchronize()
    if args.profile_range == "step":
        torch.cuda.profiler.start()
    e0.record(stream)
    for _ in range(args.steps):
        step()
    e1.record(stream)
    g.synchronize()
    torch.cuda.synchronize()
    if args.profile_range == "step":
        torch.cuda.profiler.stop()
    ms = e0.elapsed_time(e1)
    clk = clocks.stop()
    barrier(ws)
    ms_max = allreduce_max(ms, ws, dev)
    ntot = allreduce_sum(float(n0), ws, dev)
    value = replica_throughput(n0 * args.steps, ms / 1000.0, ws, dev)

    # per-phase device time (timers on, a separate pass so the headline is
    # unperturbed; PP and PM as separate calls so no phase overlaps another)
    g.timing(True)
    kph = max(1, min(args.steps, 3))
    for _ in range(kph):
        step(fused=False)
    tphase = g.timing_read()
    g.timing(False)
    ab = algorithmic_bytes(p, n0)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm = float(peaks.get("hbm_gbs", 6800.0))
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    phases = {}
    for name, (tms, cnt) in tphase.items():
        if cnt == 0:
            continue
        per = tms / cnt
        gbs = ab.get(name, 0) / (per / 1000.0) / 1e9 if per > 0 else 0.0
        phases[name] = {"ms_per_launch": round(per, 4), "launches": int(cnt), "share": 0.0,
                        "algo_bytes": int(ab.get(name, 0)), "achieved_gbs": round(gbs, 1)}
    tot = sum(v["ms_per_launch"] * v["launches"] for v in phases.values())
    for v in phases.values():
        v["share"] = round(v["ms_per_launch"] * v["launches"] / tot, 4) if tot else 0.0
    own = {k: v for k, v in phases.items() if k not in ("fine_r2c", "fine_c2r", "coarse_fft")}
    dom = max(own, key=lambda k: own[k]["ms_per_launch"] * own[k]["launches"]) if own else None
    roof = None
    if dom:
        d = phases[dom]
        roof = {"kernel": dom, "bound": "hbm", "achieved": d["achieved_gbs"], "peak": hbm, "unit": "GB/s",
                "frac": round(d["achieved_gbs"] / hbm, 4), "peak_source": peak_src,
                "traffic": (round(TRAFFIC_PER_PARTICLE[dom] * n0) if dom in TRAFFIC_PER_PARTICLE else None),
                "traffic_source": "ncu capture at 256^3 scaled per particle" if dom in TRAFFIC_PER_PARTICLE else None,
                "algo_bytes_per_launch": d["algo_bytes"]}

    # e2e: host arrays in, host arrays out, every step
    ke = args.e2e_steps or max(10, args.steps)
    pin = {k: torch.from_numpy(v).pin_memory() for k, v in g.download().items()}
    hin = {k: v.numpy() for k, v in pin.items()}
    outt = {k: torch.empty_like(v).pin_memory() for k, v in pin.items()}
    out = {k: v.numpy() for k, v in outt.items()}
    h2d = sum(v.nbytes for v in hin.values())

    # xp and vp travel to the device in pieces beside the re-sort's first
    # pass, pid beside the rest of it; xp, pid, rhoc and vfield to the host
    # beside PP+PM, vp behind the coarse kick
    # every e2e step is the same step: the snapshot, its codec sigma and the
    # time state it was taken at (a time state left to advance would drift
    # the same snapshot by ever longer dt, until the re-sort's multi-cell path
    # ran every step)
    sig0 = g.get_sigma()
    ts0 = copy.deepcopy(ts)

    def e2e_step():
        ts.__dict__.update(copy.deepcopy(ts0.__dict__))
        g.upload_begin(hin["xp"], hin["vp"], hin["pid"], hin["rhoc"], hin["vfield"])
        g.set_sigma(*sig0)
        step(after_x=lambda: g.download_begin(out))
        g.download_finish()

    e2e_step()  # untimed: the copy stream's first use and the fresh pinned buffers' first transfers
    barrier(ws)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    tstep = []
    for _ in range(ke):
        t_s = time.perf_counter()
        e2e_step()  # ends when the step's download has landed in host memory
        tstep.append(1e3 * (time.perf_counter() - t_s))
    torch.cuda.synchronize()
    te = time.perf_counter() - t0
    te = allreduce_max(te, ws, dev)
    e2e = {"value": ntot * ke / te, "unit": UNIT, "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(h2d),
           "steps": ke, "step_ms": [round(t, 2) for t in tstep]}

    cpu = None
    if rank == 0 and ws == 1 and not args.no_cpu:
        cpu = cpu_baseline(p, g.download(), float(g.get_sigma()[0]), ts)
    g.close()
    return dict(value=value, ms=ms_max / args.steps, clocks=clk, phases=phases, roofline=roof, e2e=e2e,
                cpu=cpu, n=int(ntot), p=p, t_ic=t_ic, gpu_launches=gpu_launches(p, args.steps))


def run_adjoint(args, lrank, reps=3):
    """Adjoint / forward cost of the differentiable form on its workload:
    128^3 particles, 256^3 mesh, 256 Mpc/h, 10 steps z=9 -> 0, checkpoint every
    2 steps, loss = sum (rho_final - rho_target)^2 with the target from a
    second seed.  Forward = IC + 10 steps + final density; adjoint = density
    adjoint + backward (segment re-runs included) + IC adjoint.  Device times
    from CUDA events on the library's stream."""
    import torch

    from cafproject_gb300.dpm import DiffPM

    sim = DiffPM(256, 128, 9.0, 0.0, 10, ckpt_every=2, device=lrank, box=256.0)
    try:
        target = sim.density(sim.forward(sim.noise(args.seed + 1))[0])
        noise = sim.noise(args.seed)
        stream = torch.cuda.ExternalStream(sim.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        fw, bw, tot_f, tot_b = [], [], [], []
        for i in range(args.warmup + reps):
            torch.cuda.synchronize()
            x, v = sim.forward(noise)
            rho = sim.density(x)
            grho = 2.0 * (rho - target)
            torch.cuda.synchronize()
            info0 = sim.info()
            gx = sim.density_adjoint(x, grho)
            gn = sim.backward(gx, torch.zeros_like(v))
            info1 = sim.info()
            # the two mesh passes of the loss, timed alone on the library's stream
            torch.cuda.synchronize()
            ev[0].record(stream)
            sim.density(x)
            ev[1].record(stream)
            ev[2].record(stream)
            sim.density_adjoint(x, grho)
            ev[3].record(stream)
            torch.cuda.synchronize()
            if i >= args.warmup:
                fw.append(info0["forward_ms"] + ev[0].elapsed_time(ev[1]))
                bw.append(info1["backward_ms"] + ev[2].elapsed_time(ev[3]))
                tot_f.append(info0["forward_ms"])
                tot_b.append(info1["backward_ms"])
        f, b = statistics.median(fw), statistics.median(bw)
        assert torch.isfinite(gn).all()
        return {"workload": "dpm128: 128^3 particles, 256^3 mesh, 256 Mpc/h, 10 steps z=9->0, checkpoint every 2",
                "forward_ms": round(f, 3), "adjoint_ms": round(b, 3), "ratio": round(b / f, 3), "target_ratio": 3.0,
                "graph_forward_ms": round(statistics.median(tot_f), 3),
                "graph_backward_ms": round(statistics.median(tot_b), 3), "reps": reps,
                "gradient_checks": "tests/test_gpu_dpm.py (FP64 autograd and central differences)"}
    finally:
        sim.close()


def run_two_species(args, lrank, m_nu=0.05, z_init=10.0):
    """The two-species workload: 512^3 CDM (np_nc 2, PP on) plus 1024^3
    thermal neutrinos (np_nc 4, m_nu 0.05 eV, Fermi-Dirac speeds) in a
    1 Gpc/h box, nc 256 over 4^3 tiles, the neutrinos sharing the meshes
    (cube_create_linked); initial conditions on the device at z = 10, then
    steps under the reference's dt constraints with both species' vmax.  The
    neutrinos move several coarse cells a step, so their re-sort takes the
    sort of all landings."""
    import torch

    from cafproject_gb300 import cube as C
    from cafproject_gb300 import params as P
    from cafproject_gb300.cosmology import TimeState

    torch.cuda.set_device(lrank)
    h0, om = 0.7, 0.3
    # mean density one per fine cell, split by Omega_nu h^2 = m_nu / 93.14 eV
    f_nu = m_nu / 93.14 / h0 ** 2 / om
    pc = P.CubeParams(nc=256, nnt=4, pp_on=True, rsoft=0.1, box=1000.0, np_nc=2, mass_p=8.0 * (1 - f_nu))
    pn = P.CubeParams(nc=256, nnt=4, pp_on=False, box=1000.0, np_nc=4, mass_p=1.0 * f_nu)
    t0 = time.perf_counter()
    g = C.CubeGPU(pc, device=lrank)
    nu = C.CubeGPU(pn, owner=g)
    try:
        sc, vc = g.ic_zeldovich(z_init, args.seed)
        sn, vn = nu.ic_zeldovich_nu(z_init, args.seed, m_nu, args.seed + 7)
        g.synchronize()
        t_ic = time.perf_counter() - t0
        ts = TimeState(a=np.float32(1.0 / (1.0 + z_init)), omega_m=om, omega_l=1 - om)
        ts.vz_max = np.float32(max(vc[2], vn[2]))
        ts.dt_vmax = np.float32(np.float32(18.0) / np.float32(max(max(vc), max(vn))))
        stream = torch.cuda.ExternalStream(g.stream())
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(5)]
        parts = []
        info = {}

        def step(timed):
            dt, a_mid = ts.timestep()
            if timed:
                ev[0].record(stream)
            uc = g.update_x(ts.dt_old, dt, ts.vz_max)
            if timed:
                ev[1].record(stream)
            un = nu.update_x(ts.dt_old, dt, ts.vz_max)
            if timed:
                ev[2].record(stream)
            pp = g.ext_pp_force(a_mid, dt)
            if timed:
                ev[3].record(stream)
            st, stn = g.particle_mesh2(nu, a_mid, dt)
            if timed:
                ev[4].record(stream)
                torch.cuda.synchronize()
                parts.append([ev[i].elapsed_time(ev[i + 1]) for i in range(4)])
            ts.constrain({"f2_max_fine": st["f2_max_fine"], "f2_max_coarse": st["f2_max_coarse"],
                          "vmax": [max(st["vmax"][d], stn["vmax"][d]) for d in range(3)]}, pp, pc.ncell)
            info.update(nu_rank_path=int(un["rank_walked"]), nu_max_disp=int(un["max_disp"]),
                        nu_nlayer=int(un["nlayer"]), cdm_rank_path=int(uc["rank_walked"]),
                        nu_ndup=int(un["ndup"]))

        for _ in range(max(1, args.warmup - 1)):
            step(False)
        for _ in range(args.steps):
            step(True)
        n = g.nplocal() + nu.nplocal()
        # per-phase device time of one more step, timers on (not in the value)
        g.timing(True)
        nu.timing(True)
        step(False)
        phases = {"cdm": {k: round(v[0], 2) for k, v in g.timing_read().items() if v[1]},
                  "nu": {k: round(v[0], 2) for k, v in nu.timing_read().items() if v[1]}}
        g.timing(False)
        nu.timing(False)
        ms = [sum(x) for x in parts]
        med = statistics.median(ms)
        brk = {k: round(statistics.median(x[i] for x in parts), 2)
               for i, k in enumerate(("update_cdm", "update_nu", "pp_cdm", "pm_both"))}
        return {"metric": "particle-steps/s, 512^3 CDM + 1024^3 neutrinos", "value": n / (med / 1000.0),
                "unit": UNIT, "ms_per_step": round(med, 2), "steps": args.steps, "ms_breakdown": brk,
                "particles": {"cdm": int(g.nplocal()), "nu": int(nu.nplocal())}, "ic_s": round(t_ic, 1),
                "z_init": z_init, "m_nu_ev": m_nu, "timing": "CUDA events on the library stream, per step",
                "phases_ms": phases,
                "config": {"workload": "two-species 1 Gpc/h", "nc": 256, "nf": 1024, "nnt": 4, "pp": "cdm",
                           "np_nc": {"cdm": 2, "nu": 4}}, **info}
    finally:
        nu.close()
        g.close()


def run_batched(args, lrank, nsteps=50):
    """Boxes/s of the batched ensemble against the plain form run serially:
    256 boxes, each 32^3..128^3 particles (uniform choice), fine mesh twice the
    particle grid, Omega_m ~ U[0.25, 0.35], sigma_8 ~ U[0.7, 0.9], seed
    base+box, PM+PP, 50 steps equal in ln a from z=19 to z=0.  Graph mode: one
    captured CUDA graph launch per step for all boxes; serial: the plain entry
    points box after box.  Both produce the same state bit for bit
    (tests/test_gpu_batch.py).  Wall-clock time of the 50 steps; creation and
    initial conditions reported apart."""
    from cafproject_gb300 import batch as B

    ens = B.ensemble(args.boxes, base_seed=args.seed)
    out = {}
    for name, mode in (("graph", B.GRAPH), ("serial", B.SERIAL)):
        t0 = time.perf_counter()
        b = B.Batch(ens, z_init=19.0, mode=mode, device=lrank)
        b.set_schedule(0.0, nsteps)
        levels = b.autotune() if mode == B.GRAPH else None
        t1 = time.perf_counter()
        b.step(nsteps)
        t2 = time.perf_counter()
        tm = b.time()
        last = b.history(nsteps - 1)
        per = b.step_times()
        b.close()
        out[name] = {"boxes_per_s": round(args.boxes / (t2 - t1), 3),
                     "box_steps_per_s": round(args.boxes * nsteps / (t2 - t1), 1), "steps_s": round(t2 - t1, 3),
                     "device_s": round(tm["device_ms"] / 1000.0, 3), "setup_s": round(t1 - t0, 3),
                     "final_npairs": int(sum(h["npairs"] for h in last)),
                     "step_ms_first_mid_last": [round(float(per[0]), 1), round(float(per[nsteps // 2]), 1),
                                                round(float(per[-1]), 1)]}
        if levels is not None:  # autotuned (PP level, fine deposit shape, coarse deposit shape) per geometry
            tuned = {}
            for (pn, _), ch in zip(ens, levels):
                tuned["%d^3" % (pn.nc * 2)] = [int(x) for x in ch]
            out[name]["tuned"] = tuned
    nper = [p.nc * 2 for p, _ in ens]
    return {"workload": "%d boxes of %s^3 particles (uniform), fine mesh 2x the particle grid, PM+PP, %d steps "
                        "z=19->0 (equal in ln a), Omega_m U[0.25,0.35], sigma_8 U[0.7,0.9]"
                        % (args.boxes, "/".join(str(s) for s in sorted(set(nper))), nsteps),
            "particles": int(sum(n ** 3 for n in nper)), "graph": out["graph"], "serial": out["serial"],
            "speedup": round(out["graph"]["boxes_per_s"] / out["serial"]["boxes_per_s"], 3), "target_speedup": 4.0,
            "same_state": "bitwise (tests/test_gpu_batch.py)"}


def workload_config(p, n, z_init):
    """The config dict both arms print: the workload, its sizes and inputs
    (the same keys and values for the same workload on either arm)."""
    from cafproject_gb300 import params as P
    name = "custom"
    for k, f in P.WORKLOADS.items():
        q = f()
        if (q.nc, q.nnt, q.pp_on, q.box, q.np_nc) == (p.nc, p.nnt, p.pp_on, p.box, p.np_nc):
            name = k
    state_gb = n * (3 * p.izipx + 3 * p.izipv + 4) / 1e9
    mesh_gb = 4.0 * (p.nf + 2) * p.nf * p.nf / 1e9
    return {"workload": name, "particles": int(n), "nc": p.nc, "nf": p.nf, "nnt": p.nnt, "pp": bool(p.pp_on),
            "rsoft": p.rsoft, "izipx": p.izipx, "izipv": p.izipv, "box_mpc_h": p.box, "z_init": z_init,
            "l2": "inputs larger than L2 (state %.1f GB, fine mesh %.1f GB)" % (state_gb, mesh_gb)}


def gpu_launches(p, steps):
    """Launches of this library's kernels per step (cuFFT kernels not counted)."""
    upd = 1 + 3 + 3 + 3 + 1 + 1  # dest, counting ranks (3: local, dense cells, base), scan (3),
    #                               place + two vfield passes, scatter, sigma
    # PP: the prefilter (occupancy, neighbour masks with the activity bits, a
    # scan of 3, compaction, cell starts), six staging levels, the active
    # particles' kick
    pp = 7 + 6 + 1 if p.pp_on else 0
    fine = 4                     # deposit, green, maxima + kick factors, kick (PP's zero kicks inside)
    coarse = 4
    codec = 3                    # decode table, encode boundaries and zero-kick table for the new sigma
    return steps * (upd + pp + fine + coarse + codec)


def cpu_baseline(p, state, sigma, ts):
    from oracle import cube_oracle as O
    ncore = os.cpu_count() or 1
    r = O.time_sample(p, state, sigma, float(ts.a_mid), float(ts.dt), float(ts.dt_old), float(ts.vz_max),
                      tile=0, nthreads=0)
    n = state["xp"].shape[0]
    return {"value": n / r["step_estimate"], "unit": UNIT, "cores": ncore, "kind": "port",
            "sample": "one of %d tiles of update_xp, PP and fine PM plus the image-wide buffering and coarse PM "
                      "(%.1f s of CPU work); step = %d x tile + image-wide" % (p.nnt ** 3, r["sampled"],
                                                                                p.nnt ** 3),
            "detail": {k: round(v, 3) for k, v in r.items()}}


# -------------------------------------------------------------- reference arm


REF_MAX_STEPS = 2  # whole 512^3 steps of the CPU path, about a minute each on 16 cores


def run_reference(args, ws, rank):
    """The reference's CPU algorithm (the oracle restatement: OpenMP over all
    host cores, FP64 pair and velocity arithmetic, scipy FFTs) stepping the
    same workload: whole steps -- timestep, update_x with its buffering,
    ext_pp_force, particle_mesh over every tile, buffer_v -- timed one by
    one.  Kernel construction and the first buffering are set-up
    (initialize, particle_initialization) and untimed; no warm-up step is
    needed for host code, and at most REF_MAX_STEPS steps are timed so the
    run ends within a few minutes."""
    if rank != 0:
        return None
    import torch

    from cafproject_gb300 import ic, params as P
    from cafproject_gb300.cosmology import TimeState
    from oracle import cube_oracle as O

    p = P.WORKLOADS[args.workload]()
    dev = torch.device("cuda", 0) if torch.cuda.is_available() else torch.device("cpu")
    st = ic.zeldovich(p, args.z, args.seed, device=dev)
    state = {k: st[k].cpu().numpy() for k in ("xp", "vp", "pid", "rhoc", "vfield")}
    sigma, a0, vm = st["sigma_vi"], st["a"], st["vmax"]
    del st
    torch.cuda.empty_cache() if torch.cuda.is_available() else None
    ts = TimeState(a=np.float32(a0), omega_m=p.omega_m, omega_l=p.omega_l)
    ts.vz_max = np.float32(vm[2])
    ts.dt_vmax = np.float32(np.float32(18.0) / np.float32(max(vm)))
    n = state["xp"].shape[0]
    img = O.OracleImage(p, nthreads=0)
    img.kern_f()
    img.kern_c()
    img.load(state["xp"], state["vp"], state["pid"], state["rhoc"], state["vfield"])
    img.sigma_vi = img.sigma_vi_new = np.float32(sigma)
    del state
    times = []
    for _ in range(max(1, min(args.steps, REF_MAX_STEPS))):
        t0 = time.perf_counter()
        dt, a_mid = ts.timestep()
        img.update_x(ts.dt_old, dt, ts.vz_max)
        pp = img.pp_force(a_mid, dt) if p.pp_on else None
        pm = img.particle_mesh(a_mid, dt)
        ts.constrain(pm, pp, p.ncell)
        times.append(time.perf_counter() - t0)
    value = n * len(times) / sum(times)
    return dict(value=value, ms=1000.0 * sum(times) / len(times), n=n, p=p, steps=len(times),
                step_s=[round(t, 2) for t in times])


def main():
    args = parse()
    ws, rank, lrank = dist_init()
    if args.impl == "reference":
        r = run_reference(args, ws, rank)
        if rank == 0:
            ncore = os.cpu_count() or 1
            p = r["p"]
            cfg = workload_config(p, r["n"], args.z)
            line = {"impl": "reference", "parallelism": "host OpenMP, %d threads" % ncore, "metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": args.gpus,
                    "steps": r["steps"], "steps_requested": args.steps, "warmup": 0, "ms_per_step": r["ms"],
                    "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
                    "dtype": "int8/int16 state, fp32/fp64 arithmetic",
                    "data": "synthetic (seeded Zel'dovich ICs, Eisenstein-Hu no-wiggle P(k), z=%g)" % args.z,
                    "config": cfg,
                    "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": ncore, "kind": "port",
                                     "sample": "%d whole steps of the %d-tile image, timed one by one (s: %s); "
                                               "host OpenMP on every core" % (r["steps"], p.nnt ** 3, r["step_s"])},
                    "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
            print(json.dumps(line), flush=True)
        return
    if args.adjoint_only:
        if rank == 0:
            print(json.dumps({"adjoint": run_adjoint(args, lrank)}), flush=True)
        return
    if args.batched_only:
        if rank == 0:
            print(json.dumps({"batched": run_batched(args, lrank)}), flush=True)
        return
    if args.two_species_only:
        if rank == 0:
            print(json.dumps({"two_species": run_two_species(args, lrank)}), flush=True)
        return
    r = run_gb300(args, ws, rank, lrank)
    adj = run_adjoint(args, lrank) if (rank == 0 and ws == 1 and not args.no_adjoint) else None
    bat = run_batched(args, lrank) if (rank == 0 and ws == 1 and not args.no_batched) else None
    two = run_two_species(args, lrank) if (rank == 0 and ws == 1 and not args.no_two_species) else None
    zs = (run_redshifts(args, lrank, tuple(float(z) for z in args.redshifts.split(",")))
          if (rank == 0 and ws == 1 and not args.no_redshifts) else None)
    if rank == 0:
        p = r["p"]
        line = {"metric": METRIC, "value": r["value"], "unit": UNIT, "n_gpus": ws, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": r["ms"], "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "int8/int16 state, fp32 mesh, fp64 velocity codes",
                "data": "synthetic (seeded Zel'dovich ICs, Eisenstein-Hu no-wiggle P(k), z=%g)" % args.z,
                "config": workload_config(p, r["n"], args.z),
                "parallelism": "replicas x%d" % ws if ws > 1 else "single GPU",
                "clocks": r["clocks"], "e2e": r["e2e"], "roofline": r["roofline"], "gpu_launches": r["gpu_launches"],
                "phases": r["phases"]}
        if r["cpu"]:
            line["cpu_baseline"] = r["cpu"]
        if adj:
            line["adjoint"] = adj
        if bat:
            line["batched"] = bat
        if two:
            line["two_species"] = two
        if zs:
            zs = {"%g" % args.z: {"ms_per_step": round(r["ms"], 2), "value": r["value"]}, **zs}
            line["redshifts"] = zs
        print(json.dumps(line), flush=True)
    if ws > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
