#!/usr/bin/env python
"""Benchmark of the GB300 thermal Monte Carlo (pdspy Model.run_thermal, code="gb300").

Workload (default): 64 MCMC-walker power-law disks in one batched plan, 1e6 photon
packets per model, parameters drawn from a seed (Mdisk log-uniform 1e-5..1e-2 Msun, Rout
20..300 au, h0 0.03..0.2, flaring 1.0..1.3, surface-density index 0..1.5, nr 64..256,
ntheta 64..192), small-grain dust with HG scattering, modified random walk on with
pdspy's production settings (gamma 2, tauthres 10, count trigger 100).  Synthetic
inputs, built in memory.

A step is one full thermal run of the batch (all epochs, both continuation stages and the
temperature inversion).  ``value`` is packets/s with the densities resident in HBM (CUDA
events around the run); ``e2e`` is the same step through the public API with host arrays,
timed on the same stream from the pinned H2D copy of the densities to the D2H copy of the
temperatures.  The longest packet walks of this workload (about 1.5e8 interactions for one
walker at 1e6 packets with the default seed; the walk lengths are heavy-tailed, as in
sequential Bjorkman & Wood) set most of a step's time, so step k runs Monte Carlo seed
seed + k and the line reports every step's time with its tail (the warp-per-packet stage)
and bulk parts; warm-up runs are cut at a short device deadline.  The reference arm
(``--impl reference``) times the CPU restatement of the same algorithm (the reference's
own path is the external RADMC-3D binary, which is not available) on a bounded sample of
the workload, every walker at 1e4 packets in a pool of single-threaded workers
(``--cpu-full``: the whole workload).

The same JSON line carries the adjoint gradient rate, the scattering source of an SED
(with its CPU restatement), gridded vs direct visibility sampling and, with
``--lnprob-walkers``, the batched MCMC lnprob; ``--workload plain|envelope|spiral`` runs
the single small disk, the disk plus envelope (256 x 256 cells) or four phases of the 3-D
spiral (128^3 cells) instead of the walkers.

With torchrun (N > 1) every rank runs its own independent batch of walkers (the models
shard with no data-path collective): weak scaling, value = all ranks' packets / max time.
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

MRW = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)
METRIC = "packets/s batched vs plain GPU at <=1% median dT/T; adjoint grads/s; host CPU"


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched",
                    choices=["batched", "plain", "envelope", "spiral"],
                    help="batched walkers (default), one small disk (plain), the disk plus "
                         "envelope on 256 x 256 cells (envelope) or four phases of the 3-D "
                         "two-population spiral disk on 128^3 cells (spiral)")
    ap.add_argument("--models", type=int, default=64)
    ap.add_argument("--packets", type=int, default=1000000, help="packets per model")
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-adjoint", action="store_true")
    ap.add_argument("--adjoint-reps", type=int, default=10)
    ap.add_argument("--no-scattering", action="store_true")
    ap.add_argument("--lnprob-walkers", type=int, default=0,
                    help="also time the batched MCMC lnprob of this many walkers (0: off)")
    ap.add_argument("--lnprob-packets", type=int, default=100000)
    ap.add_argument("--cpu-models", type=int, default=64)
    ap.add_argument("--cpu-packets", type=int, default=10000)
    ap.add_argument("--cpu-full", action="store_true",
                    help="reference arm: run the whole workload (every model at --packets)")
    ap.add_argument("--timelimit", type=float, default=1800.0,
                    help="device-side deadline per timed thermal run (s)")
    ap.add_argument("--warmup-deadline", type=float, default=10.0,
                    help="device-side deadline of each warm-up run (s)")
    return ap.parse_args()


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Clocks:
    """Samples nvidia-smi clocks and throttle reasons while the timed region runs."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.samples = []
        self.stop = threading.Event()
        self.t = threading.Thread(target=self.loop, daemon=True)

    def loop(self):
        while not self.stop.is_set():
            try:
                out = subprocess.run(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                      "--format=csv,noheader,nounits"], capture_output=True,
                                     text=True, timeout=5).stdout.strip()
                if out:
                    self.samples.append([x.strip() for x in out.split(",")])
            except Exception:
                pass
            self.stop.wait(0.2)

    def __enter__(self):
        self.t.start()
        return self

    def __exit__(self, *a):
        self.stop.set()
        self.t.join(timeout=10)

    def summary(self):
        if not self.samples:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = set()
        for s in self.samples:
            for n, v in zip(names, s[4:8]):
                if v.strip().lower() == "active":
                    reasons.add(n)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": sorted(reasons),
                "samples": len(self.samples)}


def l2_roofs(dev):
    """Measured L2 roofs on this GPU (lower bounds: torch kernels, not tuned ones): an
    L2-resident copy (two 32 MB buffers, read + write bytes) and int64 atomic adds into a
    32 MB array (torch.index_add_), best of 5."""
    import torch
    n = (32 << 20) // 4
    a = torch.ones(n, dtype=torch.float32, device=dev)
    b = torch.empty_like(a)
    acc = torch.zeros(4 << 20, dtype=torch.int64, device=dev)
    m = 16 << 20
    idx = torch.randint(0, acc.numel(), (m,), device=dev)
    one = torch.ones(m, dtype=torch.int64, device=dev)
    best_c, best_a = 0.0, 0.0
    for _ in range(5):
        e = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
        e[0].record()
        for _ in range(50):
            b.copy_(a)
        e[1].record()
        acc.index_add_(0, idx, one)
        e[2].record()
        torch.cuda.synchronize(dev)
        best_c = max(best_c, 50 * 2 * 4 * n / (e[0].elapsed_time(e[1]) / 1e3) / 1e9)
        best_a = max(best_a, m / (e[1].elapsed_time(e[2]) / 1e3))
    return {"copy_gbs": best_c, "red_per_s": best_a,
            "how": "L2-resident torch copy of 32 MB (read + write bytes) and torch.index_add_ of "
                   "16M int64 ones into 4M cells, best of 5, this run"}


def cpu_model():
    """Host CPU model string and thread count (lscpu's model name, else platform)."""
    import platform
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.lower().startswith("model name"):
                name = line.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"model": name or platform.processor() or platform.machine(),
            "threads": os.cpu_count(), "machine": platform.machine()}


def max_over_ranks(v, world, device=None):
    """The maximum of v over all ranks (every rank's timed region ends at the slowest)."""
    if world <= 1:
        return float(v)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def weak_scaling_rate(world, packets_per_rank, steps, t_max_ms):
    """Whole-job packets/s: every rank ran its own batch in the same timed region."""
    return world * packets_per_rank * steps / (t_max_ms / 1e3)


def build_models(args, rank):
    """The rank's walker batch: independent walkers per rank (seed + 1000 rank), so the
    ranks shard the ensemble with no data-path collective."""
    from pdspy_gb300 import workloads
    if args.workload == "plain":
        args.models = 1
        return [workloads.small_disk()]
    if args.workload == "envelope":
        args.models = 1
        return [workloads.disk_envelope(nr=256, ntheta=256)]
    if args.workload == "spiral":
        args.models = 4
        rng = np.random.default_rng(args.seed + 1000 * rank)
        return [workloads.spiral_disk(nr=128, ntheta=128, nphi=128, mass=1e-4,
                                      phase=float(ph)) for ph in rng.uniform(0, 2 * np.pi, 4)]
    return workloads.walker_models(n=args.models, seed=args.seed + 1000 * rank)


def _cpu_walker(job):
    """One model of the workload through the CPU restatement, single-threaded (a worker of
    cpu_sample's process pool): returns (packets, events, longest walk)."""
    wl, nmodels, wseed, i, nphot, seed = job
    from tests import _cases  # CPU baseline leg only
    ns = argparse.Namespace(workload=wl, models=nmodels, seed=wseed)
    m = build_models(ns, 0)[i]
    r = _cases.run_oracle(m, nphot, seed=seed, model_id=i, nthreads=1, fp64_walls=True, **MRW)
    return nphot, r["stats"]["events"], r["stats"]["max_packet_events"]


def cpu_sample(models, args, threads, seed=None, packets=None, nmodels=None):
    """The CPU restatement (FP64-geometry build: native double precision is the fast choice
    on host cores) on the first nmodels models of the workload (all of them by default, so
    the sample has the workload's mix of light and heavy walkers) at ``packets`` packets
    each.  The models run in a spawn-started pool of ``threads`` single-threaded workers,
    the way pdspy's MPI pool spreads walkers over cores; a long walk occupies one core while
    the others go on.  Returns (packets/s, seconds, interactions, longest walk)."""
    import multiprocessing as mp
    seed = args.seed if seed is None else seed
    packets = args.cpu_packets if packets is None else packets
    nm = min(args.cpu_models if nmodels is None else nmodels, len(models))
    jobs = [(args.workload, args.models, args.seed, i, packets, seed) for i in range(nm)]
    jobs.sort(key=lambda j: -models[j[3]].grid.density[0].size)   # big grids first
    t0 = time.time()
    with mp.get_context("spawn").Pool(max(1, min(threads, nm))) as pool:
        res = pool.map(_cpu_walker, jobs, chunksize=1)
    dt = time.time() - t0
    pk = sum(r[0] for r in res)
    return pk / dt, dt, int(sum(r[1] for r in res)), int(max(r[2] for r in res))


def adjoint_rate(dev, seed, reps):
    """Gradients of an interferometric chi^2 per second (the adjoint workload): disk plus
    Ulrich envelope on 256 x 256 cells, 1.3 mm image of 256 x 256 pixels spanning +-1.2
    Rout at 140 pc, inclination uniform in [0, 80] deg, 20,000 uv points (baselines uniform
    in 10-2000 klambda, uniform position angle), data = model + N(0, 1 mJy).  One gradient
    = chi^2 and its derivatives w.r.t. every cell density (both species) and (Mdisk, h0,
    beta, gamma).  Temperatures are frozen (an analytic profile stands in for the thermal
    run: the cost of a gradient does not depend on the temperature values)."""
    import torch
    from pdspy_gb300 import adjoint, vis, workloads
    rng = np.random.default_rng(seed)
    m = workloads.disk_envelope(nr=256, ntheta=256)
    g = m.grid
    rr = np.meshgrid(g.r, g.theta, g.phi, indexing="ij")[0]
    g.temperature = [np.maximum(150.0 * rr ** -0.5, 10.0)] * len(g.density)
    incl = float(rng.uniform(0.0, 80.0))
    npix, dpc = 256, 140.0
    pixelsize = 2.4 * 100.0 / dpc / npix        # arcsec: +-1.2 Rout (100 au) across the field
    u, v = vis.synthetic_uv(20000, seed=seed)
    nuv = len(u)
    data = vis.UVData(u, v, np.zeros(nuv), np.zeros(nuv), np.full(nuv, 1.0 / 1e-3 ** 2))
    prob = adjoint.Chi2Problem(m, data, npix=npix, pixelsize=pixelsize, dpc=dpc, incl=incl,
                               device=dev)
    p_true = torch.tensor([1e-2, 0.1, 1.25, 1.0], dtype=torch.float64, device=dev)
    with torch.no_grad():
        re, im = prob.visibilities(prob.rho_from_params(p_true, 0.1, 100.0))
        noise = torch.as_tensor(rng.normal(0.0, 1e-3, (2, nuv)), device=dev)
        prob.re_d = re.double() + noise[0]
        prob.im_d = im.double() + noise[1]
    p = torch.tensor([8e-3, 0.11, 1.2, 0.9], dtype=torch.float64, device=dev)

    def one():
        pv = p.clone().requires_grad_(True)
        rho = prob.rho_from_params(pv, 0.1, 100.0)
        rho.retain_grad()
        chi = prob.chi2(rho)
        chi.backward()
        return chi, pv.grad, rho.grad

    for _ in range(3):
        one()
    torch.cuda.synchronize(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        chi, gp, gr = one()
    b.record()
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    return {"grads_per_s": 1e3 / ms, "ms_per_grad": ms, "unit": "gradients/s",
            "config": "disk+envelope 256x256 cells, 256x256 px at 1300 um, incl %.1f deg, "
                      "20000 uv points; d chi2 / d(every cell density, Mdisk, h0, beta, gamma)"
                      % incl, "chi2": float(chi.item()),
            "grad_params": [float(x) for x in gp.cpu()]}


def scattering_rate(dev, seed, reps=5, cpu=True):
    """Scattering Monte Carlo of an SED (the scattering-source workload): disk plus Ulrich
    envelope on 256 x 256 cells, 100 wavelengths log-spaced over 0.1-1e4 microns, 1e4
    packets per wavelength and mc_scat_maxtauabs = 5 (pdspy's run_sed call in
    run_disk_model.py), photons from the star and the dust (analytic temperatures).
    GPU packets/s by CUDA events; the CPU restatement on every tenth wavelength."""
    import torch
    from pdspy_gb300 import image, scatter, thermal, workloads
    m = workloads.disk_envelope(nr=256, ntheta=256)
    g = m.grid
    rr = np.meshgrid(g.r, g.theta, g.phi, indexing="ij")[0]
    g.temperature = [np.maximum(150.0 * rr ** -0.5, 10.0)] * len(g.density)
    lam = np.logspace(-1, 4, 100)
    nphot, mt = 10000, 5.0
    rho, T = image.model_state(m, dev)
    ka, ks = image.opacities(g, lam)
    emis = image.thermal_emissivity(rho, T, torch.as_tensor(ka, device=dev), lam)
    plan = scatter.ScatterPlan(g, lam, ka, ks, nphot, maxtauabs=mt, seed=seed, device=dev)
    for _ in range(3):
        plan.run(rho, emis)
    torch.cuda.synchronize(dev)
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        plan.run(rho, emis)
    b.record()
    torch.cuda.synchronize(dev)
    ms = a.elapsed_time(b) / reps
    st = plan.stats()
    out = {"gpu_packets_per_s": st["packets"] / (ms / 1e3), "ms_per_sed": ms,
           "packets_per_sed": st["packets"], "scatterings_per_sed": st["scatterings"],
           "config": "disk+envelope 256x256 cells, 100 wavelengths 0.1-1e4 um, 1e4 "
                     "packets each, maxtauabs 5, star + dust sources"}
    if cpu:
        from oracle import orc
        r, t, p = thermal.grid_arrays(g)
        radius, temp = thermal._stars(g)
        sel = np.arange(0, 100, 10)
        t0 = time.perf_counter()
        o = orc.mcscat(r, t, p, rho.float().cpu().numpy(), lam[sel], ka[:, sel], ks[:, sel],
                       radius, temp, nphot, emis=emis[sel].cpu().numpy(), maxtauabs=mt,
                       seed=seed)
        dt = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": o["stats"]["packets"] / dt, "unit": "packets/s",
                               "cores": os.cpu_count(), "kind": "port",
                               "sample": "every tenth wavelength (%d packets, %.2f s)" %
                                         (o["stats"]["packets"], dt)}
    return out


def lnprob_rate(dev, seed, nwalkers, nphot):
    """Batched lnprob of an emcee ensemble (the power-law disk family of pdspy's
    run_disk_model.py): walkers with log-uniform disk masses 1e-5..1e-3 Msun, h_0 in
    [0.05, 0.15], inclination in [20, 70] deg on run_disk_model's 99 x 100 grid; one
    visibility set of 20,000 points at 1.3 mm, 256^2-pixel images of 0.02 arcsec.  One
    evaluation = device densities, one batched thermal launch, an image and an FFT
    sampling per walker."""
    import torch
    from pdspy_gb300 import fitting, vis
    P = fitting.base_parameters()
    for k in ("h_0", "i", "logM_disk"):
        P[k]["fixed"] = False
    P["logR_disk"]["value"] = 1.5
    rng = np.random.default_rng(seed)
    walkers = np.stack([rng.uniform(0.05, 0.15, nwalkers), rng.uniform(20, 70, nwalkers),
                        rng.uniform(-5, -3, nwalkers)], axis=1)
    u, v = vis.synthetic_uv(20000, seed=seed, bmin_klam=10, bmax_klam=1500)
    data = vis.UVData(u, v, np.zeros(u.size), np.zeros(u.size), np.full(u.size, 1e6),
                      freq=2.99792458e10 / 0.13)
    sets = [dict(data=data, npix=256, pixelsize=0.02)]
    fitting.lnprob_batched(walkers[:2], sets, P, nphot=10000, device=dev, seed=seed)
    torch.cuda.synchronize(dev)
    t0 = time.perf_counter()
    lp = fitting.lnprob_batched(walkers, sets, P, nphot=nphot, device=dev, seed=seed)
    torch.cuda.synchronize(dev)
    dt = time.perf_counter() - t0
    return {"walkers": nwalkers, "packets_per_walker": nphot, "s": dt,
            "lnprob_per_s": nwalkers / dt, "finite": int(np.isfinite(lp).sum())}


def vis_rate(dev, seed):
    """Visibility sampling of a 1024^2 image (0.01 arcsec pixels) at 1e5 uv points up to
    5000 klambda: the gridded FFT path (pad 2, cuFFT + bilinear sampling) against the
    direct sum, both on the GPU; forward only."""
    import torch
    from pdspy_gb300 import vis
    n, nuv = 1024, 100000
    rng = np.random.default_rng(seed)
    x = (np.arange(n) - n // 2) * 0.01
    img = np.exp(-0.5 * (x[None, :] ** 2 + x[:, None] ** 2) / 0.3 ** 2)
    img = torch.as_tensor(img, dtype=torch.float32, device=dev)
    u, v = vis.synthetic_uv(nuv, seed=seed, bmin_klam=10, bmax_klam=5000)
    u = torch.as_tensor(u, dtype=torch.float32, device=dev)
    v = torch.as_tensor(v, dtype=torch.float32, device=dev)
    geo = vis.pixel_grid(n, 0.01)
    out = {"npix": n, "points": nuv, "pad": 2}
    for name, fn in (("fft", lambda: vis.VisFFT.apply(img, u, v, geo, 2)),
                     ("dft", lambda: vis.VisDFT.apply(img, u, v, geo))):
        fn()
        torch.cuda.synchronize(dev)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(3):
            re, im = fn()
        b.record()
        torch.cuda.synchronize(dev)
        out[name + "_ms"] = a.elapsed_time(b) / 3
        out[name] = (re, im)
    re_f, im_f = out.pop("fft")
    re_d, im_d = out.pop("dft")
    scale = float(torch.sqrt(re_d ** 2 + im_d ** 2).max())
    out["max_abs_diff_rel"] = float(torch.maximum((re_f - re_d).abs(), (im_f - im_d).abs()).max()) / scale
    return out


def workload_name(args):
    if args.workload == "plain":
        return "plain-disk-100x100-%g-packets-mrw" % args.packets
    if args.workload == "envelope":
        return "disk-envelope-256x256-%g-packets-mrw" % args.packets
    if args.workload == "spiral":
        return "spiral-3d-128^3-two-populations-4-phases-%g-packets-each-mrw" % args.packets
    return "batched-%d-walker-disks-%g-packets-each-mrw" % (args.models, args.packets)


def run_reference(args, world, rank):
    if rank != 0:
        return
    threads = os.cpu_count()
    models = build_models(args, 0)
    # warm-up: page the library and the interpreter in on a small sample (one model)
    for _ in range(args.warmup):
        cpu_sample(models, args, threads, packets=2000, nmodels=1)
    full = args.cpu_full
    packets = args.packets if full else args.cpu_packets
    nm = len(models) if full else min(args.cpu_models, len(models))
    times, events, longest = [], [], []
    for k in range(args.steps):
        # step k uses Monte Carlo seed seed + k, as the GPU arm's step k does
        v, dt, ev, lw = cpu_sample(models, args, threads, seed=args.seed + k, packets=packets,
                                   nmodels=nm)
        times.append(dt)
        events.append(ev)
        longest.append(lw)
    value = float(nm * packets * args.steps / np.sum(times))
    sample = ("%d models x %d packets (%s the %d x %g workload), CPU restatement (FP64 "
              "geometry), %d single-threaded workers" % (nm, packets, "all of" if full else
                                                          "a sample of", args.models,
                                                          args.packets, threads))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "packets/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(times) * 1e3), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic",
            "config": {"workload": workload_name(args), "sample": sample},
            "cpu_baseline": {"value": value, "unit": "packets/s", "cores": threads,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "packets/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0},
            "interactions": {"per_s": float(np.sum(events) / np.sum(times)),
                             "longest_walk": longest},
            "seeds": {"mc_seeds": [args.seed + k for k in range(args.steps)],
                      "ms_per_step": [round(t * 1e3, 1) for t in times]},
            "host_cpu": cpu_model()}
    print(json.dumps(line), flush=True)


def main():
    args = parse()
    world, rank, local = dist_setup()
    if args.impl == "reference":
        run_reference(args, world, rank)
        return
    import torch
    import torch.distributed as dist
    from pdspy_gb300 import thermal
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl")
    dev = torch.device("cuda", local)
    models = build_models(args, rank)
    # one plan per timed step: step k runs the same models with Monte Carlo seed seed + k, so
    # the steps sample the heavy tail of the walk lengths instead of repeating one draw
    plans = [thermal.ThermalPlan([m.grid for m in models], args.packets, seed=args.seed + k,
                                 time_launches=True, timelimit=args.timelimit, **MRW)
             for k in range(max(args.steps, 1))]
    plan = plans[0]
    host_rho = torch.from_numpy(np.concatenate(
        [thermal.stack_density(m.grid).reshape(-1) for m in models])).pin_memory()
    rho, T = plan.new_buffers()
    rho.copy_(host_rho)
    host_T = torch.empty(T.shape, dtype=T.dtype, pin_memory=True)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)  # > L2 (129 MB)
    total_packets = args.models * args.packets
    stream = torch.cuda.current_stream(dev)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    # Warm-up: the same plan and kernels, each run cut at a short device deadline (the
    # longest packet walk of this workload alone takes minutes; warm-up only has to load
    # the modules and settle clocks and caches).
    plan.set_timelimit(args.warmup_deadline)
    for _ in range(args.warmup):
        plan.run(rho, T)
        torch.cuda.synchronize(dev)
    plan.set_timelimit(args.timelimit)

    # Timed steps.  Per step, on the run's stream: event a, pinned host -> device copy of the
    # densities, event b, the thermal run, event c, device -> pinned host copy of the
    # temperatures, event d.  value uses b..c (inputs resident in HBM), e2e uses a..d.
    step_ms, e2e_ms, launch_ms, launch_stats, stats = [], [], [], [], []
    launch_counts = []
    with Clocks(local) as clk:
        for k in range(args.steps):
            plan = plans[k]
            flush.zero_()
            barrier()
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
            ev[0].record(stream)
            rho.copy_(host_rho, non_blocking=True)
            ev[1].record(stream)
            plan.run(rho, T)
            ev[2].record(stream)
            host_T.copy_(T, non_blocking=True)
            ev[3].record(stream)
            barrier()
            step_ms.append(ev[1].elapsed_time(ev[2]))
            e2e_ms.append(ev[0].elapsed_time(ev[3]))
            launch_ms.append(plan.launch_ms())
            launch_stats.append(plan.launch_stats())
            launch_counts.append(plan.launch_counts())
            stats.append(plan.check_status())

    # per step: the warp-per-packet stage (the last launch: the longest walks) and
    # everything before it
    tail_ms = [lm[-1] if lm else 0.0 for lm in launch_ms]
    bulk_ms = [a - b for a, b in zip(step_ms, tail_ms)]
    seeds = {"mc_seeds": [args.seed + k for k in range(args.steps)],
             "ms_per_step": [round(x, 1) for x in step_ms],
             "median_ms": float(np.median(step_ms)), "min_ms": float(np.min(step_ms)),
             "max_ms": float(np.max(step_ms)),
             "bulk_ms": [round(x, 1) for x in bulk_ms],
             "tail_ms": [round(x, 1) for x in tail_ms],
             "longest_walk": [max([b for (_, b, _) in ls] or [0]) for ls in launch_stats],
             "events": [int(st_["events"]) for st_ in stats]}
    t_max = max_over_ranks(float(np.sum(step_ms)), world, dev)
    te = max_over_ranks(float(np.sum(e2e_ms)), world, dev)
    value = weak_scaling_rate(world, total_packets, args.steps, t_max)
    e2e = {"value": weak_scaling_rate(world, total_packets, args.steps, te), "unit": "packets/s",
           "h2d_bytes_per_step": int(host_rho.numel() * 4),
           "d2h_bytes_per_step": int(host_T.numel() * 8)}

    # roofline of the walk launches (transport and continuation kernels)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    peak = float(peaks.get("hbm_gbs", 6800.0))
    st = stats[-1]
    ns = plan.nspec
    alg_bytes = (st["crossings"] * 4 * ns + (st["absorptions"] + st["mrw_steps"] * ns) * 8 +
                 (st["absorptions"] + st["mrw_steps"]) * 4)
    lm = [x for x in launch_ms[-1] if x > 0]
    n_launch = max(len(lm), 1)
    avg_launch = float(np.sum(lm)) / n_launch
    traffic = None
    tf = os.path.join(ROOT, "profiles", "mc_transport_traffic.json")
    if os.path.exists(tf):
        try:
            traffic = json.load(open(tf)).get("dram_bytes_per_launch")
        except Exception:
            traffic = None
    events_all = float(np.sum([st_["events"] for st_ in stats]))
    t_bulk = max_over_ranks(float(np.sum(bulk_ms)), world, dev)
    interactions = {"per_s": world * events_all / (t_max / 1e3),
                    "bulk_per_s": world * events_all / (t_bulk / 1e3) if t_bulk > 0 else None,
                    "note": "interactions (absorptions, scatterings, MRW steps) per second over the "
                            "timed steps; bulk_per_s divides by the time before the "
                            "warp-per-packet stage"}
    # per launch of the last step: algorithmic bytes = 4 nspec B per crossing (densities)
    # + 8 B per deposit (int64 atomic) + 4 B per reemission (temperature snapshot)
    lc = launch_counts[-1]

    def alg(d):
        return 4 * ns * d["crossings"] + 12 * d["deposits"]

    tail = lc[-1] if lc else None
    bulk = lc[:-1]
    t_bulk_k = sum(d["ms"] for d in bulk) / 1e3
    dominant = max(lc, key=lambda d: d["ms"]) if lc else None
    sm_mhz = 2070.0
    roofline = {"bound": "hbm", "peak": peak, "unit": "GB/s",
                "peak_source": "measured" if peaks else "fallback",
                "kernel": "mc_continue_kernel (the warp-per-packet stage: the longest walks, "
                          "%.0f%% of the last step)" % (100 * tail["ms"] / step_ms[-1])
                          if tail and dominant is tail else "mc_transport_kernel",
                "traffic": traffic,
                "traffic_source": "null: the walk kernels' working set (densities, snapshots, "
                                  "deposits) stays in L2; profiles/ holds the ncu DRAM bytes",
                "launches_per_step": n_launch,
                "walk_kernel_ms_last_step": float(np.sum(lm)),
                "algorithmic_bytes_last_step": int(sum(alg(d) for d in lc))}
    if dominant is not None:
        a_dom = alg(dominant) / (dominant["ms"] / 1e3) / 1e9
        roofline.update(achieved=a_dom, frac=a_dom / peak)
        if dominant is tail and tail["longest"] > 0:
            # the stage lasts as long as its longest walk, one interaction after another
            roofline["cycles_per_interaction_longest_walk"] = (
                tail["ms"] * 1e-3 * sm_mhz * 1e6 / tail["longest"])
            roofline["latency_note"] = ("the stage is one dependent chain per packet and lasts "
                                        "as long as the longest walk: the bound is the latency "
                                        "of one interaction, not a memory or issue roof")
    l2 = l2_roofs(dev) if rank == 0 else None
    if l2 and t_bulk_k > 0:
        ab = sum(alg(d) for d in bulk) / t_bulk_k / 1e9
        at = sum(d["deposits"] for d in bulk) / t_bulk_k
        roofline["bulk"] = {"kernel": "mc_transport_kernel (pilot, epoch and first continuation "
                                      "launches) with the epochs' drained walks "
                                      "(mc_continue_kernel)",
                            "l2_achieved_gbs": ab, "l2_peak_gbs": l2["copy_gbs"],
                            "l2_frac": ab / l2["copy_gbs"], "atomics_per_s": at,
                            "atomic_peak_per_s": l2["red_per_s"],
                            "atomic_frac": at / l2["red_per_s"],
                            "interactions_per_s": sum(d["events"] for d in bulk) / t_bulk_k,
                            "peaks_source": l2["how"]}

    adj = None
    if rank == 0 and not args.no_adjoint:
        adj = adjoint_rate(dev, args.seed, args.adjoint_reps)

    scat = None
    if rank == 0 and not args.no_scattering:
        scat = scattering_rate(dev, args.seed, cpu=not args.no_cpu)

    vrate = None
    if rank == 0 and not args.no_adjoint:
        vrate = vis_rate(dev, args.seed)

    lnp = None
    if rank == 0 and args.lnprob_walkers > 0:
        lnp = lnprob_rate(dev, args.seed, args.lnprob_walkers, args.lnprob_packets)

    cpu = None
    if rank == 0 and not args.no_cpu:
        v, dt, ev, lw = cpu_sample(models, args, os.cpu_count())
        cpu = {"value": v, "unit": "packets/s", "cores": os.cpu_count(), "kind": "port",
               "interactions_per_s": ev / dt, "longest_walk": lw,
               "sample": "%d models x %d packets of the workload (Monte Carlo seed %d), CPU "
                         "restatement in %d single-threaded workers (%.1f s)" %
               (min(args.cpu_models, len(models)), args.cpu_packets, args.seed,
                os.cpu_count(), dt)}

    K, P = plan.opts.nepoch, plan.opts.npilot
    # start + a prep per pass and epoch + the transport launches (each pass and epoch, its
    # drained walks one per warp, the two continuation launches) + temperature + finish
    launches_per_step = st["launches"] + K + P + 3
    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": "packets/s", "n_gpus": world,
                "steps": args.steps, "warmup": args.warmup,
                "ms_per_step": t_max / args.steps, "higher_is_better": True, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic",
                "config": {"workload": workload_name(args), "models_per_gpu": args.models,
                           "packets_per_model": args.packets, "mrw": True, "nepoch": K,
                           "npilot": P, "late_after": int(plan.opts.late_after),
                           "l2": "256 MB buffer written between timed steps",
                           "warmup": "same plan, each run cut at a %g s device deadline" %
                                     args.warmup_deadline,
                           "geometry": "double-single (FP32 pipe); FP64 energy->temperature",
                           "parallelism": "replicas: independent walker batches per GPU"},
                "e2e": e2e, "roofline": roofline, "cpu_baseline": cpu, "adjoint": adj,
                "scattering": scat, "lnprob": lnp, "visibility_sampling": vrate,
                "clocks": clk.summary(), "gpu_launches": launches_per_step * args.steps,
                "seeds": seeds, "interactions": interactions, "host_cpu": cpu_model(),
                "stats": {k: st[k] for k in ("events", "crossings", "absorptions", "mrw_steps",
                                            "parked", "drained", "killed", "late_units")},
                "launch_ms": [round(x, 3) for x in launch_ms[-1]],
                "launch_longest_walk": [b for (_, b, _) in launch_stats[-1]]}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
