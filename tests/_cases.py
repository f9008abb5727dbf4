"""Shared helpers: build small models and run the oracle on exactly the inputs the GPU
path receives."""
import numpy as np

from oracle import orc
from pdspy_gb300 import thermal, workloads


def oracle_inputs(model):
    g = model.grid
    r, t, p = thermal.grid_arrays(g)
    ka, ks, gg = [], [], []
    for d in g.dust:
        a, s, gv = thermal.opacity_on_grid(d, g.lam)
        ka.append(a); ks.append(s); gg.append(np.zeros_like(a) if gv is None else gv)
    sr, st = thermal._stars(g)
    rho = thermal.stack_density(g)
    return dict(r_edges=r, th_edges=t, ph_edges=p, rho=rho, lam_um=np.asarray(g.lam, float),
                kabs=np.stack(ka), ksca=np.stack(ks), g=np.stack(gg), star_radius=sr,
                star_temp=st)


def run_oracle(model, nphot, **kw):
    """Oracle run with the product's defaults for the epoch schedule."""
    for k in ("nepoch", "npilot", "late_after", "mrw_eager_after"):
        kw.setdefault(k, thermal.DEFAULTS[k])
    return orc.mctherm(nphot=nphot, **oracle_inputs(model), **kw)


def case(name):
    """Small models that exercise each branch of the walk."""
    if name == "disk_full":        # theta over [0, pi], HG scattering
        return workloads.small_disk(nr=24, ntheta=24, mass=1e-5, g=0.6), {}
    if name == "disk_mirror":      # theta over [0, pi/2], mirrored about the midplane
        return workloads.small_disk(nr=20, ntheta=12, mass=1e-5, theta_max=np.pi / 2, g=0.0), {}
    if name == "two_species_mrw":  # disk + envelope, modified random walk on
        m = workloads.disk_envelope(nr=24, ntheta=24, mdisk=1e-3, menv=0.01, renv=1000.0)
        return m, dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=5)
    if name == "spiral_3d":        # phi walls, two species
        return workloads.spiral_disk(nr=12, ntheta=12, nphi=12, mass=1e-5), {}
    if name == "parked":           # packets parked after 40 events, resumed at the end
        m = workloads.small_disk(nr=24, ntheta=24, mass=1e-3, g=0.6)
        return m, dict(late_after=40, mrw=True, mrw_count_trigger=20)
    if name == "parked_mrw2":      # two species, eager MRW in the resumed walks
        m = workloads.disk_envelope(nr=20, ntheta=20, mdisk=3e-3, menv=0.01, renv=1000.0)
        return m, dict(late_after=30, mrw=True, mrw_count_trigger=8, mrw_eager_after=60)
    raise KeyError(name)


def image_model(kind="disk", nr=16, ntheta=16, nphi=1, mass=1e-3, lam=None):
    """Small model with an analytic temperature (T = 150 K (r/au)^-0.5 per species)."""
    import numpy as np
    if kind == "disk":
        m = workloads.small_disk(nr=nr, ntheta=ntheta, mass=mass, lam_um=lam)
    elif kind == "mirror":
        m = workloads.small_disk(nr=nr, ntheta=ntheta, mass=mass, theta_max=np.pi / 2, lam_um=lam)
    elif kind == "spiral":
        m = workloads.spiral_disk(nr=nr, ntheta=ntheta, nphi=nphi, mass=mass)
    elif kind == "envelope":
        m = workloads.disk_envelope(nr=nr, ntheta=ntheta, mdisk=mass, menv=0.01, renv=1000.0)
    else:
        raise KeyError(kind)
    g = m.grid
    rr = np.meshgrid(g.r, g.theta, g.phi, indexing="ij")[0]
    T = 150.0 * rr ** -0.5
    g.temperature = [T * (1.0 + 0.1 * i) for i in range(len(g.density))]
    return m


def _pool_run(args):
    """One single-threaded oracle run (worker of oracle_ensemble): (temperature, crossings)."""
    builder, bkw, nphot, seed, kw = args
    from pdspy_gb300 import workloads as w
    m = getattr(w, builder)(**bkw)
    r = run_oracle(m, nphot, seed=seed, crossings=True, nthreads=1, **kw)
    return r["temperature"], r["crossings"]


def oracle_ensemble(builder, bkw, nphot, seeds, workers=8, **kw):
    """Oracle runs of workloads.<builder>(**bkw) for each seed, in a spawn-started process
    pool.  Returns (temperatures [seed][spec][nr][nt][np], summed crossings)."""
    import multiprocessing as mp
    args = [(builder, bkw, nphot, int(s), kw) for s in seeds]
    with mp.get_context("spawn").Pool(min(workers, len(args))) as pool:
        res = pool.map(_pool_run, args)
    return np.array([r[0] for r in res]), np.sum([r[1] for r in res], axis=0)


def four_sigma(T_a, T_b, crossings, min_crossings=1000):
    """Per-cell comparison of two ensembles (spec criterion): z = difference of the
    seed means over its standard error, on cells crossed >= min_crossings times per run with
    a positive mean temperature in both ensembles.  Returns (z, relative difference of the
    means) on those cells."""
    na, nb = len(T_a), len(T_b)
    ma, mb = T_a.mean(0), T_b.mean(0)
    sig = np.sqrt(T_a.var(0, ddof=1) / na + T_b.var(0, ddof=1) / nb)
    C = np.broadcast_to(crossings / na, ma.shape)
    sel = (C >= min_crossings) & (ma > 0) & (mb > 0) & (sig > 0)
    return (ma - mb)[sel] / sig[sel], (ma - mb)[sel] / mb[sel]
