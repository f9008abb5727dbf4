"""Thermal Monte Carlo behind ``Model.run_thermal(code="gb300")``.

Replaces pdspy's radmc3d branch (pdspy/modeling/Model.py:221-256): instead of writing
RADMC-3D input files (Model.py:723-825), running ``radmc3d mctherm`` in a subprocess
(pdspy/radmc3d/run.py:9-38) and parsing ``dust_temperature.dat``
(pdspy/radmc3d/read.pyx:433-478), the grid, densities and opacities go to device
buffers and one plan runs the transport on the GPU.  The result lands in
``grid.temperature`` exactly as the reference leaves it: a list with one float64 array
of shape (nr, ntheta, nphi) per dust species, in K.

Keywords follow ``radmc3d.write.control`` (pdspy/radmc3d/write.py:1-146):
``modified_random_walk``, ``mrw_gamma``, ``mrw_tauthres``, ``mrw_count_trigger`` and
``iseed`` are honoured; ``timelimit`` becomes a device-side deadline and a run that
reaches it raises ``subprocess.TimeoutExpired`` like the reference's subprocess call;
``setthreads``, ``nice`` and ``verbose`` are accepted and have no effect on the GPU.
"""
import ctypes as C
import subprocess
import warnings

import numpy as np
import torch

from . import _lib
from .constants import AU, R_sun

_IGNORED = {"setthreads", "nice", "verbose", "nphot_scat", "nphot_spec", "incl_dust",
            "camera_scatsrc_allfreq", "mc_scat_maxtauabs", "writeimage_unformatted",
            "scattering_mode_max", "istar_sphere", "itempdecoup"}

DEFAULTS = dict(nepoch=8, npilot=2, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100,
                max_interactions=2_000_000_000, late_after=100000, mrw_eager_after=10000)


def _dptr(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def opacity_on_grid(dust, lam_um):
    """kabs, ksca, g of one pdspy Dust object on the model wavelength grid (microns).

    pdspy hands RADMC-3D the dust table on its own wavelength grid (write.dustkappa,
    pdspy/radmc3d/write.py:316-342) and RADMC-3D maps it onto the global grid.  Here the
    map is a log-log linear interpolation with power-law extrapolation from the end
    segments; when the two grids coincide the values pass through unchanged.
    """
    lam_d = np.asarray(dust.lam, dtype=np.float64) * 1.0e4
    kabs = np.asarray(dust.kabs, dtype=np.float64)
    ksca = np.asarray(dust.ksca, dtype=np.float64)
    g = getattr(dust, "g", None)
    g = None if g is None else np.broadcast_to(np.asarray(g, dtype=np.float64), kabs.shape)
    lam_um = np.asarray(lam_um, dtype=np.float64)
    order = np.argsort(lam_d)
    lam_d, kabs, ksca = lam_d[order], kabs[order], ksca[order]
    if g is not None:
        g = np.asarray(g)[order]
    if lam_d.shape == lam_um.shape and np.allclose(lam_d, lam_um, rtol=1e-10, atol=0):
        return kabs.copy(), ksca.copy(), None if g is None else g.copy()

    def loglog(y):
        x = np.log(lam_d)
        yy = np.log(np.maximum(y, 1e-300))
        xi = np.log(lam_um)
        out = np.interp(xi, x, yy)
        lo = xi < x[0]
        hi = xi > x[-1]
        if lo.any():
            sl = (yy[1] - yy[0]) / (x[1] - x[0])
            out[lo] = yy[0] + sl * (xi[lo] - x[0])
        if hi.any():
            sl = (yy[-1] - yy[-2]) / (x[-1] - x[-2])
            out[hi] = yy[-1] + sl * (xi[hi] - x[-1])
        res = np.exp(out)
        res[np.interp(xi, x, (y > 0).astype(float)) < 0.5] = 0.0
        return res

    gi = None if g is None else np.interp(np.log(lam_um), np.log(lam_d), g)
    return loglog(kabs), loglog(ksca), gi


def _same_dust(a, b):
    if len(a.dust) != len(b.dust) or not np.array_equal(np.asarray(a.lam), np.asarray(b.lam)):
        return False
    for da, db in zip(a.dust, b.dust):
        if da is db:
            continue
        for attr in ("lam", "kabs", "ksca"):
            if not np.array_equal(np.asarray(getattr(da, attr)), np.asarray(getattr(db, attr))):
                return False
    return True


class _Keep:
    def __init__(self):
        self.items = []

    def __call__(self, a):
        a = np.ascontiguousarray(a, dtype=np.float64)
        self.items.append(a)
        return a


def grid_arrays(grid):
    """(r_edges_cm, theta_edges, phi_edges) of a pdspy spherical Grid."""
    if getattr(grid, "coordsystem", "spherical") != "spherical":
        raise ValueError("the gb300 backend supports spherical grids only (got %r)"
                         % grid.coordsystem)
    return (np.asarray(grid.w1, dtype=np.float64) * AU, np.asarray(grid.w2, dtype=np.float64),
            np.asarray(grid.w3, dtype=np.float64))


def _stars(grid):
    if len(grid.stars) == 0:
        raise ValueError("run_thermal needs at least one star (Grid.add_star)")
    for s in grid.stars:
        if abs(getattr(s, "x", 0.0)) + abs(getattr(s, "y", 0.0)) + abs(getattr(s, "z", 0.0)) > 0:
            raise ValueError("the gb300 backend places stars at the origin only")
    return (np.array([s.radius * R_sun for s in grid.stars], dtype=np.float64),
            np.array([s.temperature for s in grid.stars], dtype=np.float64))


def stack_density(grid):
    """Densities of all species as one float32 array [nspec, nr, ntheta, nphi]."""
    return np.ascontiguousarray(np.stack([np.asarray(d, dtype=np.float64) for d in grid.density])
                                .astype(np.float32))


class ThermalPlan:
    """A prepared thermal run for one model or a batch of models with the same dust.

    The plan owns a device workspace and the constant tables uploaded into it.  ``run``
    enqueues the whole epoch schedule on the current CUDA stream and can be captured in a
    CUDA graph (``capture``) and replayed with new densities written in place.
    """

    def __init__(self, grids, nphot, seed=0, nepoch=DEFAULTS["nepoch"], npilot=DEFAULTS["npilot"],
                 mrw=False, mrw_gamma=DEFAULTS["mrw_gamma"],
                 mrw_tauthres=DEFAULTS["mrw_tauthres"],
                 mrw_count_trigger=DEFAULTS["mrw_count_trigger"],
                 max_interactions=DEFAULTS["max_interactions"], late_after=DEFAULTS["late_after"],
                 mrw_eager_after=DEFAULTS["mrw_eager_after"], timelimit=None, device=None,
                 block_threads=0, blocks_per_sm=0, abort_flag=None, time_launches=False,
                 fp64_walls=False, drain_below=0):
        if not isinstance(grids, (list, tuple)):
            grids = [grids]
        self.L = _lib.lib()
        self.device = torch.device("cuda", torch.cuda.current_device() if device is None
                                   else torch.device(device).index or 0)
        nphot = np.broadcast_to(np.asarray(nphot, dtype=np.int64), (len(grids),))
        g0 = grids[0]
        for g in grids[1:]:
            if not _same_dust(g0, g):
                raise ValueError("a batched plan needs the same dust and wavelength grid in "
                                 "every model")
        keep = _Keep()
        self.shapes = []
        descs = (_lib.ModelDesc * len(grids))()
        for i, g in enumerate(grids):
            r, t, p = grid_arrays(g)
            sr, st = _stars(g)
            r, t, p, sr, st = keep(r), keep(t), keep(p), keep(sr), keep(st)
            descs[i] = _lib.ModelDesc(len(r) - 1, len(t) - 1, len(p) - 1, _dptr(r), _dptr(t),
                                      _dptr(p), len(sr), _dptr(sr), _dptr(st), int(nphot[i]))
            self.shapes.append((len(g.density), len(r) - 1, len(t) - 1, len(p) - 1))
            if len(g.density) != len(g0.density):
                raise ValueError("every model of a batch needs the same number of species")
        lam = keep(np.asarray(g0.lam, dtype=np.float64))
        ka, ks, gg = [], [], []
        any_g = False
        for d in g0.dust:
            a, s, g = opacity_on_grid(d, lam)
            ka.append(a); ks.append(s); gg.append(np.zeros_like(a) if g is None else g)
            any_g = any_g or g is not None
        ka, ks, gg = keep(np.stack(ka)), keep(np.stack(ks)), keep(np.stack(gg))
        dust = _lib.DustDesc(len(lam), ka.shape[0], _dptr(lam), _dptr(ka), _dptr(ks),
                             _dptr(gg) if any_g else None)
        self.nlam = len(lam)
        self.nspec = ka.shape[0]
        deadline = 0 if not timelimit else int(float(timelimit) * 1e9)
        self.opts = _lib.McOptions(int(seed) & 0xFFFFFFFFFFFFFFFF, int(nepoch), int(npilot),
                                   int(bool(mrw)), float(mrw_gamma), float(mrw_tauthres),
                                   int(mrw_count_trigger), int(max_interactions), deadline,
                                   abort_flag, int(block_threads), int(blocks_per_sm),
                                   int(late_after), int(bool(time_launches)),
                                   int(mrw_eager_after), int(bool(fp64_walls)),
                                   int(drain_below))
        self.timelimit = timelimit
        self._plan = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.L.pdgpu_mc_plan_create(len(grids), descs, C.byref(dust),
                                                   C.byref(self.opts), C.byref(self._plan)),
                       "pdgpu_mc_plan_create")
            self.layout = _lib.McLayout()
            _lib.check(self.L.pdgpu_mc_plan_layout(self._plan, C.byref(self.layout)),
                       "pdgpu_mc_plan_layout")
            self.workspace = torch.empty(self.layout.total_bytes, dtype=torch.uint8,
                                         device=self.device)
            stream = torch.cuda.current_stream(self.device)
            _lib.check(self.L.pdgpu_mc_plan_upload(self._plan, self.workspace.data_ptr(),
                                                   self.layout.total_bytes, stream.cuda_stream),
                       "pdgpu_mc_plan_upload")
        self.nmodels = len(grids)
        self.total_cells = int(self.layout.total_cells)
        self.nphot = nphot.copy()

    def __del__(self):
        try:
            if self._plan:
                self.L.pdgpu_mc_plan_destroy(self._plan)
                self._plan = C.c_void_p()
        except Exception:
            pass

    # -- device views -----------------------------------------------------------------
    def energy_main(self):
        """int64 energy absorbed in the first late_after events of each packet (the part
        that feeds later epochs), in units of 2^-20 packet energies."""
        o = self.layout.energy_offset
        return self.workspace[o:o + 8 * self.total_cells].view(torch.int64)

    def energy_late(self):
        """int64 energy absorbed after a packet's first late_after events."""
        o = self.layout.late_offset
        return self.workspace[o:o + 8 * self.total_cells].view(torch.int64)

    def energy(self):
        """Total int64 absorbed energy per cell (main + late)."""
        return self.energy_main() + self.energy_late()

    def escape(self):
        o = self.layout.escape_offset
        return self.workspace[o:o + 8 * self.nmodels * self.nlam].view(torch.int64).view(
            self.nmodels, self.nlam)

    def raw_stats(self):
        o = self.layout.stats_offset
        return self.workspace[o:o + 8 * 256].view(torch.int64)

    def launch_stats(self):
        """Per transport launch: (duration ms, longest packet in events, parked packets)."""
        return [(d["ms"], d["longest"], d["parked"]) for d in self.launch_counts()]

    def launch_counts(self):
        """Per transport launch of the last run: device-clock duration (ms), longest packet
        (events), packets parked, interactions, crossings and deposits."""
        r = self.raw_stats().cpu().numpy()
        out = []
        for l in range(24):
            t0, t1, mx, pk, ev, cr, dep = r[32 + 8 * l: 39 + 8 * l]
            if t1 > 0 and t0 < (1 << 62):
                out.append(dict(ms=(t1 - t0) / 1e6, longest=int(mx), parked=int(pk),
                                events=int(ev), crossings=int(cr), deposits=int(dep)))
        return out

    def set_timelimit(self, seconds):
        """Device-clock budget (s) of the following runs; None or 0 removes it."""
        ns = 0 if not seconds else int(float(seconds) * 1e9)
        _lib.check(self.L.pdgpu_mc_plan_set_deadline(self._plan, ns), "pdgpu_mc_plan_set_deadline")
        self.timelimit = seconds

    def set_model_timelimits(self, seconds):
        """Per-model device-clock budgets (s) of the following runs: a sequence with one entry
        per model (None or 0: no limit), one number for every model, or None to clear.  A
        model that has not finished in time stops with status 2 (timeout) and the others
        finish unchanged (run_disk_model.py:251-273 times out each walker on its own)."""
        if seconds is None:
            arr = None
        else:
            sec = np.broadcast_to(np.asarray([0.0 if x is None else float(x) for x in
                                              np.atleast_1d(np.asarray(seconds, dtype=object))]),
                                  (self.nmodels,))
            arr = np.ascontiguousarray(np.round(sec * 1e9).astype(np.int64))
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.L.pdgpu_mc_plan_set_model_deadlines(
            self._plan, None if arr is None else arr.ctypes.data, stream.cuda_stream),
            "pdgpu_mc_plan_set_model_deadlines")

    def model_status(self):
        """Status of every model after the last run: int32 array (0 ok, 2 timed out)."""
        out = np.zeros(self.nmodels, dtype=np.int32)
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.L.pdgpu_mc_plan_model_status(self._plan, self.workspace.data_ptr(),
                                                     stream.cuda_stream, out.ctypes.data),
                   "pdgpu_mc_plan_model_status")
        return out

    def launch_ms(self):
        """CUDA-event durations (ms) of the last run's transport launches."""
        buf = (C.c_float * 32)()
        n = self.L.pdgpu_mc_plan_launch_ms(self._plan, buf, 32)
        return [float(buf[i]) for i in range(n)]

    def new_buffers(self):
        rho = torch.empty(self.total_cells, dtype=torch.float32, device=self.device)
        T = torch.empty(self.total_cells, dtype=torch.float64, device=self.device)
        return rho, T

    # -- execution ---------------------------------------------------------------------
    def run(self, rho, T):
        """Enqueue one run on the current stream: rho float32 [cells] -> T float64."""
        assert rho.dtype == torch.float32 and T.dtype == torch.float64
        assert rho.numel() == self.total_cells and T.numel() == self.total_cells
        assert rho.is_contiguous() and T.is_contiguous()
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.L.pdgpu_mc_plan_run(self._plan, rho.data_ptr(), T.data_ptr(),
                                            self.workspace.data_ptr(), self.layout.total_bytes,
                                            stream.cuda_stream), "pdgpu_mc_plan_run")
        return T

    def capture(self, rho, T):
        """Capture ``run(rho, T)`` in a CUDA graph; replay it after updating rho in place."""
        g = torch.cuda.CUDAGraph()
        s = torch.cuda.Stream(self.device)
        s.wait_stream(torch.cuda.current_stream(self.device))
        with torch.cuda.stream(s):
            self.run(rho, T)  # warm-up outside capture (kernel attributes, lazy loading)
        torch.cuda.current_stream(self.device).wait_stream(s)
        torch.cuda.synchronize(self.device)
        with torch.cuda.graph(g):
            self.run(rho, T)
        return g

    def stats(self):
        st = _lib.McStats()
        stream = torch.cuda.current_stream(self.device)
        _lib.check(self.L.pdgpu_mc_plan_stats(self._plan, self.workspace.data_ptr(),
                                              stream.cuda_stream, C.byref(st)),
                   "pdgpu_mc_plan_stats")
        return st.asdict()

    def check_status(self, stats=None):
        stats = self.stats() if stats is None else stats
        status = stats["status"]
        if status == 2:
            raise subprocess.TimeoutExpired("gb300 mctherm", self.timelimit)
        if status != 0:
            raise _lib.PdgpuError(status, "thermal run")
        return stats

    def split(self, T):
        """Per-model list of per-species float64 numpy arrays (nr, ntheta, nphi)."""
        Th = T.detach().cpu().numpy() if isinstance(T, torch.Tensor) else np.asarray(T)
        out, o = [], 0
        for (ns, nr, nt, np_) in self.shapes:
            n = ns * nr * nt * np_
            a = Th[o:o + n].reshape(ns, nr, nt, np_)
            out.append([np.array(a[s], dtype=np.float64) for s in range(ns)])
            o += n
        return out


def _options(keywords):
    kw = dict(keywords)
    opts = {}
    if "iseed" in kw:
        opts["seed"] = int(kw.pop("iseed"))
    if "seed" in kw:
        opts["seed"] = int(kw.pop("seed"))
    if "modified_random_walk" in kw:
        opts["mrw"] = bool(kw.pop("modified_random_walk"))
    for k in ("mrw_gamma", "mrw_tauthres", "mrw_count_trigger", "nepoch", "npilot",
              "max_interactions", "block_threads", "blocks_per_sm", "late_after",
              "mrw_eager_after", "fp64_walls", "drain_below"):
        if k in kw:
            opts[k] = kw.pop(k)
    if "timelimit" in kw:
        opts["timelimit"] = kw.pop("timelimit")
    for k in list(kw):
        if k in _IGNORED:
            kw.pop(k)
    if kw:
        warnings.warn("gb300 run_thermal ignores keywords: %s" % ", ".join(sorted(kw)))
    return opts


def run_thermal(model, nphot=1e6, **keywords):
    """``Model.run_thermal`` for code="gb300": fills ``model.grid.temperature``."""
    opts = _options(keywords)
    plan = ThermalPlan([model.grid], int(nphot), **opts)
    rho_h = torch.from_numpy(stack_density(model.grid).reshape(-1)).pin_memory()
    rho, T = plan.new_buffers()
    rho.copy_(rho_h, non_blocking=True)
    plan.run(rho, T)
    Th = torch.empty(T.shape, dtype=T.dtype, pin_memory=True)
    Th.copy_(T, non_blocking=True)
    stats = plan.check_status()
    model.grid.temperature = plan.split(Th)[0]
    model.thermal_stats = stats
    return stats


def run_thermal_batched(models, nphot=1e6, model_timelimit=None, **keywords):
    """Thermal runs of many models (e.g. MCMC walkers) in one persistent launch per epoch.

    ``timelimit`` bounds the whole launch (every model times out together and
    subprocess.TimeoutExpired is raised, as for one model).  ``model_timelimit`` (seconds,
    one number or one per model) is the per-walker limit of run_disk_model.py:251-273: a
    model that has not finished in time is stopped alone; its ``grid.temperature`` is set
    to None and its entry of ``stats["model_status"]`` is 2, while the others finish with
    the results they have without the limit."""
    opts = _options(keywords)
    plan = ThermalPlan([m.grid for m in models], nphot, **opts)
    if model_timelimit is not None:
        plan.set_model_timelimits(model_timelimit)
    rho_h = torch.from_numpy(np.concatenate([stack_density(m.grid).reshape(-1) for m in models])
                             ).pin_memory()
    rho, T = plan.new_buffers()
    rho.copy_(rho_h, non_blocking=True)
    plan.run(rho, T)
    Th = torch.empty(T.shape, dtype=T.dtype, pin_memory=True)
    Th.copy_(T, non_blocking=True)
    stats = plan.check_status()
    status = plan.model_status()
    stats["model_status"] = [int(x) for x in status]
    for m, temps, st in zip(models, plan.split(Th), status):
        m.grid.temperature = temps if st == 0 else None
    return stats


# Schedule knobs of a thermal plan.  Every setting gives identical results (the walk does
# not depend on which thread or warp runs it); only the time changes.
SCHEDULES = [
    dict(),
    dict(block_threads=128),
    dict(blocks_per_sm=1),
    dict(drain_below=-1),
    dict(drain_below=16384),
    dict(drain_below=4096),
]


def autotune(models, nphot, probe_nphot=20000, schedules=None, cache=None, **keywords):
    """Block and queue schedule for a (batched) thermal run, chosen by timing a short run of
    each candidate schedule on the same models with ``probe_nphot`` packets per model.

    Returns ``(best_schedule, timings_ms)``.  With ``cache`` (a JSON file path) the choice
    is stored under a key of the device name, the number of models and cells and the packet
    count, and reused.  The schedule is a dict of ThermalPlan keywords."""
    import json
    import os
    schedules = SCHEDULES if schedules is None else schedules
    opts = _options(keywords)
    grids = [m.grid for m in models]
    ncell = int(sum(np.asarray(g.density[0]).size * len(g.density) for g in grids))
    key = "%s|%d|%d|%d" % (torch.cuda.get_device_name(), len(grids), ncell, int(nphot))
    if cache and os.path.exists(cache):
        try:
            known = json.load(open(cache))
            if key in known:
                return dict(known[key]["schedule"]), known[key]["timings_ms"]
        except (OSError, ValueError):
            pass
    rho_h = np.concatenate([stack_density(g).reshape(-1) for g in grids])
    timings = []
    for sched in schedules:
        plan = ThermalPlan(grids, probe_nphot, **opts, **sched)
        rho, T = plan.new_buffers()
        rho.copy_(torch.from_numpy(rho_h))
        plan.run(rho, T)                      # warm-up (module load, caches)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record()
        plan.run(rho, T)
        b.record()
        torch.cuda.synchronize()
        plan.check_status()
        timings.append(a.elapsed_time(b))
    best = dict(schedules[int(np.argmin(timings))])
    if cache:
        try:
            known = json.load(open(cache)) if os.path.exists(cache) else {}
        except (OSError, ValueError):
            known = {}
        known[key] = {"schedule": best, "timings_ms": timings}
        with open(cache, "w") as f:
            json.dump(known, f, indent=1)
    return best, timings
