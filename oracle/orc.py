"""ctypes front end of the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and bench.py's CPU-baseline leg import this
module.  It loads ``oracle/_build/liborc.so`` (built by ``oracle/build.py``) and exposes
numpy-level wrappers whose arguments mirror pdspy's Model state: r edges in cm, theta and
phi edges in radians, densities as a list of (nr, ntheta, nphi) arrays, dust opacities on
the wavelength grid in microns (pdspy/modeling/Model.py:723-825 for the conventions).
"""
import ctypes as C
import os

import numpy as np

from . import build as _build

_lib = None

ORC_NROW = 128
ORC_NINV = 4096


class Grid(C.Structure):
    _fields_ = [("nr", C.c_int), ("nt", C.c_int), ("np", C.c_int),
                ("r_edges", C.POINTER(C.c_double)), ("th_edges", C.POINTER(C.c_double)),
                ("ph_edges", C.POINTER(C.c_double))]


class Dust(C.Structure):
    _fields_ = [("nlam", C.c_int), ("nspec", C.c_int), ("lam_um", C.POINTER(C.c_double)),
                ("kabs", C.POINTER(C.c_double)), ("ksca", C.POINTER(C.c_double)),
                ("g", C.POINTER(C.c_double))]


class Stars(C.Structure):
    _fields_ = [("nstar", C.c_int), ("radius_cm", C.POINTER(C.c_double)),
                ("temp_k", C.POINTER(C.c_double))]


class Opts(C.Structure):
    _fields_ = [("nphot", C.c_int64), ("seed", C.c_uint64), ("nepoch", C.c_int),
                ("npilot", C.c_int), ("sequential", C.c_int), ("mrw", C.c_int),
                ("mrw_gamma", C.c_float), ("mrw_tauthres", C.c_float),
                ("mrw_count_trigger", C.c_int), ("max_interactions", C.c_int64),
                ("nthreads", C.c_int), ("model_id", C.c_int), ("late_after", C.c_int64),
                ("mrw_eager_after", C.c_int64), ("fp64_walls", C.c_int),
                ("own_heating", C.c_int)]


class Stats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("packets", "killed", "escaped", "crossings", "events",
                                         "absorptions", "scatterings", "mrw_steps",
                                         "max_packet_events")] + \
        [("events_hist", C.c_int64 * 10)]

    def asdict(self):
        d = {n: int(getattr(self, n)) for n, _ in self._fields_[:-1]}
        d["events_hist"] = list(self.events_hist)
        return d


def lib():
    global _lib
    if _lib is None:
        path = _build.build()
        _lib = C.CDLL(path)
        _lib.orc_mctherm.restype = C.c_int
        _lib.orc_build_tables.restype = C.c_double
        _lib.orc_logf.restype = C.c_float
        _lib.orc_logf.argtypes = [C.c_float]
        _lib.orc_expm.restype = C.c_float
        _lib.orc_expm.argtypes = [C.c_float]
        _lib.orc_expm_frac.restype = C.c_float
        _lib.orc_expm_frac.argtypes = [C.c_float, C.c_float]
        _lib.orc_cbrt01.restype = C.c_float
        _lib.orc_cbrt01.argtypes = [C.c_float]
        _lib.orc_mcscat.restype = C.c_int
    return _lib


def _dp(a):
    return a.ctypes.data_as(C.POINTER(C.c_double))


def philox(ctr, key):
    ctr = (C.c_uint32 * 4)(*ctr)
    key = (C.c_uint32 * 2)(*key)
    out = (C.c_uint32 * 4)()
    lib().orc_philox4x32_10(ctr, key, out)
    return list(out)


def logf(x):
    return lib().orc_logf(C.c_float(x))


def expm(x):
    return lib().orc_expm(C.c_float(x))


def expm_frac(x, e):
    return lib().orc_expm_frac(C.c_float(x), C.c_float(e))


def cbrt01(x):
    return lib().orc_cbrt01(C.c_float(x))


def wall_solve(r_edges, th_edges, ph_edges, pos, direction, ir, itv, ip, last_wall=0,
               fp64=False):
    """(distance, wall code) of one wall solve of the walk (see mcrt_oracle.h)."""
    keep = _Keep()
    g = _grid(r_edges, th_edges, ph_edges, keep)
    P = (C.c_double * 3)(*[float(x) for x in pos])
    D = (C.c_float * 3)(*[float(x) for x in direction])
    d, w = C.c_double(), C.c_int()
    rc = lib().orc_wall_solve(C.byref(g), P, D, int(ir), int(itv), int(ip), int(last_wall),
                              int(bool(fp64)), C.byref(d), C.byref(w))
    if rc:
        raise ValueError("oracle rejected the grid")
    return d.value, w.value


def sincospif2(u):
    s, c = C.c_float(), C.c_float()
    lib().orc_sincospif2(C.c_float(u), C.byref(s), C.byref(c))
    return s.value, c.value


class _Keep:
    """Holds numpy buffers alive while ctypes structs point at them."""

    def __init__(self):
        self.items = []

    def arr(self, a, dtype=np.float64):
        a = np.ascontiguousarray(a, dtype=dtype)
        self.items.append(a)
        return a


def _structs(r_edges, th_edges, ph_edges, lam_um, kabs, ksca, g, star_radius, star_temp, keep):
    r = keep.arr(r_edges); t = keep.arr(th_edges); p = keep.arr(ph_edges)
    grid = Grid(len(r) - 1, len(t) - 1, len(p) - 1, _dp(r), _dp(t), _dp(p))
    lam = keep.arr(lam_um)
    ka = keep.arr(np.atleast_2d(kabs)); ks = keep.arr(np.atleast_2d(ksca))
    gp = None
    if g is not None:
        gg = keep.arr(np.broadcast_to(np.atleast_2d(g), ka.shape))
        gp = _dp(gg)
    dust = Dust(len(lam), ka.shape[0], _dp(lam), _dp(ka), _dp(ks), gp)
    sr = keep.arr(np.atleast_1d(star_radius)); st = keep.arr(np.atleast_1d(star_temp))
    stars = Stars(len(sr), _dp(sr), _dp(st))
    return grid, dust, stars


def build_tables(lam_um, kabs, ksca, g, star_radius, star_temp):
    keep = _Keep()
    _, dust, stars = _structs([1, 2], [0, np.pi], [0, 2 * np.pi], lam_um, kabs, ksca, g,
                              star_radius, star_temp, keep)
    ns, nl = dust.nspec, dust.nlam
    F = np.zeros((ns, ORC_NROW)); cdf = np.zeros((ns, ORC_NROW, nl), np.float32)
    Finv = np.zeros((ns, ORC_NINV)); scdf = np.zeros(nl, np.float32)
    kP = np.zeros((ns, ORC_NROW), np.float32); kR = np.zeros((ns, ORC_NROW), np.float32)
    L = lib().orc_build_tables(C.byref(dust), C.byref(stars), _dp(F),
                               cdf.ctypes.data_as(C.c_void_p), _dp(Finv),
                               scdf.ctypes.data_as(C.c_void_p), kP.ctypes.data_as(C.c_void_p),
                               kR.ctypes.data_as(C.c_void_p))
    return dict(lum=L, F=F, cdf=cdf, Finv=Finv, star_cdf=scdf, kP=kP, kR=kR)


def mctherm(r_edges, th_edges, ph_edges, rho, lam_um, kabs, ksca, g, star_radius, star_temp,
            nphot, seed=0, nepoch=8, npilot=2, sequential=False, mrw=False, mrw_gamma=2.0,
            mrw_tauthres=10.0, mrw_count_trigger=100, max_interactions=10 ** 9, nthreads=0,
            model_id=0, crossings=False, late_after=0, mrw_eager_after=0, fp64_walls=False,
            own_heating=1):
    """Run the oracle; returns dict(energy, temperature, escape, stats[, crossings])."""
    keep = _Keep()
    grid, dust, stars = _structs(r_edges, th_edges, ph_edges, lam_um, kabs, ksca, g,
                                 star_radius, star_temp, keep)
    rho = np.ascontiguousarray(np.asarray(rho, dtype=np.float32).reshape(dust.nspec, -1))
    ncell = grid.nr * grid.nt * grid.np
    assert rho.shape[1] == ncell
    E = np.zeros((dust.nspec, ncell), np.int64)
    T = np.zeros((dust.nspec, ncell), np.float64)
    esc = np.zeros(dust.nlam, np.int64)
    cc = np.zeros(ncell, np.int64) if crossings else None
    opts = Opts(int(nphot), int(seed), nepoch, npilot, int(sequential), int(mrw), mrw_gamma,
                mrw_tauthres, mrw_count_trigger, int(max_interactions), nthreads, model_id,
                int(late_after), int(mrw_eager_after), int(bool(fp64_walls)), int(own_heating))
    st = Stats()
    rc = lib().orc_mctherm(C.byref(grid), C.byref(dust), C.byref(stars),
                           rho.ctypes.data_as(C.c_void_p), C.byref(opts),
                           E.ctypes.data_as(C.c_void_p), T.ctypes.data_as(C.c_void_p),
                           esc.ctypes.data_as(C.c_void_p),
                           cc.ctypes.data_as(C.c_void_p) if cc is not None else None,
                           C.byref(st))
    if rc != 0:
        raise ValueError("oracle rejected the input (rc=%d)" % rc)
    shape = (dust.nspec, grid.nr, grid.nt, grid.np)
    out = dict(energy=E.reshape(shape), temperature=T.reshape(shape), escape=esc,
               stats=st.asdict())
    if cc is not None:
        out["crossings"] = cc.reshape(shape[1:])
    return out


class ScatOpts(C.Structure):
    _fields_ = [("nphot", C.c_int64), ("seed", C.c_uint64), ("maxtauabs", C.c_float),
                ("max_scatter", C.c_int), ("nthreads", C.c_int)]


class ScatStats(C.Structure):
    _fields_ = [(n, C.c_int64) for n in ("packets", "escaped", "dropped", "capped",
                                         "scatterings", "crossings")]

    def asdict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


def mcscat(r_edges, th_edges, ph_edges, rho, lam_um, kabs, ksca, star_radius, star_temp,
           nphot, emis=None, seed=0, maxtauabs=30.0, max_scatter=0, nthreads=0):
    """Scattering Monte Carlo oracle: dict(J [nlam, ncell], acc [nlam, ncell] int64,
    stats).  kabs/ksca [nspec, nlam] at lam_um; rho [nspec, ncell]; emis [nlam, ncell]."""
    keep = _Keep()
    g = _grid(r_edges, th_edges, ph_edges, keep)
    lam = keep.arr(np.atleast_1d(lam_um))
    ka = keep.arr(np.atleast_2d(kabs)); ks = keep.arr(np.atleast_2d(ksca))
    ns, nl = ka.shape
    assert nl == len(lam) and ks.shape == ka.shape
    sr = keep.arr(np.atleast_1d(star_radius)); stt = keep.arr(np.atleast_1d(star_temp))
    stars = Stars(len(sr), _dp(sr), _dp(stt))
    ncell = g.nr * g.nt * g.np
    r = np.ascontiguousarray(np.asarray(rho, dtype=np.float32).reshape(ns, ncell))
    e = None
    if emis is not None:
        e = keep.arr(np.asarray(emis, dtype=np.float64).reshape(nl, ncell))
    J = np.zeros((nl, ncell))
    acc = np.zeros((nl, ncell), np.int64)
    o = ScatOpts(int(nphot), int(seed), float(maxtauabs), int(max_scatter), int(nthreads))
    st = ScatStats()
    rc = lib().orc_mcscat(C.byref(g), nl, _dp(lam), ns, _dp(ka), _dp(ks), C.byref(stars),
                          r.ctypes.data_as(C.c_void_p), _dp(e) if e is not None else None,
                          C.byref(o), _dp(J), acc.ctypes.data_as(C.c_void_p), C.byref(st))
    if rc:
        raise ValueError("oracle rejected the input (rc=%d)" % rc)
    return dict(J=J, acc=acc, stats=st.asdict())


class Camera(C.Structure):
    _fields_ = [("npix_x", C.c_int), ("npix_y", C.c_int), ("pixel_cm", C.c_double),
                ("incl_deg", C.c_double), ("pa_deg", C.c_double), ("phi_deg", C.c_double),
                ("nostar", C.c_int), ("max_refine", C.c_int), ("refine_factor", C.c_double)]


def _grid(r_edges, th_edges, ph_edges, keep):
    r = keep.arr(r_edges); t = keep.arr(th_edges); p = keep.arr(ph_edges)
    return Grid(len(r) - 1, len(t) - 1, len(p) - 1, _dp(r), _dp(t), _dp(p))


def image(r_edges, th_edges, ph_edges, alpha, S, star_flux, npix, pixel_cm, incl=0.0, pa=0.0,
          phi=0.0, nostar=False, max_refine=6, refine_factor=0.5):
    """Pixel-averaged intensity at 1 pc, [nlam, ny, nx]; alpha and S are [nlam, ncell]."""
    keep = _Keep()
    g = _grid(r_edges, th_edges, ph_edges, keep)
    a = np.ascontiguousarray(alpha, dtype=np.float32)
    s = np.ascontiguousarray(S, dtype=np.float32)
    nlam = a.shape[0]
    sf = keep.arr(np.broadcast_to(np.asarray(star_flux, dtype=np.float64), (nlam,)))
    cam = Camera(npix, npix, pixel_cm, incl, pa, phi, int(nostar), max_refine, refine_factor)
    out = np.zeros((nlam, npix, npix))
    rc = lib().orc_image(C.byref(g), nlam, a.ctypes.data_as(C.c_void_p),
                         s.ctypes.data_as(C.c_void_p), _dp(sf), C.byref(cam), _dp(out))
    if rc:
        raise ValueError("oracle rejected the grid")
    return out


def refine_levels(r_edges, th_edges, ph_edges, npix, pixel_cm, max_refine=6, refine_factor=0.5):
    keep = _Keep()
    g = _grid(r_edges, th_edges, ph_edges, keep)
    cam = Camera(npix, npix, pixel_cm, 0.0, 0.0, 0.0, 1, max_refine, refine_factor)
    lv = np.zeros(npix * npix, np.int32)
    lib().orc_refine_levels(C.byref(g), C.byref(cam), lv.ctypes.data_as(C.c_void_p))
    return lv.reshape(npix, npix)


def ray_segments(r_edges, th_edges, ph_edges, npix, pixel_cm, px, py, sub, level, incl=0.0,
                 pa=0.0, phi=0.0, cap=100000):
    keep = _Keep()
    g = _grid(r_edges, th_edges, ph_edges, keep)
    cam = Camera(npix, npix, pixel_cm, incl, pa, phi, 1, 0, 0.5)
    cells = np.zeros(cap, np.int32)
    lens = np.zeros(cap)
    n = lib().orc_ray_segments(C.byref(g), C.byref(cam), px, py, sub, level,
                               cells.ctypes.data_as(C.c_void_p), _dp(lens), cap)
    return cells[:n], lens[:n]
