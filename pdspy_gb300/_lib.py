"""ctypes binding of the C ABI declared in include/pdgpu.h.

The library is built in-tree (``pdspy_gb300/_build/libpdgpu.so``).  Loading fails loudly
when it is missing: there is no CPU fallback for any entry point.
"""
import ctypes as C
import os

from . import _build

_lib = None


class ModelDesc(C.Structure):
    _fields_ = [("nr", C.c_int32), ("ntheta", C.c_int32), ("nphi", C.c_int32),
                ("r_edges_cm", C.POINTER(C.c_double)), ("theta_edges", C.POINTER(C.c_double)),
                ("phi_edges", C.POINTER(C.c_double)), ("nstar", C.c_int32),
                ("star_radius_cm", C.POINTER(C.c_double)),
                ("star_temperature", C.POINTER(C.c_double)), ("nphot", C.c_int64)]


class DustDesc(C.Structure):
    _fields_ = [("nlam", C.c_int32), ("nspec", C.c_int32), ("lam_um", C.POINTER(C.c_double)),
                ("kabs", C.POINTER(C.c_double)), ("ksca", C.POINTER(C.c_double)),
                ("g", C.POINTER(C.c_double))]


class McOptions(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("nepoch", C.c_int32), ("npilot", C.c_int32),
                ("mrw", C.c_int32), ("mrw_gamma", C.c_float), ("mrw_tauthres", C.c_float),
                ("mrw_count_trigger", C.c_int32), ("max_interactions", C.c_int64),
                ("deadline_ns", C.c_int64), ("abort_flag", C.c_void_p),
                ("block_threads", C.c_int32), ("blocks_per_sm", C.c_int32),
                ("late_after", C.c_int64), ("time_launches", C.c_int32),
                ("mrw_eager_after", C.c_int64), ("fp64_walls", C.c_int32),
                ("drain_below", C.c_int64)]


class McStats(C.Structure):
    _fields_ = [("packets", C.c_int64), ("killed", C.c_int64), ("escaped", C.c_int64),
                ("crossings", C.c_int64), ("events", C.c_int64), ("absorptions", C.c_int64),
                ("scatterings", C.c_int64), ("mrw_steps", C.c_int64), ("status", C.c_int32),
                ("launches", C.c_int32), ("parked", C.c_int64), ("late_units", C.c_int64),
                ("drained", C.c_int64)]

    def asdict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class McLayout(C.Structure):
    _fields_ = [("tables_bytes", C.c_size_t), ("energy_offset", C.c_size_t),
                ("late_offset", C.c_size_t), ("escape_offset", C.c_size_t), ("stats_offset", C.c_size_t),
                ("total_bytes", C.c_size_t), ("total_cells", C.c_int64),
                ("nmodels", C.c_int32), ("nspec", C.c_int32), ("nlam", C.c_int32),
                ("smem_tables", C.c_int32)]


class ScatOptions(C.Structure):
    _fields_ = [("seed", C.c_uint64), ("nphot", C.c_int64), ("maxtauabs", C.c_float),
                ("max_scatter", C.c_int32), ("block_threads", C.c_int32),
                ("blocks_per_sm", C.c_int32)]


class ScatStats(C.Structure):
    _fields_ = [("packets", C.c_int64), ("escaped", C.c_int64), ("dropped", C.c_int64),
                ("capped", C.c_int64), ("scatterings", C.c_int64), ("crossings", C.c_int64),
                ("status", C.c_int32)]

    def asdict(self):
        return {n: int(getattr(self, n)) for n, _ in self._fields_}


class Camera(C.Structure):
    _fields_ = [("npix_x", C.c_int32), ("npix_y", C.c_int32), ("pixel_cm", C.c_double),
                ("incl_deg", C.c_double), ("pa_deg", C.c_double), ("phi_deg", C.c_double),
                ("nostar", C.c_int32), ("max_refine", C.c_int32), ("refine_factor", C.c_double)]


STATUS = {0: "ok", 1: "invalid argument", 2: "time limit reached", 3: "aborted",
          4: "packet cap", 5: "overflow", 6: "CUDA error", 7: "no device", 8: "workspace",
          9: "too large for the static scratch"}

# Every symbol include/pdgpu.h declares (checked by the CPU test suite).
EXPORTS = [
    "pdgpu_abi_version", "pdgpu_status_string",
    "pdgpu_mc_plan_create", "pdgpu_mc_plan_destroy", "pdgpu_mc_plan_layout",
    "pdgpu_mc_plan_upload", "pdgpu_mc_plan_run", "pdgpu_mc_plan_stats",
    "pdgpu_mctherm", "pdgpu_mctherm_workspace_bytes", "pdgpu_mc_plan_launch_ms",
    "pdgpu_mc_plan_set_deadline", "pdgpu_mc_plan_set_model_deadlines",
    "pdgpu_mc_plan_model_status",
    "pdgpu_image_plan_create", "pdgpu_image_plan_destroy", "pdgpu_image_plan_info",
    "pdgpu_image_plan_upload", "pdgpu_image_run", "pdgpu_image_adjoint", "pdgpu_image_flux",
    "pdgpu_vis_dft", "pdgpu_vis_dft_adjoint", "pdgpu_mctherm_static",
    "pdgpu_scat_plan_create", "pdgpu_scat_plan_destroy", "pdgpu_scat_plan_info",
    "pdgpu_scat_plan_upload", "pdgpu_scat_run", "pdgpu_scat_plan_stats",
    "pdgpu_vis_grid_sample", "pdgpu_vis_grid_sample_adjoint",
]


class PdgpuError(RuntimeError):
    def __init__(self, status, what=""):
        self.status = int(status)
        super().__init__("%s: %s (status %d)" % (what, STATUS.get(self.status, "?"), self.status))


def lib(build_if_missing=True):
    """Load (building first if needed) the CUDA library."""
    global _lib
    if _lib is not None:
        return _lib
    path = _build.LIB
    if build_if_missing:
        path = _build.build()
    if not os.path.exists(path):
        raise RuntimeError("pdspy_gb300 CUDA library missing at %s; run build()" % path)
    L = C.CDLL(path)
    vp, i32, sz = C.c_void_p, C.c_int32, C.c_size_t
    L.pdgpu_abi_version.restype = i32
    L.pdgpu_status_string.restype = C.c_char_p
    L.pdgpu_status_string.argtypes = [i32]
    L.pdgpu_mc_plan_create.restype = i32
    L.pdgpu_mc_plan_create.argtypes = [i32, C.POINTER(ModelDesc), C.POINTER(DustDesc),
                                       C.POINTER(McOptions), C.POINTER(vp)]
    L.pdgpu_mc_plan_destroy.restype = None
    L.pdgpu_mc_plan_destroy.argtypes = [vp]
    L.pdgpu_mc_plan_layout.restype = i32
    L.pdgpu_mc_plan_layout.argtypes = [vp, C.POINTER(McLayout)]
    L.pdgpu_mc_plan_upload.restype = i32
    L.pdgpu_mc_plan_upload.argtypes = [vp, vp, sz, vp]
    L.pdgpu_mc_plan_run.restype = i32
    L.pdgpu_mc_plan_run.argtypes = [vp, vp, vp, vp, sz, vp]
    L.pdgpu_mc_plan_stats.restype = i32
    L.pdgpu_mc_plan_stats.argtypes = [vp, vp, vp, C.POINTER(McStats)]
    L.pdgpu_mc_plan_launch_ms.restype = i32
    L.pdgpu_mc_plan_launch_ms.argtypes = [vp, C.POINTER(C.c_float), i32]
    L.pdgpu_mc_plan_set_deadline.restype = i32
    L.pdgpu_mc_plan_set_deadline.argtypes = [vp, C.c_int64]
    L.pdgpu_mc_plan_set_model_deadlines.restype = i32
    L.pdgpu_mc_plan_set_model_deadlines.argtypes = [vp, vp, vp]
    L.pdgpu_mc_plan_model_status.restype = i32
    L.pdgpu_mc_plan_model_status.argtypes = [vp, vp, vp, vp]
    L.pdgpu_mctherm.restype = i32
    L.pdgpu_mctherm.argtypes = [i32, C.POINTER(ModelDesc), C.POINTER(DustDesc),
                                C.POINTER(McOptions), vp, vp, vp, sz, vp, C.POINTER(McStats)]
    L.pdgpu_mctherm_workspace_bytes.restype = sz
    L.pdgpu_mctherm_workspace_bytes.argtypes = [i32, C.POINTER(ModelDesc), C.POINTER(DustDesc),
                                                C.POINTER(McOptions)]
    dp = C.POINTER(C.c_double)
    L.pdgpu_image_plan_create.restype = i32
    L.pdgpu_image_plan_create.argtypes = [i32, i32, i32, dp, dp, dp, C.POINTER(Camera), i32, dp,
                                          C.POINTER(vp)]
    L.pdgpu_image_plan_destroy.restype = None
    L.pdgpu_image_plan_destroy.argtypes = [vp]
    L.pdgpu_image_plan_info.restype = i32
    L.pdgpu_image_plan_info.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_int64), vp]
    L.pdgpu_image_plan_upload.restype = i32
    L.pdgpu_image_plan_upload.argtypes = [vp, vp, sz, vp]
    L.pdgpu_image_run.restype = i32
    L.pdgpu_image_run.argtypes = [vp, vp, vp, vp, vp, sz, vp]
    L.pdgpu_image_flux.restype = i32
    L.pdgpu_image_flux.argtypes = [vp, vp, vp, vp]
    L.pdgpu_image_adjoint.restype = i32
    L.pdgpu_image_adjoint.argtypes = [vp, vp, vp, vp, vp, vp, vp, sz, vp]
    L.pdgpu_mctherm_static.restype = i32
    L.pdgpu_mctherm_static.argtypes = [i32, C.POINTER(ModelDesc), C.POINTER(DustDesc),
                                       C.POINTER(McOptions), vp, vp, vp, C.POINTER(McStats)]
    L.pdgpu_scat_plan_create.restype = i32
    L.pdgpu_scat_plan_create.argtypes = [C.POINTER(ModelDesc), i32, dp, i32, dp, dp,
                                         C.POINTER(ScatOptions), C.POINTER(vp)]
    L.pdgpu_scat_plan_destroy.restype = None
    L.pdgpu_scat_plan_destroy.argtypes = [vp]
    L.pdgpu_scat_plan_info.restype = i32
    L.pdgpu_scat_plan_info.argtypes = [vp, C.POINTER(C.c_size_t), C.POINTER(C.c_int64)]
    L.pdgpu_scat_plan_upload.restype = i32
    L.pdgpu_scat_plan_upload.argtypes = [vp, vp, sz, vp]
    L.pdgpu_scat_run.restype = i32
    L.pdgpu_scat_run.argtypes = [vp, vp, vp, vp, vp, sz, vp]
    L.pdgpu_scat_plan_stats.restype = i32
    L.pdgpu_scat_plan_stats.argtypes = [vp, vp, vp, C.POINTER(ScatStats)]
    d = C.c_double
    L.pdgpu_vis_dft.restype = i32
    L.pdgpu_vis_dft.argtypes = [i32, i32, d, d, d, d, vp, i32, vp, vp, vp, vp, vp]
    L.pdgpu_vis_dft_adjoint.restype = i32
    L.pdgpu_vis_dft_adjoint.argtypes = [i32, i32, d, d, d, d, i32, vp, vp, vp, vp, vp, vp]
    L.pdgpu_vis_grid_sample.restype = i32
    L.pdgpu_vis_grid_sample.argtypes = [i32, vp, d, d, d, d, i32, vp, vp, vp, vp, vp]
    L.pdgpu_vis_grid_sample_adjoint.restype = i32
    L.pdgpu_vis_grid_sample_adjoint.argtypes = [i32, d, d, d, d, i32, vp, vp, vp, vp, vp, vp]
    _lib = L
    return L


def check(status, what):
    if status != 0:
        raise PdgpuError(status, what)
