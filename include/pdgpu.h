/*
 * pdgpu: GB300 (sm_103a) backend for pdspy's radiative-transfer hot path.
 *
 * C ABI: plain pointers and sizes, no C++ or torch types.  Every entry point replaces a
 * step of pdspy's radmc3d branch, which today serialises the model to ASCII files, runs
 * the external RADMC-3D binary in a subprocess and parses its output files:
 *
 *   pdgpu_mc_*          Model.run_thermal -> run_thermal_radmc3d
 *                       (pdspy/modeling/Model.py:54-72, :221-256): write_radmc3d
 *                       (Model.py:723-825, radmc3d/write.py:1-342), radmc3d.run.thermal
 *                       (radmc3d/run.py:9-38), radmc3d.read.dust_temperature
 *                       (radmc3d/read.pyx:433-478) and the reshape at Model.py:250-254.
 *   pdgpu_image*        Model.run_image -> run_image_radmc3d (Model.py:324-348,
 *                       :515-577): radmc3d.run.image (radmc3d/run.py:157-289) and
 *                       radmc3d.read.image (radmc3d/read.pyx:25-152).
 *   pdgpu_image_adjoint reverse-mode derivative of the same ray trace; no counterpart in
 *                       the reference (pdspy fits by sampling, utils/emcee.py:6-61).
 *   pdgpu_image_flux    the whole-field spectrum of radmc3d.run.sed / read.spectrum
 *                       behind Model.run_sed (Model.py:608-650, radmc3d/run.py:69-155).
 *   pdgpu_vis_*         visibilities of an image at uv points: the direct sum and the
 *                       gridded (FFT + bilinear) sampling of galario's sampleImage that
 *                       interferometry/interpolate_model.py:11-57 calls, for the chi^2 of
 *                       interferometry/libinterferometry.pyx:610-633 (chisq_calc).
 *   pdgpu_scat_*        the scattering Monte Carlo RADMC-3D runs inside "radmc3d image" /
 *                       "radmc3d spectrum" and as "radmc3d mcscat" (Model.py:258-322,
 *                       radmc3d/run.py:40-67; nphot_scat, mc_scat_maxtauabs from
 *                       radmc3d/write.py:33-38, :141-142).
 *
 * Conventions.  Arrays marked "device" are caller-owned device buffers; arrays marked
 * "host" are read during the call only.  Cell arrays use numpy's C order of pdspy's
 * (nr, ntheta, nphi) grids (pdspy/modeling/Grid.py:71-80); species are stacked in front
 * ([nspec][nr][ntheta][nphi]) and models in front of species for batched plans.  Radii
 * are in cm (pdspy multiplies grid.w1 by AU at Model.py:754-756), angles in radians,
 * wavelengths in microns, opacities in cm^2/g, temperatures in K.
 *
 * Errors are returned as pdgpu_status; no exception crosses the ABI.  Entry points
 * allocate no device memory: the caller passes a workspace of the queried size.
 * Calls on different plans and streams are independent; a plan must not be run on two
 * streams at once.
 */
#ifndef PDGPU_H
#define PDGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PDGPU_ABI_VERSION 4

typedef int32_t pdgpu_status;
enum {
    PDGPU_OK = 0,
    PDGPU_INVALID_ARG = 1,   /* bad sizes, grid not spherical [0,pi] or [0,pi/2], ...   */
    PDGPU_TIMEOUT = 2,       /* deadline_ns elapsed; mirrors radmc3d's timelimit        */
    PDGPU_ABORTED = 3,       /* the abort flag was raised by the host                   */
    PDGPU_PACKET_CAP = 4,    /* informational: packets hit max_interactions             */
    PDGPU_OVERFLOW = 5,      /* a fixed-point accumulator would overflow                */
    PDGPU_CUDA_ERROR = 6,    /* a CUDA runtime call failed                              */
    PDGPU_NO_DEVICE = 7,     /* no usable sm_103 device                                 */
    PDGPU_WORKSPACE = 8,     /* workspace missing, too small or not uploaded            */
    PDGPU_TOO_LARGE = 9      /* needs more than the library's static scratch            */
};

/* Library identity. Replaces nothing in the reference (version probe for the binding). */
int32_t pdgpu_abi_version(void);
const char* pdgpu_status_string(pdgpu_status status);

/* ------------------------------------------------------------------------- */
/* Thermal Monte Carlo (Model.run_thermal)                                    */
/* ------------------------------------------------------------------------- */

/* One model: its spherical grid, its stars and its packet count.
 * Replaces write.amr_grid (radmc3d/write.py:198-244), write.stars (:148-172) and the
 * nphot_therm keyword of write.control (:31-32). */
typedef struct {
    int32_t nr, ntheta, nphi;
    const double* r_edges_cm;       /* host [nr+1], r_edges_cm[0] > 0                  */
    const double* theta_edges;      /* host [ntheta+1]: 0..pi, or 0..pi/2 (mirrored)    */
    const double* phi_edges;        /* host [nphi+1]: 0..2 pi                           */
    int32_t nstar;                  /* blackbody point stars at the origin              */
    const double* star_radius_cm;   /* host [nstar]                                     */
    const double* star_temperature; /* host [nstar], K                                  */
    int64_t nphot;                  /* photon packets for this model                    */
} pdgpu_model_desc;

/* Dust opacities of every species on the shared wavelength grid.
 * Replaces write.wavelength_micron (radmc3d/write.py:174-184), write.dustkappa
 * (:316-342) and write.dustopac (:290-314).  g may be NULL (isotropic scattering, which
 * is what pdspy's iformat-2 dustkappa files give RADMC-3D). */
typedef struct {
    int32_t nlam, nspec;
    const double* lam_um;           /* host [nlam], ascending                           */
    const double* kabs;             /* host [nspec][nlam]                               */
    const double* ksca;             /* host [nspec][nlam]                               */
    const double* g;                /* host [nspec][nlam] or NULL                       */
} pdgpu_dust_desc;

/* Run controls.  Replaces the thermal keywords of write.control
 * (radmc3d/write.py:1-146: iseed, modified_random_walk, mrw_gamma, mrw_tauthres,
 * mrw_count_trigger) and run.thermal's timelimit (radmc3d/run.py:9-38). */
typedef struct {
    uint64_t seed;
    int32_t nepoch;                 /* B&W epochs with doubling sizes (default 8)       */
    int32_t npilot;                 /* pilot passes of the first epoch (default 2)      */
    int32_t mrw;                    /* modified random walk on/off                      */
    float mrw_gamma;
    float mrw_tauthres;
    int32_t mrw_count_trigger;
    int64_t max_interactions;       /* per-packet event cap (killed and counted)        */
    int64_t deadline_ns;            /* device-clock budget for one run, 0 = none        */
    const volatile int32_t* abort_flag; /* device-readable (e.g. host-mapped) or NULL    */
    int32_t block_threads;          /* 0 = default; schedule knobs for the autotuner    */
    int32_t blocks_per_sm;          /* 0 = as many as fit                               */
    int64_t late_after;             /* events of a packet that feed later epochs'       */
                                    /* temperatures; later ones count at the end (0=all)*/
    int32_t time_launches;          /* 1: record CUDA events around transport launches  */
    int64_t mrw_eager_after;        /* beyond this many events of a packet MRW is tried */
                                    /* at every event (0 = never)                       */
    int32_t fp64_walls;             /* 0: double-single positions and wall roots (FP32  */
                                    /* pipe, default); 1: the same kernels with FP64    */
                                    /* geometry, the precision reference                */
    int64_t drain_below;            /* the packets of each pilot, epoch and resumed-    */
                                    /* packet launch run one per thread until fewer than */
                                    /* this many are left, then one per warp (0 = the    */
                                    /* warp launch's width, -1 = never)                  */
} pdgpu_mc_options;

typedef struct {
    int64_t packets, killed, escaped, crossings, events, absorptions, scatterings,
        mrw_steps;
    int32_t status;                 /* pdgpu_status reached by the device               */
    int32_t launches;               /* transport launches of the last run               */
    int64_t parked;                 /* packets resumed by the continuation launches     */
    int64_t late_units;             /* interactions after a packet's late_after-th      */
    int64_t drained;                /* resumed packets finished one per warp            */
} pdgpu_mc_stats;

/* Byte offsets of the run's device arrays inside the workspace. */
typedef struct {
    size_t tables_bytes;            /* constant tables written by plan_upload           */
    size_t energy_offset;           /* int64 [total_cells] absorbed energy, 2^-20 packets */
    size_t late_offset;             /* int64 [total_cells] energy absorbed after        */
                                    /* late_after events of a packet                     */
    size_t escape_offset;           /* int64 [nmodels][nlam] escaping packets per bin    */
    size_t stats_offset;            /* int64 [64]: counters, then per launch             */
                                    /* (t_start, t_end, max events, parked) from slot 32 */
    size_t total_bytes;
    int64_t total_cells;            /* sum over models of nspec * ncell                  */
    int32_t nmodels, nspec, nlam;
    int32_t smem_tables;            /* 1 when the tables fit in shared memory            */
} pdgpu_mc_layout;

typedef struct pdgpu_mc_plan pdgpu_mc_plan;

/* Prepare one or more models sharing one dust description (host work only: tables,
 * wall geometry, epoch schedule).  nmodels > 1 gives the batched persistent launch. */
pdgpu_status pdgpu_mc_plan_create(int32_t nmodels, const pdgpu_model_desc* models,
                                  const pdgpu_dust_desc* dust,
                                  const pdgpu_mc_options* options, pdgpu_mc_plan** plan);
void pdgpu_mc_plan_destroy(pdgpu_mc_plan* plan);
pdgpu_status pdgpu_mc_plan_layout(const pdgpu_mc_plan* plan, pdgpu_mc_layout* layout);

/* Copy the plan's constant tables into the workspace (stream-ordered H2D). */
pdgpu_status pdgpu_mc_plan_upload(pdgpu_mc_plan* plan, void* workspace, size_t bytes,
                                  void* stream);

/* Enqueue one thermal run: rho (device float [models][nspec][cells]) in, temperature
 * (device double, same layout) out.  Only kernel launches and memsets are enqueued, so
 * the call can be captured into a CUDA graph and replayed. */
pdgpu_status pdgpu_mc_plan_run(pdgpu_mc_plan* plan, const float* rho, double* temperature,
                               void* workspace, size_t bytes, void* stream);

/* Durations (ms, CUDA events on the run's stream) of the transport launches of the last
 * run when options.time_launches was set; returns the number written (<= capacity). */
int32_t pdgpu_mc_plan_launch_ms(pdgpu_mc_plan* plan, float* ms, int32_t capacity);

/* Device-clock budget of the plan's later runs (ns, 0 = none); the timelimit argument of
 * radmc3d.run.thermal (radmc3d/run.py:9-38) per run instead of per plan. */
pdgpu_status pdgpu_mc_plan_set_deadline(pdgpu_mc_plan* plan, int64_t deadline_ns);

/* Per-model time limits of a batched plan (one MCMC walker per model).  Replaces
 * run.thermal's timelimit (radmc3d/run.py:9-38) as run_disk_model.py:251-273 applies it: each
 * walker's own radmc3d subprocess may time out, and that walker alone scores -inf
 * (utils/emcee.py:22-23).  deadline_ns[m] (device clock, from the start of each run; 0 = none)
 * stops model m when it has not finished in time: its status becomes PDGPU_TIMEOUT, its
 * remaining packets are dropped (its temperatures are then meaningless) and the other models
 * finish with results identical to a run without the limit.  NULL clears every limit.  The
 * plan must be uploaded; the limits stay until changed and the call waits for the stream. */
pdgpu_status pdgpu_mc_plan_set_model_deadlines(pdgpu_mc_plan* plan, const int64_t* deadline_ns,
                                               void* stream);
/* Status of every model after the last run (host int32 [nmodels]: PDGPU_OK or
 * PDGPU_TIMEOUT); waits for the stream. */
pdgpu_status pdgpu_mc_plan_model_status(pdgpu_mc_plan* plan, const void* workspace, void* stream,
                                        int32_t* status);

/* Synchronise the stream and read the run's counters and device status (the status a
 * radmc3d.run.thermal subprocess reports through its exit and timeout). */
pdgpu_status pdgpu_mc_plan_stats(pdgpu_mc_plan* plan, const void* workspace, void* stream,
                                 pdgpu_mc_stats* stats);

/* One-shot convenience: create, upload, run, read stats, destroy. */
pdgpu_status pdgpu_mctherm(int32_t nmodels, const pdgpu_model_desc* models,
                           const pdgpu_dust_desc* dust, const pdgpu_mc_options* options,
                           const float* rho, double* temperature, void* workspace,
                           size_t bytes, void* stream, pdgpu_mc_stats* stats);
size_t pdgpu_mctherm_workspace_bytes(int32_t nmodels, const pdgpu_model_desc* models,
                                     const pdgpu_dust_desc* dust,
                                     const pdgpu_mc_options* options);

/* Scratch-free thermal run, for callers that cannot allocate device memory: host codes
 * whose GPU memory is owned by another runtime or pool (a Fortran or C walker sharing the
 * GPU with an MCMC framework, code running where cudaMalloc is not permitted).  No
 * counterpart in the reference.  Same arguments and results as pdgpu_mctherm except that
 * the workspace is a file-scope device array of PDGPU_STATIC_WORKSPACE_BYTES held by every
 * GPU that loads the library until the process exits; the caller still passes rho and
 * temperature.  The entry point calls no cudaMalloc/cudaFree.  Its first call on a device
 * looks up the array's device address (cudaGetSymbolAddress) and keeps it for the life of
 * the process, so make that first call before any stream capture, and do not keep using
 * the library across a device reset (cudaDeviceReset) by another part of the process.
 * Every call copies its tables in and its statistics out and waits for the stream to
 * finish before it returns.  Runs whose workspace would exceed the array return
 * PDGPU_TOO_LARGE before any copy or launch.  All calls share the array (each run clears
 * what it accumulates), so calls that overlap on the GPU — on different streams or host
 * threads — race; serialise them. */
#define PDGPU_STATIC_WORKSPACE_BYTES (32u << 20)
pdgpu_status pdgpu_mctherm_static(int32_t nmodels, const pdgpu_model_desc* models,
                                  const pdgpu_dust_desc* dust, const pdgpu_mc_options* options,
                                  const float* rho, double* temperature, void* stream,
                                  pdgpu_mc_stats* stats);

/* ------------------------------------------------------------------------- */
/* Ray-traced images and SEDs (Model.run_image, Model.run_sed)                */
/* ------------------------------------------------------------------------- */

/* Camera of one image.  Replaces the image keywords of radmc3d.run.image
 * (radmc3d/run.py:157-289: npix, zoomau, incl, posang, phi, nostar) as pdspy computes
 * them in Model.run_image_radmc3d (Model.py:515-535).  Pixel (px, py) is centred at
 * ((px - nx/2) pixel_cm, (py - ny/2) pixel_cm) in the sky plane through the origin. */
typedef struct {
    int32_t npix_x, npix_y;
    double pixel_cm;                /* pixel size at the source, cm                     */
    double incl_deg, pa_deg, phi_deg;
    int32_t nostar;
    int32_t max_refine;             /* sub-pixel refinement: at most 4^max_refine rays  */
    double refine_factor;           /* sub-pixel size <= factor x smallest cell size    */
} pdgpu_camera;

typedef struct pdgpu_image_plan pdgpu_image_plan;

/* Prepare one camera over one grid for nlam wavelengths; star_flux[nlam] (host, may be
 * NULL) is the stars' flux at 1 pc, erg/s/cm^2/Hz, put into the centre pixel. */
pdgpu_status pdgpu_image_plan_create(int32_t nr, int32_t ntheta, int32_t nphi,
                                     const double* r_edges_cm, const double* theta_edges,
                                     const double* phi_edges, const pdgpu_camera* camera,
                                     int32_t nlam, const double* star_flux,
                                     pdgpu_image_plan** plan);
void pdgpu_image_plan_destroy(pdgpu_image_plan* plan);
/* Workspace size, number of sub-rays and the per-pixel refinement levels (host int
 * [npix_y][npix_x], may be NULL). */
pdgpu_status pdgpu_image_plan_info(const pdgpu_image_plan* plan, size_t* workspace_bytes,
                                   int64_t* nrays, int32_t* levels);
pdgpu_status pdgpu_image_plan_upload(pdgpu_image_plan* plan, void* workspace, size_t bytes,
                                     void* stream);
/* Image of the per-cell extinction alpha and source S (device float [nlam][ncell], cm^-1
 * and erg/s/cm^2/Hz/ster): device double image[nlam][ny][nx], pixel-averaged intensity
 * at 1 pc (the unit of radmc3d/read.pyx:25-152 before pdspy's Jy conversion). */
pdgpu_status pdgpu_image_run(pdgpu_image_plan* plan, const float* alpha, const float* S,
                             double* image, void* workspace, size_t bytes, void* stream);
/* Whole-field flux of an image from pdgpu_image_run: flux[l] (device double [nlam],
 * erg/s/cm^2/Hz at 1 pc) = pixel solid angle at 1 pc x sum of the pixels of plane l -- the
 * spectrum "radmc3d spectrum" writes (pdspy/radmc3d/run.py:69-155, read.pyx:337-375),
 * which run_sed scales by 1/dpc^2 and converts to Jy (pdspy/modeling/Model.py:639-648). */
pdgpu_status pdgpu_image_flux(pdgpu_image_plan* plan, const double* image, double* flux,
                              void* stream);
/* Reverse-mode derivative of pdgpu_image_run: given dL/dimage (device double, as image)
 * writes dL/dalpha and dL/dS (device double [nlam][ncell]).  No counterpart in the
 * reference, which fits models by sampling (pdspy/utils/emcee.py:6-61). */
pdgpu_status pdgpu_image_adjoint(pdgpu_image_plan* plan, const float* alpha, const float* S,
                                 const double* grad_image, double* grad_alpha,
                                 double* grad_S, void* workspace, size_t bytes, void* stream);

/* ------------------------------------------------------------------------- */
/* Visibilities and chi^2 (interferometry.chisq)                              */
/* ------------------------------------------------------------------------- */

/* Direct Fourier transform of image (device float [ny][nx], Jy per pixel, pixel (i, j) at
 * x = x0 + i dx, y = y0 + j dy radians) at nuv points (device float u, v in wavelengths):
 * re/im (device double [nuv]) = sum F exp(-2 pi i (u x + v y)).  The chi^2
 * sum w [(Re_d - Re)^2 + (Im_d - Im)^2] of pdspy's chisq_calc
 * (interferometry/libinterferometry.pyx:610-633) is formed from these by the caller.
 * Replaces galario's sampleImage in interferometry/interpolate_model.py:11-57. */
pdgpu_status pdgpu_vis_dft(int32_t nx, int32_t ny, double x0_rad, double dx_rad, double y0_rad,
                           double dy_rad, const float* image, int32_t nuv, const float* u,
                           const float* v, double* re, double* im, void* stream);
/* Adjoint of pdgpu_vis_dft: grad_image[p] = sum_k grad_re[k] cos(phi_kp) -
 * grad_im[k] sin(phi_kp).  No counterpart in the reference. */
pdgpu_status pdgpu_vis_dft_adjoint(int32_t nx, int32_t ny, double x0_rad, double dx_rad,
                                   double y0_rad, double dy_rad, int32_t nuv, const float* u,
                                   const float* v, const double* grad_re,
                                   const double* grad_im, double* grad_image, void* stream);

/* Gridded sampling (galario's sampleImage method, pdspy/interferometry/interpolate_model.py:
 * 11-57): grid (device complex64 [n][n], interleaved re/im) is the 2-D FFT
 * G[l][k] = sum_j,i F[j][i] exp(-2 pi i (k i + l j) / n) of an n x n (zero-padded, n even)
 * image whose centre pixel (n/2, n/2) sits at (xc, yc) radians; du = 1 / (n dx) and
 * dv = 1 / (n dy).  re/im (device double [nuv]) = bilinear interpolation of
 * (-1)^(k+l) G at (u / du, v / dv) times exp(-2 pi i (u xc + v yc)): the sum of
 * pdgpu_vis_dft up to the interpolation error.  Points with |u / du| or |v / dv| >= n/2 - 1
 * give NaN. */
pdgpu_status pdgpu_vis_grid_sample(int32_t n, const float* grid, double du, double dv, double xc,
                                   double yc, int32_t nuv, const float* u, const float* v,
                                   double* re, double* im, void* stream);
/* Adjoint of pdgpu_vis_grid_sample: accumulates into grad_grid (device complex128 [n][n],
 * zeroed by the caller) the grid-side gradient H; the image gradient is
 * Re(FFT2(H)) over the image's pixels.  No counterpart in the reference. */
pdgpu_status pdgpu_vis_grid_sample_adjoint(int32_t n, double du, double dv, double xc, double yc,
                                           int32_t nuv, const float* u, const float* v,
                                           const double* grad_re, const double* grad_im,
                                           double* grad_grid, void* stream);

/* ------------------------------------------------------------------------- */
/* Monte Carlo scattering source (images and spectra at albedo > 0)           */
/* ------------------------------------------------------------------------- */

/* Controls of the monochromatic scattering Monte Carlo RADMC-3D runs before "radmc3d
 * image" / "radmc3d spectrum" when the dust scatters, and as "radmc3d mcscat" behind
 * Model.run_scattering (pdspy/modeling/Model.py:258-322, pdspy/radmc3d/run.py:40-67).
 * The keywords pdspy writes to radmc3d.inp map to: nphot_scat / nphot_spec
 * (radmc3d/write.py:33-34; Model.py:520 passes run_image's nphot) -> nphot, and
 * mc_scat_maxtauabs (write.py:141-142) -> maxtauabs.  Scattering is isotropic: pdspy
 * writes dustkappa files without the asymmetry parameter (Model.py:774-776). */
typedef struct pdgpu_scat_options {
    uint64_t seed;
    int64_t nphot;            /* packets per wavelength                                  */
    float maxtauabs;          /* a packet is dropped once the absorption optical depth   */
                              /* along its path exceeds this (<= 0: 30)                  */
    int32_t max_scatter;      /* scatterings per packet before it is dropped (<= 0: 1e6) */
    int32_t block_threads;    /* 0: 256                                                  */
    int32_t blocks_per_sm;    /* 0: from the occupancy calculator                       */
} pdgpu_scat_options;

typedef struct pdgpu_scat_stats {
    int64_t packets, escaped, dropped, capped, scatterings, crossings;
    int32_t status;
} pdgpu_scat_stats;

typedef struct pdgpu_scat_plan pdgpu_scat_plan;

/* One grid (model->nr.. phi_edges, the stars of model; model->nphot is ignored), nlam
 * wavelengths (microns) and the opacities there (host double [nspec][nlam], cm^2/g). */
pdgpu_status pdgpu_scat_plan_create(const pdgpu_model_desc* model, int32_t nlam,
                                    const double* lam_um, int32_t nspec, const double* kabs,
                                    const double* ksca, const pdgpu_scat_options* opts,
                                    pdgpu_scat_plan** plan);
void pdgpu_scat_plan_destroy(pdgpu_scat_plan* plan);
pdgpu_status pdgpu_scat_plan_info(const pdgpu_scat_plan* plan, size_t* workspace_bytes,
                                  int64_t* ncell);
pdgpu_status pdgpu_scat_plan_upload(pdgpu_scat_plan* plan, void* workspace, size_t bytes,
                                    void* stream);
/* Mean intensity of the radiation field in every cell at every wavelength, J (device
 * double [nlam][ncell], erg/s/cm^2/Hz/ster), from packets emitted by the stars and, when
 * emis is given, by the dust (device double [nlam][ncell], thermal emissivity
 * sum_s rho_s kabs_s B_nu(T), erg/s/cm^3/Hz/ster).  rho: device float [nspec][ncell].
 * The isotropic scattering source of a cell is sum_s rho_s ksca_s J.  Enqueues kernels
 * and memsets only. */
pdgpu_status pdgpu_scat_run(pdgpu_scat_plan* plan, const float* rho, const double* emis,
                            double* J, void* workspace, size_t bytes, void* stream);
/* Counters of the last run (synchronises the stream); stats->status as pdgpu_status. */
pdgpu_status pdgpu_scat_plan_stats(pdgpu_scat_plan* plan, const void* workspace, void* stream,
                                   pdgpu_scat_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
