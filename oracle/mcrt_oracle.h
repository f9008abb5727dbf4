/*
 * CPU oracle for the thermal Monte Carlo, the scattering Monte Carlo and the ray-traced
 * images of pdspy's Model.run_thermal / run_scattering / run_image (radmc3d branch,
 * pdspy/modeling/Model.py:221-256, :258-322, :515-577).  TEST INFRASTRUCTURE ONLY: only
 * tests/, __graft_entry__.smoke() and the cpu_baseline leg of bench.py may load this
 * library, and only as the checker or as the timed CPU baseline.  The product (pdspy_gb300) never links or calls it.
 *
 * The arithmetic inside pdspy's radmc3d branch lives in the external RADMC-3D binary,
 * whose source is not part of pdspy and is not pinned by it (pdspy/radmc3d/run.py:9-38
 * only shells out to "radmc3d mctherm").  This oracle therefore restates the published
 * methods RADMC-3D implements:
 *   - Bjorkman & Wood 2001 (ApJ 554, 615): immediate reemission from the
 *     kappa_nu dB_nu/dT spectrum, absorbed-energy counting, T from radiative equilibrium;
 *   - Min et al. 2009 (A&A 497, 155) and Robitaille 2010 (A&A 520, A70): the modified
 *     random walk in optically thick cells;
 *   - Salmon et al. 2011 (SC'11): the Philox4x32-10 counter-based generator.
 * Inputs and units follow pdspy's own conventions: r edges in cm (Model.py:754-756
 * multiplies grid.w1 by AU), theta/phi edges in radians, densities in g cm^-3 laid out
 * as numpy (nr, ntheta, nphi) C-order arrays (Grid.py:22-24), opacities in cm^2 g^-1 on
 * the wavelength grid in microns (Dust.py:181-188, write.py:316-342), stars as
 * blackbodies of radius R and temperature T (Star.py:7-16, write.py:148-172).
 *
 * Parity status: the published algorithm is restated; RADMC-3D itself cannot run here
 * (no binary, no source), so the comparison with RADMC-3D is "parity unpinned".  The
 * oracle is pinned instead by known-answer tests (Philox KAT vectors, the optically thin
 * grey-shell temperature law, energy conservation, isothermal ray traces) and by the
 * density builders of pdspy itself, whose outputs are committed as golden fixtures.
 */
#ifndef PDSPY_MCRT_ORACLE_H
#define PDSPY_MCRT_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Table geometry shared by the oracle and the GPU path (a documented part of the
 * algorithm, so both implementations use the same values). */
#define ORC_NROW 128          /* reemission temperature rows, log-spaced          */
#define ORC_TROW_LO 1.0       /* K                                                 */
#define ORC_TROW_HI 1.0e4     /* K                                                 */
#define ORC_NINV 4096         /* rows of the absorbed-energy -> T inversion table  */
#define ORC_TINV_LO 1.0e-2    /* K                                                 */
#define ORC_TINV_HI 1.0e5     /* K                                                 */
#define ORC_NMRW 1024         /* rows of the MRW diffusion-time table              */
#define ORC_EUNIT_SHIFT 20    /* one absorbed packet = 2^20 fixed-point units      */

typedef struct {
    int nr, nt, np;               /* cell counts                                 */
    const double* r_edges;        /* [nr+1] cm, r_edges[0] > 0                    */
    const double* th_edges;       /* [nt+1] rad, 0..pi or 0..pi/2 (mirror)        */
    const double* ph_edges;       /* [np+1] rad, 0..2pi                           */
} orc_grid;

typedef struct {
    int nlam, nspec;
    const double* lam_um;         /* [nlam] microns, ascending                    */
    const double* kabs;           /* [nspec][nlam] cm^2/g                         */
    const double* ksca;           /* [nspec][nlam] cm^2/g                         */
    const double* g;              /* [nspec][nlam] HG asymmetry, or NULL          */
} orc_dust;

typedef struct {
    int nstar;
    const double* radius_cm;      /* [nstar]                                      */
    const double* temp_k;         /* [nstar]; every star sits at the origin       */
} orc_stars;

typedef struct {
    int64_t nphot;
    uint64_t seed;
    int nepoch;                   /* epochs with doubling packet counts           */
    int npilot;                   /* pilot passes for the first epoch             */
    int sequential;               /* 1: classic sequential B&W (running T)        */
    int mrw;                      /* modified random walk on/off                  */
    float mrw_gamma;              /* sphere radius >= gamma Rosseland mfp          */
    float mrw_tauthres;           /* extinction depth to the nearest wall         */
    int mrw_count_trigger;        /* events in one cell before MRW is tried       */
    int64_t max_interactions;     /* per-packet event cap (packet killed beyond)  */
    int nthreads;                 /* OpenMP threads for the epoch mode (0 = all)  */
    int model_id;                 /* third Philox counter word                     */
    int64_t late_after;           /* events of a packet that feed later epochs;   */
                                  /* later deposits count only at the end (0=all) */
    int64_t mrw_eager_after;      /* beyond this many events MRW is tried at      */
                                  /* every event (0 = never)                      */
    int fp64_walls;               /* 1: FP64 positions and walls; 0: double-single */
                                  /* (pairs of floats, the GPU's default)         */
    int own_heating;              /* 1: reemission and MRW mean opacities add the */
                                  /* packet's own deposits in the cell (the GPU's */
                                  /* algorithm); 0: the epoch snapshot alone      */
} orc_opts;

typedef struct {
    int64_t packets, killed, escaped, crossings, events, absorptions, scatterings,
        mrw_steps;
    int64_t max_packet_events;    /* longest packet (events), final passes only   */
    int64_t events_hist[10];      /* packets per decade of events: [0,10), ...    */
} orc_stats;

/* Philox4x32-10 block for (counter, key); used by the known-answer test. */
void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]);

/* The math helpers the walk uses (exposed for unit tests). */
float orc_logf(float x);
void orc_sincospif2(float u, float* s, float* c); /* sin/cos of 2*pi*u */

/* Tables (host, double precision) for inspection by tests.
 * F[s][ORC_NROW] emissivity per gram at the reemission rows, cdf[s][ORC_NROW][nlam],
 * Finv[s][ORC_NINV], star_cdf[nlam]; returns the total source luminosity (erg/s). */
double orc_build_tables(const orc_dust* dust, const orc_stars* stars, double* F,
                        float* cdf, double* Finv, float* star_cdf, float* kplanck,
                        float* kross);

/* One wall solve of the walk (double-single, or FP64 when fp64 != 0), for the geometry
 * unit tests: exit distance (cm) and wall code (1 inner sphere, 2 outer sphere, 3 lower-
 * index cone, 4 higher-index cone, 5 lower phi plane, 6 higher phi plane) of a packet at
 * pos moving along dir in cell (ir, itv, ip), itv the virtual theta index. */
int orc_wall_solve(const orc_grid* grid, const double pos[3], const float dir[3], int ir,
                   int itv, int ip, int last_wall, int fp64, double* dist, int* wall);

/* Thermal Monte Carlo.  energy[s][cell] receives the int64 fixed-point absorbed
 * energy (unit = packet energy / 2^20), temperature[s][cell] the dust temperature
 * in K.  escape[nlam] (optional) counts escaping packets per wavelength bin;
 * cell_crossings[ncell] (optional) counts packet crossings per cell.
 * Returns 0 on success, 1 on invalid input. */
int orc_mctherm(const orc_grid* grid, const orc_dust* dust, const orc_stars* stars,
                const float* rho, const orc_opts* opts, int64_t* energy,
                double* temperature, int64_t* escape, int64_t* cell_crossings,
                orc_stats* stats);

/* Scattering Monte Carlo (mcscat_oracle.c): mean intensity J per cell and wavelength. */
typedef struct {
    int64_t nphot;                /* packets per wavelength                        */
    uint64_t seed;
    float maxtauabs;              /* drop a packet beyond this absorption depth    */
                                  /* (<= 0: 30)                                    */
    int max_scatter;              /* scatterings before a packet is dropped (<= 0: */
                                  /* 1e6)                                          */
    int nthreads;                 /* OpenMP threads (0 = all)                      */
} orc_scat_opts;

typedef struct {
    int64_t packets, escaped, dropped, capped, scatterings, crossings;
} orc_scat_stats;

/* exp(-x) for x >= 0, (1 - exp(-x)) / x given e = exp(-x), and the cube root on (0, 1]
 * as the scattering walk evaluates them (exposed for unit tests). */
float orc_expm(float x);
float orc_expm_frac(float x, float e);
float orc_cbrt01(float x);

/* J[nlam][ncell] (erg/s/cm^2/Hz/ster) at wavelengths lam_um (microns) for opacities
 * kabs/ksca [nspec][nlam] (cm^2/g), densities rho [nspec][ncell] (g/cm^3), the stars
 * (at the origin) and, when emis is not NULL, the thermal emissivity of the cells
 * emis[nlam][ncell] (erg/s/cm^3/Hz/ster).  acc_out (optional, int64 [nlam][ncell])
 * receives the fixed-point path sums.  Returns 0 on success, 1 on invalid input. */
int orc_mcscat(const orc_grid* grid, int nlam, const double* lam_um, int nspec,
               const double* kabs, const double* ksca, const orc_stars* stars,
               const float* rho, const double* emis, const orc_scat_opts* opts, double* J,
               int64_t* acc_out, orc_scat_stats* stats);

#ifdef __cplusplus
}
#endif
#endif
