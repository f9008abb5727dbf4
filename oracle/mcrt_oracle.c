/*
 * CPU oracle: thermal Monte Carlo photon transport on a spherical grid.
 * TEST INFRASTRUCTURE ONLY (see mcrt_oracle.h).  Compiled with -ffp-contract=off and
 * without fast-math so that every floating-point operation is a single IEEE operation;
 * together with the explicitly ordered expressions below this makes the packet walk
 * reproducible operation for operation.
 *
 * Algorithm (restated from the published methods; pdspy hands this job to RADMC-3D at
 * pdspy/radmc3d/run.py:9-38 with the controls written by pdspy/radmc3d/write.py:1-146):
 *
 *  Emission.  Every packet starts at the origin (the star), with an isotropic
 *  direction, a wavelength bin drawn from the stellar luminosity per bin
 *  L_l = 4 pi R^2 * pi B_nu(T*) dnu_l and an optical depth target -ln(u).  The packet
 *  energy is L/N with L = sum_l L_l.
 *
 *  Transport.  Cell walls are spheres r = r_i, cones theta = theta_j and half-planes
 *  phi = phi_k.  The exit distance is solved in double precision; the root of each
 *  quadric is chosen by the sign of the quadric's derivative, so that the root that
 *  leaves the current cell is taken and the wall just entered is never re-crossed at
 *  zero distance.  tau accumulates rho * kext in single precision.
 *
 *  Interaction.  Scattering with probability albedo (Henyey-Greenstein, isotropic when
 *  g = 0), else absorption by a species chosen in proportion to rho_s kabs_s.  An
 *  absorption adds one packet (2^20 fixed-point units) to E[s][cell] and reemits the
 *  packet isotropically with a wavelength drawn from kappa_nu dB_nu/dT at the cell's
 *  current temperature (Bjorkman & Wood 2001).
 *
 *  Deterministic B&W ("epochs").  The sequential method reads the running cell
 *  temperature, so its result depends on packet order.  The epoch form splits the N
 *  packets into epochs whose sizes double; during epoch k the reemission temperature of
 *  an absorption is T(q') with q' = q_lo + u q_span, q_lo = E/m the energy absorbed in
 *  earlier epochs and q_span = q_lo (R_k - 1) the energy expected by the end of the
 *  epoch (R_k = b_{k+1}/b_k).  The first epoch, which has no history, is run npilot
 *  times to estimate its own span and then once for real.  Deposits are integer, so the
 *  final E does not depend on the order in which packets run.
 *
 *  Modified random walk (Min et al. 2009; Robitaille 2010).  After mrw_count_trigger
 *  events in one cell, if the sphere to the nearest wall holds >= gamma Rosseland mean
 *  free paths and >= tauthres extinction depths at the packet wavelength, the packet
 *  jumps to the sphere's surface; the diffusion time y is drawn from the survival law
 *  S(y) = 2 sum (-1)^(n+1) exp(-n^2 pi^2 y); the path length 3 alpha_R R0^2 y deposits
 *  rho_s kP_s l packet energies (Lucy 1999 estimator); the packet leaves with a
 *  cosine-weighted outward direction and a B&W reemission wavelength.
 *
 *  Temperature.  4 pi sum_l kabs_l B_l(T) dnu_l = E q_unit / (rho V) is inverted from a
 *  4096-row table in double precision.
 */
#include "mcrt_oracle.h"
#include "mc_internal.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* pdspy physical constants (pdspy/constants/physics.py:1-15). */
#define C_LIGHT 2.99792458e10
#define H_PLANCK 6.6260755e-27
#define K_BOLTZ 1.380658e-16
#define PI_D 3.14159265358979323846

/* ------------------------------------------------------------------------- */
/* Philox4x32-10 (Salmon et al. 2011): 10 rounds of two 32x32->64 multiplies */
/* with Weyl key increments.                                                  */
/* ------------------------------------------------------------------------- */
#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

void orc_philox4x32_10(const uint32_t ctr[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t c0 = ctr[0], c1 = ctr[1], c2 = ctr[2], c3 = ctr[3];
    uint32_t k0 = key[0], k1 = key[1];
    for (int r = 0; r < 10; ++r) {
        uint64_t p0 = (uint64_t)PHILOX_M0 * (uint64_t)c0;
        uint64_t p1 = (uint64_t)PHILOX_M1 * (uint64_t)c2;
        uint32_t hi0 = (uint32_t)(p0 >> 32), lo0 = (uint32_t)p0;
        uint32_t hi1 = (uint32_t)(p1 >> 32), lo1 = (uint32_t)p1;
        uint32_t n0 = hi1 ^ c1 ^ k0;
        uint32_t n2 = hi0 ^ c3 ^ k1;
        c0 = n0; c1 = lo1; c2 = n2; c3 = lo0;
        k0 += PHILOX_W0; k1 += PHILOX_W1;
    }
    out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

/* Uniform in (0,1): 23 random bits as an odd multiple of 2^-24 (exact in float). */
static inline float u01(uint32_t x) {
    return (float)(((x >> 9) << 1) | 1u) * 5.9604644775390625e-08f;
}

/* ln(x) for normal positive floats: x = 2^e m, m in (sqrt(1/2), sqrt(2)],
 * ln m = 2 atanh(t), t = (m-1)/(m+1), atanh by its odd power series to t^9. */
float orc_logf(float x) {
    uint32_t bits;
    memcpy(&bits, &x, 4);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    uint32_t mb = (bits & 0x007fffffu) | 0x3f800000u;
    float m;
    memcpy(&m, &mb, 4);
    if (m > 1.41421356f) {
        m = m * 0.5f;
        e = e + 1;
    }
    float t = (m - 1.0f) / (m + 1.0f);
    float s = t * t;
    float p = 0.11111111f;
    p = p * s + 0.14285715f;
    p = p * s + 0.2f;
    p = p * s + 0.33333334f;
    float t2 = 2.0f * t;
    float lm = t2 + t2 * (s * p);
    return (float)e * 0.69314718f + lm;
}

/* sin and cos of 2 pi u for u in (0,1): reduce to the nearest quarter turn and use
 * the Taylor series of sin (to x^9) and cos (to x^8) on |x| <= pi/4. */
void orc_sincospif2(float u, float* sn, float* cs) {
    float a = 2.0f * u;                 /* half turns, in (0, 2)        */
    int n = (int)(a * 2.0f + 0.5f);     /* nearest quarter turn, 0..4   */
    float r = a - (float)n * 0.5f;      /* in [-0.25, 0.25] half turns  */
    float x = r * 3.14159265f;
    float x2 = x * x;
    float sp = 2.7557319e-06f;          /* 1/9!  */
    sp = sp * x2 - 1.9841270e-04f;      /* 1/7!  */
    sp = sp * x2 + 8.3333333e-03f;      /* 1/5!  */
    sp = sp * x2 - 1.6666667e-01f;      /* 1/3!  */
    float sx = x + x * (x2 * sp);
    float cp = 2.4801587e-05f;          /* 1/8!  */
    cp = cp * x2 - 1.3888889e-03f;      /* 1/6!  */
    cp = cp * x2 + 4.1666668e-02f;      /* 1/4!  */
    cp = cp * x2 - 0.5f;                /* 1/2!  */
    float cx = 1.0f + x2 * cp;
    switch (n & 3) {
        case 0: *sn = sx; *cs = cx; break;
        case 1: *sn = cx; *cs = -sx; break;
        case 2: *sn = -sx; *cs = -cx; break;
        default: *sn = -cx; *cs = sx; break;
    }
}

/* ------------------------------------------------------------------------- */
/* Tables                                                                     */
/* ------------------------------------------------------------------------- */
static double planck_nu(double nu, double T) {
    double x = H_PLANCK * nu / (K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double pre = 2.0 * H_PLANCK * nu * nu * nu / (C_LIGHT * C_LIGHT);
    return pre / expm1(x);
}

static double dplanck_dT(double nu, double T) {
    double x = H_PLANCK * nu / (K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double em1 = expm1(x);
    double pre = 2.0 * H_PLANCK * nu * nu * nu / (C_LIGHT * C_LIGHT);
    double bb = pre / em1;
    return bb * (x * exp(x) / em1) / T;
}

static double row_temperature(int j) {
    return ORC_TROW_LO * pow(ORC_TROW_HI / ORC_TROW_LO, (double)j / (double)(ORC_NROW - 1));
}

static double inv_temperature(int j) {
    return ORC_TINV_LO * pow(ORC_TINV_HI / ORC_TINV_LO, (double)j / (double)(ORC_NINV - 1));
}

static void freq_weights(int nlam, const double* lam_um, double* nu, double* dnu) {
    for (int l = 0; l < nlam; ++l) nu[l] = C_LIGHT / (lam_um[l] * 1.0e-4);
    for (int l = 0; l < nlam; ++l) {
        if (l == 0)
            dnu[l] = 0.5 * fabs(nu[0] - nu[1]);
        else if (l == nlam - 1)
            dnu[l] = 0.5 * fabs(nu[nlam - 2] - nu[nlam - 1]);
        else
            dnu[l] = 0.5 * fabs(nu[l - 1] - nu[l + 1]);
    }
}

/* S(y) = 2 sum_{n>=1} (-1)^(n+1) exp(-n^2 pi^2 y): probability that a walker started at
 * the centre of a sphere has not reached its surface after reduced time y = D t / R^2. */
static double mrw_survival(double y) {
    if (y < 0.005) return 1.0;
    double s = 0.0;
    for (int n = 1; n < 100000; ++n) {
        double a = (double)n * (double)n * PI_D * PI_D * y;
        if (a > 80.0) break;
        double t = exp(-a);
        s += (n & 1) ? t : -t;
    }
    return 2.0 * s;
}

static float g_mrw_table[ORC_NMRW];
static int g_mrw_ready = 0;

static void build_mrw_table(void) {
    if (g_mrw_ready) return;
    for (int i = 0; i < ORC_NMRW; ++i) {
        double xi = (double)i / (double)(ORC_NMRW - 1);
        if (i == ORC_NMRW - 1) { g_mrw_table[i] = 0.0f; continue; }
        if (i == 0) xi = 1.0e-7;
        double lo = 0.0, hi = 10.0;
        for (int it = 0; it < 100; ++it) {
            double mid = 0.5 * (lo + hi);
            if (mrw_survival(mid) > xi) lo = mid; else hi = mid;
        }
        g_mrw_table[i] = (float)(0.5 * (lo + hi));
    }
    g_mrw_ready = 1;
}

typedef struct {
    int nlam, nspec;
    double* nu; double* dnu;
    float* kabs; float* ksca; float* kext; float* g;   /* [nspec][nlam]            */
    float* star_cdf;                                    /* [nlam]                   */
    double lum;                                         /* erg/s                    */
    float* Ff;                                          /* [nspec][NROW]            */
    float* cdf;                                         /* [nspec][NROW][nlam]      */
    float* kP; float* kR;                               /* [nspec][NROW]            */
    double* Tinv; double* Finv;                         /* [NINV], [nspec][NINV]    */
} Tables;

static void free_tables(Tables* t) {
    free(t->nu); free(t->dnu); free(t->kabs); free(t->ksca); free(t->kext); free(t->g);
    free(t->star_cdf); free(t->Ff); free(t->cdf); free(t->kP); free(t->kR);
    free(t->Tinv); free(t->Finv);
}

static int make_tables(const orc_dust* d, const orc_stars* st, Tables* t,
                       double* F_out, double* Finv_out) {
    int nl = d->nlam, ns = d->nspec;
    memset(t, 0, sizeof(*t));
    t->nlam = nl; t->nspec = ns;
    t->nu = malloc(sizeof(double) * nl); t->dnu = malloc(sizeof(double) * nl);
    freq_weights(nl, d->lam_um, t->nu, t->dnu);
    t->kabs = malloc(sizeof(float) * ns * nl); t->ksca = malloc(sizeof(float) * ns * nl);
    t->kext = malloc(sizeof(float) * ns * nl); t->g = malloc(sizeof(float) * ns * nl);
    for (int i = 0; i < ns * nl; ++i) {
        t->kabs[i] = (float)d->kabs[i];
        t->ksca[i] = (float)d->ksca[i];
        t->kext[i] = t->kabs[i] + t->ksca[i];
        t->g[i] = d->g ? (float)d->g[i] : 0.0f;
    }
    /* stellar spectrum per bin */
    double* Lnu = calloc(nl, sizeof(double));
    for (int s = 0; s < st->nstar; ++s) {
        double R = st->radius_cm[s];
        for (int l = 0; l < nl; ++l)
            Lnu[l] += 4.0 * PI_D * R * R * PI_D * planck_nu(t->nu[l], st->temp_k[s]) * t->dnu[l];
    }
    double L = 0.0;
    for (int l = 0; l < nl; ++l) L += Lnu[l];
    t->lum = L;
    t->star_cdf = malloc(sizeof(float) * nl);
    double cum = 0.0;
    for (int l = 0; l < nl; ++l) {
        cum += Lnu[l];
        t->star_cdf[l] = (float)(cum / L);
    }
    t->star_cdf[nl - 1] = 1.0f;
    free(Lnu);

    t->Ff = malloc(sizeof(float) * ns * ORC_NROW);
    t->cdf = malloc(sizeof(float) * (size_t)ns * ORC_NROW * nl);
    t->kP = malloc(sizeof(float) * ns * ORC_NROW);
    t->kR = malloc(sizeof(float) * ns * ORC_NROW);
    double* cumv = malloc(sizeof(double) * nl);
    for (int s = 0; s < ns; ++s) {
        const double* ka = d->kabs + (size_t)s * nl;
        const double* ks = d->ksca + (size_t)s * nl;
        for (int j = 0; j < ORC_NROW; ++j) {
            double T = row_temperature(j);
            double sumF = 0.0, sumB = 0.0, sumD = 0.0, sumDk = 0.0, c = 0.0;
            for (int l = 0; l < nl; ++l) {
                double B = planck_nu(t->nu[l], T);
                double dB = dplanck_dT(t->nu[l], T);
                sumF += ka[l] * B * t->dnu[l];
                sumB += B * t->dnu[l];
                sumD += dB * t->dnu[l];
                double ke = ka[l] + ks[l];
                if (ke > 0.0) sumDk += dB / ke * t->dnu[l];
                c += ka[l] * dB * t->dnu[l];
                cumv[l] = c;
            }
            double Fj = 4.0 * PI_D * sumF;
            if (F_out) F_out[(size_t)s * ORC_NROW + j] = Fj;
            t->Ff[(size_t)s * ORC_NROW + j] = (float)Fj;
            float* row = t->cdf + ((size_t)s * ORC_NROW + j) * nl;
            for (int l = 0; l < nl; ++l)
                row[l] = (c > 0.0) ? (float)(cumv[l] / c) : (float)((l + 1.0) / nl);
            row[nl - 1] = 1.0f;
            t->kP[(size_t)s * ORC_NROW + j] = (float)(sumB > 0.0 ? sumF / sumB : 0.0);
            t->kR[(size_t)s * ORC_NROW + j] = (float)(sumDk > 0.0 ? sumD / sumDk : 0.0);
        }
    }
    free(cumv);

    t->Tinv = malloc(sizeof(double) * ORC_NINV);
    t->Finv = malloc(sizeof(double) * ns * ORC_NINV);
    for (int j = 0; j < ORC_NINV; ++j) t->Tinv[j] = inv_temperature(j);
    for (int s = 0; s < ns; ++s) {
        const double* ka = d->kabs + (size_t)s * nl;
        for (int j = 0; j < ORC_NINV; ++j) {
            double sumF = 0.0;
            for (int l = 0; l < nl; ++l) sumF += ka[l] * planck_nu(t->nu[l], t->Tinv[j]) * t->dnu[l];
            t->Finv[(size_t)s * ORC_NINV + j] = 4.0 * PI_D * sumF;
            if (Finv_out) Finv_out[(size_t)s * ORC_NINV + j] = 4.0 * PI_D * sumF;
        }
    }
    build_mrw_table();
    return 0;
}

double orc_build_tables(const orc_dust* dust, const orc_stars* stars, double* F, float* cdf,
                        double* Finv, float* star_cdf, float* kplanck, float* kross) {
    Tables t;
    make_tables(dust, stars, &t, F, Finv);
    if (cdf) memcpy(cdf, t.cdf, sizeof(float) * (size_t)t.nspec * ORC_NROW * t.nlam);
    if (star_cdf) memcpy(star_cdf, t.star_cdf, sizeof(float) * t.nlam);
    if (kplanck) memcpy(kplanck, t.kP, sizeof(float) * t.nspec * ORC_NROW);
    if (kross) memcpy(kross, t.kR, sizeof(float) * t.nspec * ORC_NROW);
    double L = t.lum;
    free_tables(&t);
    return L;
}

/* ------------------------------------------------------------------------- */
/* Grid                                                                       */
/* ------------------------------------------------------------------------- */

int orc__make_geo(const orc_grid* g, Geo* G) {
    memset(G, 0, sizeof(*G));
    G->nr = g->nr; G->nt = g->nt; G->np = g->np;
    G->ncell = g->nr * g->nt * g->np;
    G->r = g->r_edges;
    G->ph = g->ph_edges;
    if (g->nr < 1 || g->nt < 1 || g->np < 1) return 1;
    if (!(g->r_edges[0] > 0.0)) return 1;
    double thmax = g->th_edges[g->nt];
    if (fabs(g->th_edges[0]) > 1e-12) return 1;
    if (fabs(thmax - PI_D) < 1e-9) G->mirror = 0;
    else if (fabs(thmax - 0.5 * PI_D) < 1e-9) G->mirror = 1;
    else return 1;
    if (g->np > 1 && (fabs(g->ph_edges[0]) > 1e-12 || fabs(g->ph_edges[g->np] - 2.0 * PI_D) > 1e-9))
        return 1;
    int nt = g->nt;
    G->ntv = G->mirror ? 2 * nt : nt;
    G->mu = malloc(sizeof(double) * (G->ntv + 1));
    G->sn = malloc(sizeof(double) * (G->ntv + 1));
    for (int j = 0; j <= nt; ++j) {
        double th = g->th_edges[j];
        double m = cos(th), s = sin(th);
        if (fabs(th - 0.5 * PI_D) < 1e-12) { m = 0.0; s = 1.0; }
        if (j == 0) { m = 1.0; s = 0.0; }
        if (!G->mirror && j == nt) { m = -1.0; s = 0.0; }
        G->mu[j] = m; G->sn[j] = s;
    }
    if (G->mirror)
        for (int j = 0; j < nt; ++j) {
            G->mu[2 * nt - j] = -G->mu[j];
            G->sn[2 * nt - j] = G->sn[j];
        }
    G->cph = malloc(sizeof(double) * (g->np + 1));
    G->sph = malloc(sizeof(double) * (g->np + 1));
    for (int k = 0; k <= g->np; ++k) {
        G->cph[k] = cos(g->ph_edges[k]);
        G->sph[k] = sin(g->ph_edges[k]);
    }
    G->Vr = malloc(sizeof(double) * g->nr);
    G->Vt = malloc(sizeof(double) * nt);
    G->Vp = malloc(sizeof(double) * g->np);
    for (int i = 0; i < g->nr; ++i) {
        double r0 = g->r_edges[i], r1 = g->r_edges[i + 1];
        G->Vr[i] = (r1 * r1 * r1 - r0 * r0 * r0) / 3.0;
    }
    for (int j = 0; j < nt; ++j) {
        double v = G->mu[j] - G->mu[j + 1];
        G->Vt[j] = G->mirror ? 2.0 * v : v;
    }
    for (int k = 0; k < g->np; ++k) G->Vp[k] = g->ph_edges[k + 1] - g->ph_edges[k];
    G->rf = malloc(sizeof(float) * (g->nr + 1));
    G->muf = malloc(sizeof(float) * (G->ntv + 1));
    G->snf = malloc(sizeof(float) * (G->ntv + 1));
    G->cphf = malloc(sizeof(float) * (g->np + 1));
    G->sphf = malloc(sizeof(float) * (g->np + 1));
    for (int i = 0; i <= g->nr; ++i) G->rf[i] = (float)g->r_edges[i];
    for (int j = 0; j <= G->ntv; ++j) { G->muf[j] = (float)G->mu[j]; G->snf[j] = (float)G->sn[j]; }
    for (int k = 0; k <= g->np; ++k) { G->cphf[k] = (float)G->cph[k]; G->sphf[k] = (float)G->sph[k]; }
    /* double-single walls: hi = nearest float, lo = nearest float of the remainder */
    G->rl = malloc(sizeof(float) * (g->nr + 1));
    G->r2h = malloc(sizeof(float) * (g->nr + 1));
    G->r2l = malloc(sizeof(float) * (g->nr + 1));
    G->mu2h = malloc(sizeof(float) * (G->ntv + 1));
    G->mu2l = malloc(sizeof(float) * (G->ntv + 1));
    for (int i = 0; i <= g->nr; ++i) {
        double R = g->r_edges[i];
        double R2 = R * R;
        G->rl[i] = (float)(R - (double)(float)R);
        G->r2h[i] = (float)R2;
        G->r2l[i] = (float)(R2 - (double)(float)R2);
    }
    for (int j = 0; j <= G->ntv; ++j) {
        double m2 = G->mu[j] * G->mu[j];
        G->mu2h[j] = (float)m2;
        G->mu2l[j] = (float)(m2 - (double)(float)m2);
    }
    return 0;
}

void orc__free_geo(Geo* G) {
    free(G->mu); free(G->sn); free(G->cph); free(G->sph); free(G->Vr); free(G->Vt); free(G->Vp);
    free(G->rf); free(G->muf); free(G->snf); free(G->cphf); free(G->sphf);
    free(G->rl); free(G->r2h); free(G->r2l); free(G->mu2h); free(G->mu2l);
}

/* ------------------------------------------------------------------------- */
/* Packet                                                                     */
/* ------------------------------------------------------------------------- */

/* Random numbers of interaction n of a packet: one Philox block per stream with counter
 * (n, packet id, model, pass tag | stream << 24).  Streams: 0 albedo test, new optical
 * depth, direction cosine, azimuth; 1 reemission q', reemission row, reemission CDF,
 * species; 2 MRW diffusion time, jump cosine, jump azimuth; 3 (n = 0) the emission. */
enum { RS_EVENT = 0, RS_SECOND = 1, RS_MRW = 2, RS_EMIT = 3 };

/* Upper bound of the distance to the nearest wall, kept along the walk: set from a computed
 * wall distance D (a lower bound within a relative 5e-6), grown by every move (triangle
 * inequality, rounded up), unknown after a crossing.  MRW is tried only when the bound
 * allows a jump. */
#define ORC_DMAX_UNKNOWN 3.0e38f
static inline float dmax_of(float D) { return D * 1.00001f; }
static inline float dmax_after(float dmax, float step) {
    return dmax < ORC_DMAX_UNKNOWN ? (dmax + step) * 1.000001f : ORC_DMAX_UNKNOWN;
}

static inline void ev_block(const Pkt* p, uint32_t n, uint32_t stream, float u[4]) {
    uint32_t c[4], o[4];
    c[0] = n; c[1] = p->ctr[1]; c[2] = p->ctr[2]; c[3] = p->ctr[3] | (stream << 24);
    orc_philox4x32_10(c, p->key, o);
    for (int i = 0; i < 4; ++i) u[i] = u01(o[i]);
}


/* Candidate acceptance: the wall the packet entered through needs a strictly positive
 * distance; any other wall accepts tiny negative roots (rounding) as zero. */
static inline int accept_root(double s, int wall, int last, double tol, double* out) {
    if (wall == last) {
        if (s > tol) { *out = s; return 1; }
        return 0;
    }
    if (s >= -tol) { *out = s > 0.0 ? s : 0.0; return 1; }
    return 0;
}

double orc__next_wall(const Geo* G, const Pkt* p, int* wall_out) {
    double x = p->x, y = p->y, z = p->z;
    double kx = (double)p->kx, ky = (double)p->ky, kz = (double)p->kz;
    double kk = kx * kx + ky * ky + kz * kz;
    double r2 = x * x + y * y + z * z;
    double b = x * kx + y * ky + z * kz;
    int last = p->last_wall;
    double best = 1.0e300;
    int bw = W_NONE;
    double Ro = (p->ir < 0) ? G->r[0] : G->r[p->ir + 1];
    double tol = 1.0e-10 * Ro;
    double cand;
    /* outer sphere: always an exit */
    {
        double c = r2 - Ro * Ro;
        double D = b * b - kk * c;
        if (D < 0.0) D = 0.0;
        double sq = sqrt(D);
        double s = (b <= 0.0) ? (sq - b) / kk : -c / (b + sq);
        if (!(last == W_ROUT && s <= tol)) { best = (s > 0.0) ? s : 0.0; bw = W_ROUT; }
    }
    if (p->ir < 0) { *wall_out = bw; return best; }
    /* inner sphere */
    if (b < 0.0) {
        double Ri = G->r[p->ir];
        double c = r2 - Ri * Ri;
        double D = b * b - kk * c;
        if (D >= 0.0) {
            double s = c / (sqrt(D) - b);
            if (accept_root(s, W_RIN, last, tol, &cand) && cand < best) { best = cand; bw = W_RIN; }
        }
    }
    /* theta cones */
    for (int side = 0; side < 2; ++side) {
        int w = p->itv + side;                  /* side 0: lower wall, 1: upper wall */
        if (w == 0 || w == G->ntv) continue;    /* poles are not walls              */
        int code = side ? W_THI : W_TLO;
        double mu = G->mu[w];
        double s;
        int ok = 0;
        if (mu == 0.0) {
            if (side == 0 ? (kz > 0.0) : (kz < 0.0)) { s = -z / kz; ok = 1; }
        } else {
            double mu2 = mu * mu;
            double A = kz * kz - mu2 * kk;
            double B = z * kz - mu2 * b;
            double C = z * z - mu2 * r2;
            int want_plus = (side == 0) ? (mu > 0.0) : (mu < 0.0);
            double D = B * B - A * C;
            if (D >= 0.0) {
                double sq = sqrt(D);
                if (A == 0.0) {
                    if (want_plus ? (B > 0.0) : (B < 0.0)) { s = -C / (2.0 * B); ok = 1; }
                } else {
                    double q = (B >= 0.0) ? -(B + sq) : (sq - B);
                    if (q != 0.0) {
                        double sm, sp;
                        if (B >= 0.0) { sm = q / A; sp = C / q; }
                        else { sp = q / A; sm = C / q; }
                        s = want_plus ? sp : sm;
                        ok = 1;
                    }
                }
                if (ok) {
                    double zs = z + s * kz;
                    if (mu > 0.0 ? (zs < 0.0) : (zs > 0.0)) ok = 0;
                }
            }
        }
        if (ok && accept_root(s, code, last, tol, &cand) && cand < best) { best = cand; bw = code; }
    }
    /* phi half-planes */
    if (G->np > 1) {
        int k0 = p->ip, k1 = p->ip + 1;
        double g0 = -x * G->sph[k0] + y * G->cph[k0];
        double dg = -kx * G->sph[k0] + ky * G->cph[k0];
        if (dg < 0.0) {
            double s = -g0 / dg;
            double hx = x + s * kx, hy = y + s * ky;
            if (hx * G->cph[k0] + hy * G->sph[k0] > 0.0 &&
                accept_root(s, W_PLO, last, tol, &cand) && cand < best) { best = cand; bw = W_PLO; }
        }
        double h0 = x * G->sph[k1] - y * G->cph[k1];
        double dh = kx * G->sph[k1] - ky * G->cph[k1];
        if (dh < 0.0) {
            double s = -h0 / dh;
            double hx = x + s * kx, hy = y + s * ky;
            if (hx * G->cph[k1] + hy * G->sph[k1] > 0.0 &&
                accept_root(s, W_PHI, last, tol, &cand) && cand < best) { best = cand; bw = W_PHI; }
        }
    }
    *wall_out = bw;
    return best;
}

void orc__locate_angles(const Geo* G, Pkt* p) {
    double x = p->x, y = p->y, z = p->z;
    double r = sqrt(x * x + y * y + z * z);
    double ct = z / r;
    int lo = 0, hi = G->ntv;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (G->mu[mid] >= ct) lo = mid; else hi = mid;
    }
    p->itv = lo;
    if (G->np > 1) {
        double ph = atan2(y, x);
        if (ph < 0.0) ph += 2.0 * PI_D;
        int a = 0, bnd = G->np;
        while (bnd - a > 1) {
            int mid = a + (bnd - a) / 2;
            if (G->ph[mid] <= ph) a = mid; else bnd = mid;
        }
        p->ip = a;
    } else {
        p->ip = 0;
    }
}

int orc__cell_index(const Geo* G, const Pkt* p) {
    int it = (p->itv < G->nt) ? p->itv : (2 * G->nt - 1 - p->itv);
    return (p->ir * G->nt + it) * G->np + p->ip;
}

/* Rotate direction k by polar cosine mu and azimuth (cp, sp) about itself. */
static void rotate_dir(float* kx, float* ky, float* kz, float mu, float cp, float sp) {
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    float ax = *kx, ay = *ky, az = *kz;
    float nx, ny, nz;
    float w2 = 1.0f - az * az;
    if (w2 > 1.0e-10f) {
        float w = sqrtf(w2);
        float sw = st / w;
        nx = mu * ax + sw * (ax * az * cp - ay * sp);
        ny = mu * ay + sw * (ay * az * cp + ax * sp);
        nz = mu * az - st * cp * w;
    } else {
        nx = st * cp;
        ny = st * sp;
        nz = (az >= 0.0f) ? mu : -mu;
    }
    float rn = 1.0f / sqrtf(nx * nx + ny * ny + nz * nz);
    *kx = nx * rn; *ky = ny * rn; *kz = nz * rn;
}

static void iso_dir(Pkt* p, float umu, float uphi) {
    float mu = 2.0f * umu - 1.0f;
    float sn, cs;
    orc_sincospif2(uphi, &sn, &cs);
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    p->kx = st * cs; p->ky = st * sn; p->kz = mu;
}

static int cdf_search(const float* cdf, int n, float u) {
    int lo = -1, hi = n - 1;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (cdf[mid] > u) hi = mid; else lo = mid;
    }
    return hi;
}

/* Fractional reemission row of q on the increasing row table F. */
static void row_search(const float* F, float q, int* j_out, float* w_out) {
    int j;
    float w;
    if (q < F[0]) { j = 0; w = 0.0f; }
    else if (q >= F[ORC_NROW - 1]) { j = ORC_NROW - 2; w = 1.0f; }
    else {
        int lo = 0, hi = ORC_NROW - 1;
        while (hi - lo > 1) {
            int mid = lo + (hi - lo) / 2;
            if (F[mid] <= q) lo = mid; else hi = mid;
        }
        j = lo;
        w = (q - F[j]) / (F[j + 1] - F[j]);
        if (w < 0.0f) w = 0.0f;
        if (w > 1.0f) w = 1.0f;
    }
    *j_out = j; *w_out = w;
}

typedef struct {
    const Geo* G;
    const Tables* T;
    const float* rho;       /* [nspec][ncell]   */
    const double* mass;     /* [nspec][ncell]   */
    const float* wq;        /* [nspec][ncell] q per deposit unit: (float)(q_unit / mass) */
    float* qlo; float* qspan;
    int64_t* E;             /* deposits of a packet's first late_after events   */
    int64_t* Elate;         /* deposits of its later events                      */
    int64_t late_after;     /* 0: every deposit goes to E                        */
    int pilot;              /* pilot pass: packets stop after late_after events  */
    int64_t* escape;
    int64_t* ccross;
    double q_unit;
    int sequential;
    const orc_opts* o;
    int64_t* hist;          /* [10] packets per decade of events, or NULL */
    int64_t* maxev;
} Ctx;

static void atomic_add64(int64_t* a, int64_t v) { __atomic_fetch_add(a, v, __ATOMIC_RELAXED); }

/* The packet's own deposits per (species, cell) in a four-entry round-robin cache: the
 * reemission temperature and the MRW mean opacities of a cell are taken at the epoch's
 * snapshot plus the packet's own deposits there (sequential B&W lets a packet trapped in
 * an optically thick cell heat the cell it reemits from; the snapshot cannot see deposits
 * made after it was taken). */
#define OWNK 4
static void own_add(Pkt* p, int64_t sc, int64_t units) {
    for (int i = 0; i < OWNK; ++i)
        if (p->own_sc[i] == sc) { p->own_u[i] += units; return; }
    p->own_sc[p->own_next] = sc;
    p->own_u[p->own_next] = units;
    p->own_next = (p->own_next + 1) % OWNK;
}

static float own_q(const Ctx* X, const Pkt* p, int64_t sc) {
    for (int i = 0; i < OWNK; ++i)
        if (p->own_sc[i] == sc) return (float)p->own_u[i] * X->wq[sc];
    return 0.0f;
}

/* Deposit target of the current event: the first late_after events of a packet feed
 * the main accumulator (read by later epochs), the rest the late accumulator. */
#define DEP(X, p) (((X)->late_after > 0 && (p).nevents > (X)->late_after) ? (X)->Elate : (X)->E)

/* Reemission wavelength for species s in cell c. */
/* Reemission wavelength bin of species s in cell c from the uniforms (uq, urow, ucdf). */
static int reemit_lambda(const Ctx* X, const Pkt* p, int s, int c, float uq, float urow, float ucdf) {
    const Tables* T = X->T;
    size_t sc = (size_t)s * X->G->ncell + c;
    float q;
    if (X->sequential) {
        int64_t e = __atomic_load_n(&X->E[sc], __ATOMIC_RELAXED);
        q = (X->mass[sc] > 0.0) ? (float)((double)e * X->q_unit / X->mass[sc]) : 0.0f;
    } else {
        q = X->qlo[sc] + uq * X->qspan[sc];
        if (X->o->own_heating) q = q + own_q(X, p, (int64_t)sc);
    }
    int j;
    float w;
    row_search(T->Ff + (size_t)s * ORC_NROW, q, &j, &w);
    int row = j + ((urow < w) ? 1 : 0);
    return cdf_search(T->cdf + ((size_t)s * ORC_NROW + row) * T->nlam, T->nlam, ucdf);
}

/* Frozen-row interpolation of a [NROW] table at the cell's mid-epoch energy. */
static float row_interp(const Ctx* X, const Pkt* p, const float* tab_s, int s, int c) {
    size_t sc = (size_t)s * X->G->ncell + c;
    float q;
    if (X->sequential) {
        int64_t e = __atomic_load_n(&X->E[sc], __ATOMIC_RELAXED);
        q = (X->mass[sc] > 0.0) ? (float)((double)e * X->q_unit / X->mass[sc]) : 0.0f;
    } else {
        q = X->qlo[sc] + 0.5f * X->qspan[sc];
        if (X->o->own_heating) q = q + own_q(X, p, (int64_t)sc);
    }
    int j;
    float w;
    row_search(X->T->Ff + (size_t)s * ORC_NROW, q, &j, &w);
    return tab_s[j] + w * (tab_s[j + 1] - tab_s[j]);
}

/* Lower bound of the distance from the packet to every wall of its cell (the safety
 * distance and the MRW sphere radius).  The small differences that cancel near a wall
 * (r^2 - R^2, the cone quadric rho^2 cos^2 - z^2 sin^2, the phi-plane offsets) are
 * formed in double precision from the double position; only non-cancelling factors
 * (r + R, |rho cos| + |z sin|) use single precision.  The result has a relative error
 * below 1e-6, so the relative margin 4e-6 keeps it a lower bound; no square root or
 * division runs in double precision. */
static float wall_distance(const Geo* G, const Pkt* p) {
    double x = p->x, y = p->y, z = p->z;
    double x2 = x * x, y2 = y * y, z2 = z * z;
    double rho2 = x2 + y2;
    double r2 = rho2 + z2;
    float rf = sqrtf((float)r2);
    double Ri = G->r[p->ir], Ro = G->r[p->ir + 1];
    float d = (float)(r2 - Ri * Ri) / (rf + G->rf[p->ir]);
    float d2 = (float)(Ro * Ro - r2) / (rf + G->rf[p->ir + 1]);
    if (d2 < d) d = d2;
    float rhof = sqrtf((float)rho2);
    float zf = (float)z;
    for (int side = 0; side < 2; ++side) {
        int w = p->itv + side;
        if (w == 0 || w == G->ntv) continue;
        float a = rhof * G->muf[w];
        float b = zf * G->snf[w];
        float dt;
        if ((a > 0.0f) == (b > 0.0f)) {
            double mu = G->mu[w], sn = G->sn[w];
            double num = rho2 * (mu * mu) - z2 * (sn * sn);
            float den = fabsf(a) + fabsf(b);
            dt = den > 0.0f ? fabsf((float)num) / den : 0.0f;
        } else {
            dt = fabsf(a) + fabsf(b);
        }
        if (dt < d) d = dt;
    }
    if (G->np > 1) {
        int k0 = p->ip, k1 = p->ip + 1;
        float d0 = (float)fabs(-x * G->sph[k0] + y * G->cph[k0]);
        float d1 = (float)fabs(x * G->sph[k1] - y * G->cph[k1]);
        if (d0 < d) d = d0;
        if (d1 < d) d = d1;
    }
    float m = d * (1.0f - 4.0e-6f);
    return m > 0.0f ? m : 0.0f;
}

typedef struct { int64_t killed, escaped, crossings, events, absorptions, scatterings, mrw; } Cnt;

static int64_t run_packet(const Ctx* X, uint32_t pid, uint32_t tag, Cnt* cnt) {
    const Geo* G = X->G;
    const Tables* T = X->T;
    const orc_opts* o = X->o;
    int ns = T->nspec, nl = T->nlam;
    const int f64 = o->fp64_walls;
    Pkt p;
    memset(&p, 0, sizeof(p));
    for (int i = 0; i < 4; ++i) p.own_sc[i] = -1;
    p.ctr[1] = pid; p.ctr[2] = (uint32_t)o->model_id; p.ctr[3] = tag;
    p.key[0] = (uint32_t)(o->seed & 0xffffffffu);
    p.key[1] = (uint32_t)(o->seed >> 32);
    /* emission */
    {
        float e[4];
        ev_block(&p, 0u, RS_EMIT, e);
        float mu = 2.0f * e[0] - 1.0f;
        float sn, cs;
        orc_sincospif2(e[1], &sn, &cs);
        float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
        p.kx = st * cs; p.ky = st * sn; p.kz = mu;
        p.lam = cdf_search(T->star_cdf, nl, e[2]);
        p.tau = -orc_logf(e[3]);
        p.ir = -1; p.itv = 0; p.ip = 0;
        p.last_wall = W_NONE;
        p.dmax = ORC_DMAX_UNKNOWN;
        p.fresh = 1;
    }
    for (;;) {
        int c = -1;
        float alpha = 0.0f;
        if (p.ir >= 0) {
            c = orc__cell_index(G, &p);
            for (int s = 0; s < ns; ++s)
                alpha = alpha + X->rho[(size_t)s * G->ncell + c] * T->kext[(size_t)s * nl + p.lam];
        }
        /* Safety distance: an interaction closer than the isotropic distance to the
         * nearest wall needs no wall solve. */
        int full = 1;
        double se = 0.0;
        float sef = 0.0f;
        if (alpha > 0.0f) {
            sef = p.tau / alpha;
            /* a safety distance not computed here is refreshed before a wall solve */
            if (!(sef < p.dsafe) && !p.fresh) {
                float D = f64 ? wall_distance(G, &p) : orc__wall_distance_ds(G, &p);
                p.dsafe = 0.999999f * D;
                p.dmax = dmax_of(D);
                p.fresh = 1;
            }
            if (sef < p.dsafe) { full = 0; se = (double)sef; }
        }
        int wall = W_NONE;
        double sw = 0.0;
        /* double-single geometry: the wall distance is a pair (hi + Newton correction) and
         * an event at the wall takes the pair; comparisons use the hi part */
        ds swd = {0.0f, 0.0f}, sed = {sef, 0.0f};
        float tcell = 0.0f;
        int is_event = 1;
        if (full) {
            if (f64) {
                sw = orc__next_wall(G, &p, &wall);
            } else {
                swd = orc__next_wall_ds(G, &p, &wall);
                sw = (double)swd.h;
            }
            tcell = alpha * (float)sw;
            is_event = tcell > p.tau;
            if (is_event) {
                se = (double)(p.tau / alpha);
                sed.h = p.tau / alpha;
                sed.l = 0.0f;
                if (se > sw) { se = sw; sed = swd; }
            }
        }
        if (is_event) {
            /* interaction inside the cell */
            if (f64) {
                p.x = fma(se, (double)p.kx, p.x);
                p.y = fma(se, (double)p.ky, p.y);
                p.z = fma(se, (double)p.kz, p.z);
            } else {
                orc__move_ds(&p, sed, p.kx, p.ky, p.kz);
            }
            p.dsafe = full ? 0.0f : p.dsafe - sef;
            p.fresh = 0;
            p.last_wall = W_NONE;
            const uint32_t n = (uint32_t)p.nevents;   /* index of this interaction */
            p.cell_events += 1;
            p.nevents += 1;
            cnt->events += 1;
            float ev[4], sb[4];
            ev_block(&p, n, RS_EVENT, ev);
            p.dmax = dmax_after(p.dmax, (float)se);
            int did_mrw = 0;
            /* MRW is considered after mrw_count_trigger events in one cell, and at every
             * event once the packet has made more than mrw_eager_after events (it is
             * trapped).  It is tried (the wall distance computed) only when the distance
             * bound allows a jump; a try also refreshes the safety distance. */
            const int cond = o->mrw && (p.cell_events >= o->mrw_count_trigger ||
                                        (o->mrw_eager_after > 0 && p.nevents > o->mrw_eager_after));
            int tried = 0;
            float Dw = 0.0f;
            float aR = 0.0f;
            if (cond && 0.999f * p.dmax * alpha >= o->mrw_tauthres) {
                for (int s = 0; s < ns; ++s)
                    aR = aR + X->rho[(size_t)s * G->ncell + c] *
                                  row_interp(X, &p, T->kR + (size_t)s * ORC_NROW, s, c);
                tried = 0.999f * p.dmax * aR >= o->mrw_gamma;
            }
            if (tried) {
                Dw = f64 ? wall_distance(G, &p) : orc__wall_distance_ds(G, &p);
                float R0f = 0.999f * Dw;
                double R0 = (double)R0f;
                if (R0f * aR >= o->mrw_gamma && R0f * alpha >= o->mrw_tauthres) {
                    did_mrw = 1;
                    float mb[4];
                    ev_block(&p, n, RS_MRW, mb);
                    ev_block(&p, n, RS_SECOND, sb);
                    float uy = mb[0];
                    float f = uy * (float)(ORC_NMRW - 1);
                    int i = (int)f;
                    if (i > ORC_NMRW - 2) i = ORC_NMRW - 2;
                    float w = f - (float)i;
                    float yv = g_mrw_table[i] + w * (g_mrw_table[i + 1] - g_mrw_table[i]);
                    float ell = 3.0f * aR * R0f * R0f * yv;
                    float kp[8];
                    float aP = 0.0f;
                    for (int s = 0; s < ns; ++s) {
                        kp[s] = X->rho[(size_t)s * G->ncell + c] *
                                row_interp(X, &p, T->kP + (size_t)s * ORC_NROW, s, c);
                        aP = aP + kp[s];
                        float units_f = kp[s] * ell * 1048576.0f + 0.5f;
                        if (units_f > 9.0e18f) units_f = 9.0e18f;
                        int64_t units = (int64_t)units_f;
                        if (units > 0) {
                            atomic_add64(&DEP(X, p)[(size_t)s * G->ncell + c], units);
                            own_add(&p, (int64_t)s * G->ncell + c, units);
                        }
                    }
                    /* jump to the sphere surface */
                    float dx, dy, dz;
                    {
                        float mu = 2.0f * mb[1] - 1.0f;
                        float sn, cs;
                        orc_sincospif2(mb[2], &sn, &cs);
                        float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
                        dx = st * cs; dy = st * sn; dz = mu;
                    }
                    if (f64) {
                        p.x = fma(R0, (double)dx, p.x);
                        p.y = fma(R0, (double)dy, p.y);
                        p.z = fma(R0, (double)dz, p.z);
                    } else {
                        ds r0 = {R0f, 0.0f};
                        orc__move_ds(&p, r0, dx, dy, dz);
                    }
                    {
                        float mu = sqrtf(ev[2]);
                        float sn, cs;
                        orc_sincospif2(ev[3], &sn, &cs);
                        float kx = dx, ky = dy, kz = dz;
                        rotate_dir(&kx, &ky, &kz, mu, cs, sn);
                        p.kx = kx; p.ky = ky; p.kz = kz;
                    }
                    int sp = 0;
                    if (ns > 1) {
                        float us = sb[3] * aP;
                        float acc = 0.0f;
                        sp = ns - 1;
                        for (int s = 0; s < ns; ++s) {
                            acc = acc + kp[s];
                            if (us < acc) { sp = s; break; }
                        }
                    }
                    p.lam = reemit_lambda(X, &p, sp, c, sb[0], sb[1], sb[2]);
                    p.tau = -orc_logf(ev[1]);
                    p.cell_events = 0;
                    cnt->mrw += 1;
                }
            }
            if (!did_mrw) {
                float ua = ev[0];
                float asca = 0.0f;
                for (int s = 0; s < ns; ++s)
                    asca = asca + X->rho[(size_t)s * G->ncell + c] * T->ksca[(size_t)s * nl + p.lam];
                if (ua * alpha < asca) {
                    /* scattering */
                    int sp = 0;
                    if (ns > 1) {
                        ev_block(&p, n, RS_SECOND, sb);
                        float us = sb[3] * asca;
                        float acc = 0.0f;
                        sp = ns - 1;
                        for (int s = 0; s < ns; ++s) {
                            acc = acc + X->rho[(size_t)s * G->ncell + c] * T->ksca[(size_t)s * nl + p.lam];
                            if (us < acc) { sp = s; break; }
                        }
                    }
                    float g = T->g[(size_t)sp * nl + p.lam];
                    float umu = ev[2];
                    float mu;
                    if (fabsf(g) < 1.0e-4f) {
                        mu = 2.0f * umu - 1.0f;
                    } else {
                        float t = (1.0f - g * g) / (1.0f - g + 2.0f * g * umu);
                        mu = (1.0f + g * g - t * t) / (2.0f * g);
                        if (mu < -1.0f) mu = -1.0f;
                        if (mu > 1.0f) mu = 1.0f;
                    }
                    float sn, cs;
                    orc_sincospif2(ev[3], &sn, &cs);
                    rotate_dir(&p.kx, &p.ky, &p.kz, mu, cs, sn);
                    cnt->scatterings += 1;
                } else {
                    /* absorption + reemission */
                    ev_block(&p, n, RS_SECOND, sb);
                    int sp = 0;
                    if (ns > 1) {
                        float aabs = 0.0f;
                        for (int s = 0; s < ns; ++s)
                            aabs = aabs + X->rho[(size_t)s * G->ncell + c] * T->kabs[(size_t)s * nl + p.lam];
                        float us = sb[3] * aabs;
                        float acc = 0.0f;
                        sp = ns - 1;
                        for (int s = 0; s < ns; ++s) {
                            acc = acc + X->rho[(size_t)s * G->ncell + c] * T->kabs[(size_t)s * nl + p.lam];
                            if (us < acc) { sp = s; break; }
                        }
                    }
                    atomic_add64(&DEP(X, p)[(size_t)sp * G->ncell + c], (int64_t)1 << ORC_EUNIT_SHIFT);
                    own_add(&p, (int64_t)sp * G->ncell + c, (int64_t)1 << ORC_EUNIT_SHIFT);
                    p.lam = reemit_lambda(X, &p, sp, c, sb[0], sb[1], sb[2]);
                    iso_dir(&p, ev[2], ev[3]);
                    cnt->absorptions += 1;
                }
                p.tau = -orc_logf(ev[1]);
            }
            if (did_mrw)
                Dw = f64 ? wall_distance(G, &p) : orc__wall_distance_ds(G, &p);
            if (did_mrw || tried) {
                p.dsafe = 0.999999f * Dw;
                p.dmax = dmax_of(Dw);
                p.fresh = 1;
            }
            if (p.nevents >= o->max_interactions) { cnt->killed += 1; return p.nevents; }
            if (X->pilot && X->late_after > 0 && p.nevents >= X->late_after) return p.nevents;
        } else {
            /* move to the wall and change cell */
            if (f64) {
                p.x = fma(sw, (double)p.kx, p.x);
                p.y = fma(sw, (double)p.ky, p.y);
                p.z = fma(sw, (double)p.kz, p.z);
            } else {
                orc__move_ds(&p, swd, p.kx, p.ky, p.kz);
            }
            p.tau = p.tau - tcell;
            p.dsafe = 0.0f;          /* on a wall: a wall solve is due */
            p.dmax = ORC_DMAX_UNKNOWN;
            p.fresh = 1;
            p.ncross += 1;
            cnt->crossings += 1;
            if (X->ccross && c >= 0) atomic_add64(&X->ccross[c], 1);
            p.cell_events = 0;
            switch (wall) {
                case W_ROUT:
                    if (p.ir < 0) {
                        p.ir = 0;
                        if (f64) orc__locate_angles(G, &p); else orc__locate_angles_ds(G, &p);
                    }
                    else p.ir += 1;
                    p.last_wall = W_RIN;
                    if (p.ir >= G->nr) {
                        cnt->escaped += 1;
                        if (X->escape) atomic_add64(&X->escape[p.lam], 1);
                        return p.nevents;
                    }
                    break;
                case W_RIN: p.ir -= 1; p.last_wall = W_ROUT; break;
                case W_TLO: p.itv -= 1; p.last_wall = W_THI; break;
                case W_THI: p.itv += 1; p.last_wall = W_TLO; break;
                case W_PLO: p.ip = (p.ip == 0) ? G->np - 1 : p.ip - 1; p.last_wall = W_PHI; break;
                case W_PHI: p.ip = (p.ip == G->np - 1) ? 0 : p.ip + 1; p.last_wall = W_PLO; break;
                default: cnt->killed += 1; return p.nevents;
            }
            if (p.ncross > 100000000) { cnt->killed += 1; return p.nevents; }
        }
    }
}

static void run_range(const Ctx* X, int64_t b0, int64_t b1, uint32_t tag, Cnt* tot, int nthreads) {
    int64_t killed = 0, escaped = 0, crossings = 0, events = 0, absorptions = 0, scatterings = 0, mrw = 0;
    if (X->sequential) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 16) num_threads(nthreads) \
    reduction(+ : killed, escaped, crossings, events, absorptions, scatterings, mrw)
#endif
    for (int64_t i = b0; i < b1; ++i) {
        Cnt c;
        memset(&c, 0, sizeof(c));
        int64_t nev = run_packet(X, (uint32_t)i, tag, &c);
        killed += c.killed; escaped += c.escaped; crossings += c.crossings; events += c.events;
        absorptions += c.absorptions; scatterings += c.scatterings; mrw += c.mrw;
        if (X->hist) {
            int b = 0;
            for (int64_t v = nev; v >= 10 && b < 9; v /= 10) ++b;
            __atomic_fetch_add(&X->hist[b], 1, __ATOMIC_RELAXED);
            int64_t old = __atomic_load_n(X->maxev, __ATOMIC_RELAXED);
            while (nev > old &&
                   !__atomic_compare_exchange_n(X->maxev, &old, nev, 0, __ATOMIC_RELAXED, __ATOMIC_RELAXED)) {
            }
        }
    }
    (void)nthreads;
    tot->killed += killed; tot->escaped += escaped; tot->crossings += crossings;
    tot->events += events; tot->absorptions += absorptions; tot->scatterings += scatterings;
    tot->mrw += mrw;
}

static double q_unit_of(const Tables* T, const orc_opts* o) {
    return T->lum / (double)o->nphot / (double)((int64_t)1 << ORC_EUNIT_SHIFT);
}

static double invert_temperature(const Tables* T, int s, int64_t E, double m, double q_unit) {
    if (E <= 0 || !(m > 0.0)) return 0.0;
    const double* F = T->Finv + (size_t)s * ORC_NINV;
    double q = (double)E * q_unit / m;
    if (q <= F[0]) return T->Tinv[0] * sqrt(sqrt(q / F[0]));
    if (q >= F[ORC_NINV - 1]) return T->Tinv[ORC_NINV - 1];
    int lo = 0, hi = ORC_NINV - 1;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (F[mid] <= q) lo = mid; else hi = mid;
    }
    return T->Tinv[lo] + (T->Tinv[lo + 1] - T->Tinv[lo]) * ((q - F[lo]) / (F[lo + 1] - F[lo]));
}

/* One wall solve of the walk, exposed for the geometry unit tests: the packet at pos
 * (cm; held as a double-single pair, or as doubles when fp64 is set) moving along dir in
 * cell (ir, itv, ip) having entered through last_wall.  Returns 0 and the exit distance and
 * wall code, 1 on an invalid grid. */
int orc_wall_solve(const orc_grid* grid, const double pos[3], const float dir[3], int ir,
                   int itv, int ip, int last_wall, int fp64, double* dist, int* wall) {
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return 1; }
    Pkt p;
    memset(&p, 0, sizeof(p));
    p.x = pos[0]; p.y = pos[1]; p.z = pos[2];
    p.sx.h = (float)pos[0]; p.sx.l = (float)(pos[0] - (double)p.sx.h);
    p.sy.h = (float)pos[1]; p.sy.l = (float)(pos[1] - (double)p.sy.h);
    p.sz.h = (float)pos[2]; p.sz.l = (float)(pos[2] - (double)p.sz.h);
    p.kx = dir[0]; p.ky = dir[1]; p.kz = dir[2];
    p.ir = ir; p.itv = itv; p.ip = ip;
    p.last_wall = last_wall;
    if (fp64) {
        *dist = orc__next_wall(&G, &p, wall);
    } else {
        ds d = orc__next_wall_ds(&G, &p, wall);
        *dist = (double)d.h + (double)d.l;
    }
    orc__free_geo(&G);
    return 0;
}

int orc_mctherm(const orc_grid* grid, const orc_dust* dust, const orc_stars* stars,
                const float* rho, const orc_opts* o, int64_t* energy, double* temperature,
                int64_t* escape, int64_t* cell_crossings, orc_stats* stats) {
    if (!grid || !dust || !stars || !rho || !o || !energy) return 1;
    if (dust->nlam < 2 || dust->nspec < 1 || dust->nspec > 8 || stars->nstar < 1) return 1;
    if (o->nphot < 1 || o->nphot > 4000000000LL) return 1;
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return 1; }
    Tables T;
    make_tables(dust, stars, &T, NULL, NULL);
    int ns = dust->nspec, nc = G.ncell;
    size_t n = (size_t)ns * nc;
    double* mass = malloc(sizeof(double) * n);
    for (int s = 0; s < ns; ++s)
        for (int i = 0; i < G.nr; ++i)
            for (int j = 0; j < G.nt; ++j)
                for (int k = 0; k < G.np; ++k) {
                    int cc = (i * G.nt + j) * G.np + k;
                    double V = G.Vr[i] * G.Vt[j] * G.Vp[k];
                    mass[(size_t)s * nc + cc] = (double)rho[(size_t)s * nc + cc] * V;
                }
    float* wq = malloc(sizeof(float) * n);
    for (size_t i = 0; i < n; ++i) wq[i] = (mass[i] > 0.0) ? (float)(q_unit_of(&T, o) / mass[i]) : 0.0f;
    float* qlo = calloc(n, sizeof(float));
    float* qspan = calloc(n, sizeof(float));
    int64_t* D = calloc(n, sizeof(int64_t));
    int64_t* Elate = calloc(n, sizeof(int64_t));
    memset(energy, 0, sizeof(int64_t) * n);
    if (escape) memset(escape, 0, sizeof(int64_t) * dust->nlam);
    if (cell_crossings) memset(cell_crossings, 0, sizeof(int64_t) * nc);

    double eps = T.lum / (double)o->nphot;
    double q_unit = eps / (double)((int64_t)1 << ORC_EUNIT_SHIFT);
    Ctx X;
    X.G = &G; X.T = &T; X.rho = rho; X.mass = mass; X.wq = wq; X.qlo = qlo; X.qspan = qspan;
    X.E = energy; X.escape = escape; X.ccross = cell_crossings; X.q_unit = q_unit;
    X.Elate = Elate; X.late_after = o->sequential ? 0 : o->late_after; X.pilot = 0;
    X.sequential = o->sequential; X.o = o;
    int64_t hist[10] = {0}, maxev = 0;
    X.hist = stats ? hist : NULL;
    X.maxev = &maxev;
    int nthreads = o->nthreads;
#ifdef _OPENMP
    if (nthreads <= 0) nthreads = omp_get_max_threads();
#else
    nthreads = 1;
#endif
    Cnt tot;
    memset(&tot, 0, sizeof(tot));
    int64_t N = o->nphot;
    if (o->sequential) {
        run_range(&X, 0, N, 0u, &tot, 1);
    } else {
        int K = o->nepoch < 1 ? 1 : o->nepoch;
        while (K > 1 && (N >> (K - 1)) == 0) K--;
        int64_t* bnd = malloc(sizeof(int64_t) * (K + 1));
        bnd[0] = 0;
        for (int k = 1; k <= K; ++k) bnd[k] = N >> (K - k);
        /* first epoch: pilot passes estimate its own deposits */
        Cnt junk;
        memset(&junk, 0, sizeof(junk));
        for (int pass = o->npilot; pass >= 0; --pass) {
            for (size_t i = 0; i < n; ++i) {
                qlo[i] = 0.0f;
                qspan[i] = (mass[i] > 0.0) ? (float)((double)D[i] * q_unit / mass[i]) : 0.0f;
            }
            if (pass > 0) {
                memset(D, 0, sizeof(int64_t) * n);
                Ctx P = X;
                P.E = D; P.escape = NULL; P.ccross = NULL; P.hist = NULL; P.pilot = 1;
                run_range(&P, bnd[0], bnd[1], (uint32_t)pass, &junk, nthreads);
            } else {
                run_range(&X, bnd[0], bnd[1], 0u, &tot, nthreads);
            }
        }
        for (int k = 1; k < K; ++k) {
            if (bnd[k + 1] <= bnd[k]) continue;
            double R = (double)bnd[k + 1] / (double)bnd[k];
            for (size_t i = 0; i < n; ++i) {
                if (mass[i] > 0.0) {
                    qlo[i] = (float)((double)energy[i] * q_unit / mass[i]);
                    qspan[i] = (float)((double)energy[i] * q_unit * (R - 1.0) / mass[i]);
                } else {
                    qlo[i] = 0.0f;
                    qspan[i] = 0.0f;
                }
            }
            run_range(&X, bnd[k], bnd[k + 1], 0u, &tot, nthreads);
        }
        free(bnd);
    }
    for (size_t i = 0; i < n; ++i) energy[i] += Elate[i];
    if (temperature)
        for (int s = 0; s < ns; ++s)
            for (int cc = 0; cc < nc; ++cc) {
                size_t i = (size_t)s * nc + cc;
                temperature[i] = invert_temperature(&T, s, energy[i], mass[i], q_unit);
            }
    if (stats) {
        stats->packets = N;
        stats->killed = tot.killed; stats->escaped = tot.escaped; stats->crossings = tot.crossings;
        stats->events = tot.events; stats->absorptions = tot.absorptions;
        stats->scatterings = tot.scatterings; stats->mrw_steps = tot.mrw;
        stats->max_packet_events = maxev;
        for (int b = 0; b < 10; ++b) stats->events_hist[b] = hist[b];
    }
    free(mass); free(wq); free(qlo); free(qspan); free(D); free(Elate);
    free_tables(&T);
    orc__free_geo(&G);
    return 0;
}
