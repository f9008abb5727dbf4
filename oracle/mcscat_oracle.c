/*
 * CPU oracle of the monochromatic scattering Monte Carlo (test infrastructure only, see
 * mcrt_oracle.h): the mean intensity J per cell and camera wavelength that the
 * scattering source of pdspy's image and spectrum runs needs (the Monte Carlo RADMC-3D
 * runs inside "radmc3d image" / "radmc3d spectrum" and as "radmc3d mcscat",
 * pdspy/modeling/Model.py:258-322, :515-577, :608-650; nphot_scat / nphot_spec and
 * mc_scat_maxtauabs written by pdspy/radmc3d/write.py:33-38, :141-142).
 *
 * RADMC-3D is not available, so this restates the method from the literature:
 *   - Lucy 1999 (A&A 344, 282): J from the sum of packet path lengths per cell;
 *   - absorption as a continuous weight: over a segment of length L with absorption
 *     coefficient a a packet of surviving fraction w contributes w (1 - e^-aL) / a and
 *     keeps w e^-aL; free paths are drawn in scattering optical depth;
 *   - isotropic scattering (pdspy writes no asymmetry parameter, Model.py:774-776);
 *   - a packet is dropped once the absorption depth of its path exceeds maxtauabs
 *     (RADMC-3D's mc_scat_maxtauabs), or after max_scatter scatterings;
 *   - sources: the stars at the origin and, when an emissivity is given, the thermal
 *     emission of every cell, chosen in proportion to their luminosities.
 *
 * The sequence of operations is the GPU's (pdspy_gb300/csrc/mcscat.cu) operation for
 * operation: the same random blocks, the same double-single walk (geom_ds.c), the same
 * single-precision exp / cube-root helpers, integer path sums with 2^32 units per radial
 * cell width and an integer cumulative luminosity, so J agrees bit for bit.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mc_internal.h"

#ifdef _OPENMP
#include <omp.h>
#endif

#define C_LIGHT 2.99792458e10
#define H_PLANCK 6.6260755e-27
#define K_BOLTZ 1.380658e-16
#define PI_D 3.14159265358979323846
#define SC_TAG 0x5Cu

enum { RS_EVENT = 0, RS_EMIT = 3 };

static inline float u01(uint32_t x) {
    return (float)(((x >> 9) << 1) | 1u) * 5.9604644775390625e-08f;
}

static inline float bits_float(uint32_t b) {
    float f;
    memcpy(&f, &b, sizeof(f));
    return f;
}
static inline uint32_t float_bits(float f) {
    uint32_t b;
    memcpy(&b, &f, sizeof(b));
    return b;
}

/* exp(-x), x >= 0: Cody-Waite reduction by ln2 (two-part constant) and the Taylor series
 * of e^-r to r^7; 0 beyond x = 87. */
float orc_expm(float x) {
    if (!(x < 87.0f)) return 0.0f;
    int n = (int)(x * 1.44269504f + 0.5f);
    float r = (x - (float)n * 0.693145751953125f) - (float)n * 1.42860677e-06f;
    float p = -1.98412698e-04f;
    p = p * r + 1.38888889e-03f;
    p = p * r - 8.33333333e-03f;
    p = p * r + 4.16666667e-02f;
    p = p * r - 1.66666667e-01f;
    p = p * r + 0.5f;
    p = p * r - 1.0f;
    p = p * r + 1.0f;
    return p * bits_float((uint32_t)(127 - n) << 23);
}

/* (1 - exp(-x)) / x given e = exp(-x): series to x^5 below 0.1. */
float orc_expm_frac(float x, float e) {
    if (x < 0.1f) {
        float p = -1.38888889e-03f;
        p = p * x + 8.33333333e-03f;
        p = p * x - 4.16666667e-02f;
        p = p * x + 1.66666667e-01f;
        p = p * x - 0.5f;
        return p * x + 1.0f;
    }
    return (1.0f - e) / x;
}

/* Cube root on (0, 1]: exponent-bit guess and four Newton steps. */
float orc_cbrt01(float x) {
    float y = bits_float(float_bits(x) / 3u + 709921077u);
    for (int i = 0; i < 4; ++i) y = (2.0f * y + x / (y * y)) * 0.333333343f;
    return y;
}

static void block(const Pkt* p, uint32_t n, uint32_t stream, uint32_t o[4]) {
    uint32_t c[4];
    c[0] = n; c[1] = p->ctr[1]; c[2] = p->ctr[2]; c[3] = p->ctr[3] | (stream << 24);
    orc_philox4x32_10(c, p->key, o);
}

static int cdf_search(const float* cdf, int n, float u) {
    int lo = -1, hi = n - 1;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (cdf[mid] > u) hi = mid; else lo = mid;
    }
    return hi;
}

static double planck_nu(double nu, double T) {
    double x = H_PLANCK * nu / (K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double pre = 2.0 * H_PLANCK * nu * nu * nu / (C_LIGHT * C_LIGHT);
    return pre / expm1(x);
}

static double cell_volume(const Geo* G, int c) {
    int ir = c / (G->nt * G->np), it = (c / G->np) % G->nt, ip = c % G->np;
    return (G->Vr[ir] * G->Vt[it]) * G->Vp[ip];
}

typedef struct {
    const Geo* G;
    int nlam, ns;
    const float* kap;     /* [nlam][2][ns] */
    const float* rho;     /* [ns][ncell]   */
    const float* cdf;     /* [nlam][ncell] */
    const float* pstar;   /* [nlam]        */
    const float* phf;     /* [np+1]        */
    const float* invdr;   /* [nr]          */
    int64_t* acc;         /* [nlam][ncell] */
    int64_t nphot;
    uint32_t key[2];
    float maxtauabs;
    int max_scatter;
} SCtx;

typedef struct {
    int64_t escaped, dropped, capped, scatter, cross;
} SCnt;

static void emit(const SCtx* X, Pkt* p, int l) {
    const Geo* G = X->G;
    uint32_t e0[4], e1[4], e2[4];
    block(p, 0u, RS_EMIT, e0);
    block(p, 1u, RS_EMIT, e1);
    p->tau = -orc_logf(u01(e0[2]));
    {
        float mu = 2.0f * u01(e1[0]) - 1.0f;
        float sn, cs;
        orc_sincospif2(u01(e1[1]), &sn, &cs);
        float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
        p->kx = st * cs; p->ky = st * sn; p->kz = mu;
    }
    p->last_wall = W_NONE;
    p->nevents = 0;
    p->ncross = 0;
    if (u01(e0[0]) < X->pstar[l]) {
        p->sx.h = p->sx.l = p->sy.h = p->sy.l = p->sz.h = p->sz.l = 0.0f;
        p->ir = -1; p->itv = 0; p->ip = 0;
        return;
    }
    block(p, 2u, RS_EMIT, e2);
    int c = cdf_search(X->cdf + (size_t)l * G->ncell, G->ncell, u01(e0[1]));
    int ir = c / (G->nt * G->np), it = (c / G->np) % G->nt, ip = c % G->np;
    int itv = (G->mirror && u01(e0[3]) >= 0.5f) ? 2 * G->nt - 1 - it : it;
    float t0 = G->rf[ir] / G->rf[ir + 1];
    float a = t0 * t0 * t0;
    float r = orc_cbrt01(a + u01(e1[2]) * (1.0f - a)) * G->rf[ir + 1];
    float m0 = G->muf[itv + 1], m1 = G->muf[itv];
    float mu = m0 + u01(e1[3]) * (m1 - m0);
    float uphi = u01(e2[0]);
    if (G->np > 1) uphi = X->phf[ip] + uphi * (X->phf[ip + 1] - X->phf[ip]);
    float sp, cp;
    orc_sincospif2(uphi, &sp, &cp);
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    float rs = r * st;
    p->sx.h = rs * cp; p->sx.l = 0.0f;
    p->sy.h = rs * sp; p->sy.l = 0.0f;
    p->sz.h = r * mu; p->sz.l = 0.0f;
    p->ir = ir; p->itv = itv; p->ip = ip;
}

static void run_packet(const SCtx* X, int l, uint32_t pid, SCnt* cnt) {
    const Geo* G = X->G;
    const int ns = X->ns;
    const float* K = X->kap + (size_t)l * 2 * ns;
    Pkt p;
    memset(&p, 0, sizeof(p));
    p.ctr[1] = pid; p.ctr[2] = (uint32_t)l; p.ctr[3] = SC_TAG;
    p.key[0] = X->key[0]; p.key[1] = X->key[1];
    emit(X, &p, l);
    float w = 1.0f, tabs = 0.0f;
    for (;;) {
        int c = -1;
        float aa = 0.0f, as = 0.0f;
        if (p.ir >= 0) {
            c = orc__cell_index(G, &p);
            for (int s = 0; s < ns; ++s) {
                float r = X->rho[(size_t)s * G->ncell + c];
                aa = aa + r * K[s];
                as = as + r * K[ns + s];
            }
        }
        int wall = W_NONE;
        ds sw = orc__next_wall_ds(G, &p, &wall);
        float tw = as * sw.h;
        int scat = tw > p.tau;
        ds sl = sw;
        if (scat) {
            float se = p.tau / as;
            if (!(se > sw.h)) { sl.h = se; sl.l = 0.0f; }
        }
        float len = sl.h;
        if (c >= 0 && len > 0.0f) {
            float x = aa * len;
            float att = orc_expm(x);
            float d = w * (len * orc_expm_frac(x, att));
            float uf = d * X->invdr[p.ir] + 0.5f;
            if (uf >= 1.0f) {
                if (uf > 9.0e18f) uf = 9.0e18f;
                __atomic_fetch_add(&X->acc[(size_t)l * G->ncell + c], (int64_t)uf, __ATOMIC_RELAXED);
            }
            w = w * att;
            tabs = tabs + x;
        }
        orc__move_ds(&p, sl, p.kx, p.ky, p.kz);
        if (tabs > X->maxtauabs) { cnt->dropped += 1; return; }
        if (scat) {
            uint32_t n = (uint32_t)p.nevents;
            p.nevents += 1;
            cnt->scatter += 1;
            uint32_t b[4];
            block(&p, n, RS_EVENT, b);
            p.tau = -orc_logf(u01(b[0]));
            float mu = 2.0f * u01(b[1]) - 1.0f;
            float sn, cs;
            orc_sincospif2(u01(b[2]), &sn, &cs);
            float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
            p.kx = st * cs; p.ky = st * sn; p.kz = mu;
            p.last_wall = W_NONE;
            if (p.nevents >= X->max_scatter) { cnt->capped += 1; return; }
            continue;
        }
        p.tau = p.tau - tw;
        p.ncross += 1;
        cnt->cross += 1;
        switch (wall) {
            case W_ROUT:
                if (p.ir < 0) { p.ir = 0; orc__locate_angles_ds(G, &p); }
                else p.ir += 1;
                p.last_wall = W_RIN;
                if (p.ir >= G->nr) { cnt->escaped += 1; return; }
                break;
            case W_RIN: p.ir -= 1; p.last_wall = W_ROUT; break;
            case W_TLO: p.itv -= 1; p.last_wall = W_THI; break;
            case W_THI: p.itv += 1; p.last_wall = W_TLO; break;
            case W_PLO: p.ip = (p.ip == 0) ? G->np - 1 : p.ip - 1; p.last_wall = W_PHI; break;
            case W_PHI: p.ip = (p.ip == G->np - 1) ? 0 : p.ip + 1; p.last_wall = W_PLO; break;
            default: cnt->capped += 1; return;
        }
        if (p.ncross > 100000000) { cnt->capped += 1; return; }
    }
}

int orc_mcscat(const orc_grid* grid, int nlam, const double* lam_um, int nspec,
               const double* kabs, const double* ksca, const orc_stars* stars,
               const float* rho, const double* emis, const orc_scat_opts* o, double* J,
               int64_t* acc_out, orc_scat_stats* stats) {
    if (!grid || !lam_um || !kabs || !ksca || !rho || !o || !J || nlam < 1 || nspec < 1 ||
        o->nphot < 1)
        return 1;
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return 1; }
    const int ncell = G.ncell;
    const size_t ncl = (size_t)nlam * ncell;
    float* kap = malloc(sizeof(float) * (size_t)nlam * 2 * nspec);
    float* cdf = malloc(sizeof(float) * ncl);
    float* pstar = malloc(sizeof(float) * nlam);
    double* eps = malloc(sizeof(double) * nlam);
    float* phf = malloc(sizeof(float) * (grid->np + 1));
    float* invdr = malloc(sizeof(float) * grid->nr);
    int64_t* acc = calloc(ncl, sizeof(int64_t));
    for (int l = 0; l < nlam; ++l)
        for (int s = 0; s < nspec; ++s) {
            kap[((size_t)l * 2 + 0) * nspec + s] = (float)kabs[(size_t)s * nlam + l];
            kap[((size_t)l * 2 + 1) * nspec + s] = (float)ksca[(size_t)s * nlam + l];
        }
    for (int k = 0; k <= grid->np; ++k) phf[k] = (float)(grid->ph_edges[k] / (2.0 * PI_D));
    for (int i = 0; i < grid->nr; ++i)
        invdr[i] = (float)(4294967296.0 / (grid->r_edges[i + 1] - grid->r_edges[i]));
    int lg = 0;
    while (((int64_t)1 << lg) < (int64_t)ncell) ++lg;
    const double scale = ldexp(1.0, lg > 22 ? 62 - lg : 40);
    /* sources: stellar luminosity, cumulative thermal luminosity of the cells */
    for (int l = 0; l < nlam; ++l) {
        const double nu = C_LIGHT / (lam_um[l] * 1.0e-4);
        double ls = 0.0;
        if (stars)
            for (int k = 0; k < stars->nstar; ++k) {
                const double R = stars->radius_cm[k];
                ls = ls + 4.0 * PI_D * PI_D * R * R * planck_nu(nu, stars->temp_k[k]);
            }
        const double* e = emis ? emis + (size_t)l * ncell : NULL;
        double Lmax = 0.0;
        if (e)
            for (int c = 0; c < ncell; ++c) {
                double L = (e[c] * cell_volume(&G, c)) * (4.0 * PI_D);
                Lmax = fmax(Lmax, L);
            }
        uint64_t U = 0;
        uint64_t* units = malloc(sizeof(uint64_t) * ncell);
        for (int c = 0; c < ncell; ++c) {
            uint64_t u = 0;
            if (e) {
                double L = (e[c] * cell_volume(&G, c)) * (4.0 * PI_D);
                if (L > 0.0 && Lmax > 0.0) u = (uint64_t)(int64_t)((L / Lmax) * scale + 0.5);
            }
            units[c] = u;
            U += u;
        }
        uint64_t run = 0;
        for (int c = 0; c < ncell; ++c) {
            run += units[c];
            cdf[(size_t)l * ncell + c] = U > 0 ? (float)((double)run / (double)U) : 1.0f;
        }
        free(units);
        const double ld = (double)U * (Lmax / scale);
        const double lt = ls + ld;
        pstar[l] = lt > 0.0 ? (float)(ls / lt) : 1.0f;
        eps[l] = lt / (double)o->nphot;
    }
    SCtx X;
    X.G = &G; X.nlam = nlam; X.ns = nspec; X.kap = kap; X.rho = rho; X.cdf = cdf;
    X.pstar = pstar; X.phf = phf; X.invdr = invdr; X.acc = acc; X.nphot = o->nphot;
    X.key[0] = (uint32_t)(o->seed & 0xffffffffu);
    X.key[1] = (uint32_t)(o->seed >> 32);
    X.maxtauabs = o->maxtauabs > 0.0f ? o->maxtauabs : 30.0f;
    X.max_scatter = o->max_scatter > 0 ? o->max_scatter : 1000000;
    SCnt tot = {0, 0, 0, 0, 0};
    const int64_t total = (int64_t)nlam * o->nphot;
    int nth = o->nthreads;
#ifdef _OPENMP
    if (nth <= 0) nth = 0;
#pragma omp parallel num_threads(nth > 0 ? nth : omp_get_max_threads())
#endif
    {
        SCnt cnt = {0, 0, 0, 0, 0};
#ifdef _OPENMP
#pragma omp for schedule(dynamic, 256)
#endif
        for (int64_t g = 0; g < total; ++g) {
            int l = (int)(g / o->nphot);
            run_packet(&X, l, (uint32_t)(g - (int64_t)l * o->nphot), &cnt);
        }
#ifdef _OPENMP
#pragma omp critical
#endif
        {
            tot.escaped += cnt.escaped; tot.dropped += cnt.dropped; tot.capped += cnt.capped;
            tot.scatter += cnt.scatter; tot.cross += cnt.cross;
        }
    }
    for (size_t i = 0; i < ncl; ++i) {
        int l = (int)(i / ncell), c = (int)(i - (size_t)l * ncell);
        double v = 0.0;
        if (acc[i]) {
            int ir = c / (G.nt * G.np);
            v = (((double)acc[i] / (double)invdr[ir]) * eps[l]) / ((4.0 * PI_D) * cell_volume(&G, c));
        }
        J[i] = v;
    }
    if (acc_out) memcpy(acc_out, acc, sizeof(int64_t) * ncl);
    if (stats) {
        stats->packets = total;
        stats->escaped = tot.escaped;
        stats->dropped = tot.dropped;
        stats->capped = tot.capped;
        stats->scatterings = tot.scatter;
        stats->crossings = tot.cross;
    }
    free(kap); free(cdf); free(pstar); free(eps); free(phf); free(invdr); free(acc);
    orc__free_geo(&G);
    return 0;
}
