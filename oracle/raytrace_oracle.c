/*
 * CPU oracle of the ray-traced images (test infrastructure only; see raytrace_oracle.h).
 *
 * Camera.  The observer direction is o = (sin i sin phi, -sin i cos phi, cos i); the image
 * axes are ex = (cos phi, sin phi, 0) and ey = (-cos i sin phi, cos i cos phi, sin i), so
 * incl = 0 looks down the z axis and incl = 90 deg sees the disk edge-on along ex.  A sky
 * position (X, Y) maps to image coordinates (u, v) = (X cos pa + Y sin pa,
 * -X sin pa + Y cos pa).  Pixel (px, py) is centred at ((px - nx/2) d, (py - ny/2) d), so
 * the origin falls on the centre of pixel (nx/2, ny/2) as with pdspy's zoomau
 * (pdspy/modeling/Model.py:522-527).
 *
 * Refinement.  A pixel whose closest approach to the origin is b_min gets level
 * L = min{L : d 2^-L <= f s(b_min)} (capped), s(b) = min(radial width of the cell at
 * radius max(b, r_in), max(b, r_in) * min theta width); its 4^L sub-rays are averaged.
 */
#include "raytrace_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "mc_internal.h"

#define PI_D 3.14159265358979323846

typedef struct {
    double o[3], ex[3], ey[3];
    double cpa, spa, d;
    int nx, ny;
} Cam;

static void make_cam(const orc_camera* c, Cam* C) {
    double i = c->incl_deg * PI_D / 180.0, f = c->phi_deg * PI_D / 180.0;
    double pa = c->pa_deg * PI_D / 180.0;
    double si = sin(i), ci = cos(i), sf = sin(f), cf = cos(f);
    C->o[0] = si * sf; C->o[1] = -si * cf; C->o[2] = ci;
    C->ex[0] = cf; C->ex[1] = sf; C->ex[2] = 0.0;
    C->ey[0] = -ci * sf; C->ey[1] = ci * cf; C->ey[2] = si;
    C->cpa = cos(pa); C->spa = sin(pa);
    C->d = c->pixel_cm;
    C->nx = c->npix_x; C->ny = c->npix_y;
}

static int refine_level(const Geo* G, const orc_camera* c, int px, int py, double dth_min) {
    double d = c->pixel_cm;
    double X = (double)(px - c->npix_x / 2) * d, Y = (double)(py - c->npix_y / 2) * d;
    double ax = fabs(X) - 0.5 * d, ay = fabs(Y) - 0.5 * d;
    if (ax < 0.0) ax = 0.0;
    if (ay < 0.0) ay = 0.0;
    double b = sqrt(ax * ax + ay * ay);
    if (b < G->r[0]) b = G->r[0];
    if (b >= G->r[G->nr]) return 0;
    int lo = 0, hi = G->nr;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (G->r[mid] <= b) lo = mid; else hi = mid;
    }
    double s = G->r[lo + 1] - G->r[lo];
    double st = b * dth_min;
    if (st < s) s = st;
    double lim = c->refine_factor * s;
    int L = 0;
    double w = d;
    while (L < c->max_refine && w > lim) {
        w = w * 0.5;
        L = L + 1;
    }
    return L;
}

static double min_theta_width(const orc_grid* g) {
    double m = 1e30;
    for (int j = 0; j < g->nt; ++j) {
        double w = g->th_edges[j + 1] - g->th_edges[j];
        if (w < m) m = w;
    }
    return m;
}

void orc_refine_levels(const orc_grid* grid, const orc_camera* cam, int* levels) {
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return; }
    double dth = min_theta_width(grid);
    for (int py = 0; py < cam->npix_y; ++py)
        for (int px = 0; px < cam->npix_x; ++px)
            levels[py * cam->npix_x + px] = refine_level(&G, cam, px, py, dth);
    orc__free_geo(&G);
}

/* Start a packet-like ray at image position (u, v), travelling towards -o.  Returns 0 if
 * the ray misses the grid. */
static int ray_start(const Geo* G, const Cam* C, double u, double v, Pkt* p) {
    memset(p, 0, sizeof(*p));
    double Rm = G->r[G->nr];
    double D = 1.01 * Rm;
    p->x = u * C->ex[0] + v * C->ey[0] + D * C->o[0];
    p->y = u * C->ex[1] + v * C->ey[1] + D * C->o[1];
    p->z = u * C->ex[2] + v * C->ey[2] + D * C->o[2];
    p->kx = (float)(-C->o[0]);
    p->ky = (float)(-C->o[1]);
    p->kz = (float)(-C->o[2]);
    double kx = (double)p->kx, ky = (double)p->ky, kz = (double)p->kz;
    double kk = kx * kx + ky * ky + kz * kz;
    double b = p->x * kx + p->y * ky + p->z * kz;
    double r2 = p->x * p->x + p->y * p->y + p->z * p->z;
    double c = r2 - Rm * Rm;
    double D2 = b * b - kk * c;
    if (!(D2 > 0.0) || b >= 0.0) return 0;
    double s = c / (sqrt(D2) - b);   /* near root of the outer sphere */
    p->x = fma(s, kx, p->x);
    p->y = fma(s, ky, p->y);
    p->z = fma(s, kz, p->z);
    p->ir = G->nr - 1;
    orc__locate_angles(G, p);
    p->last_wall = W_ROUT;
    return 1;
}

/* Walk one ray: callback per segment (cell, length). */
typedef void (*seg_fn)(void* ctx, int cell, double len);

static void ray_walk(const Geo* G, Pkt* p, seg_fn fn, void* ctx) {
    for (int guard = 0; guard < 10000000; ++guard) {
        int wall;
        double sw = orc__next_wall(G, p, &wall);
        if (p->ir >= 0) fn(ctx, orc__cell_index(G, p), sw);
        p->x = fma(sw, (double)p->kx, p->x);
        p->y = fma(sw, (double)p->ky, p->y);
        p->z = fma(sw, (double)p->kz, p->z);
        switch (wall) {
            case W_ROUT:
                if (p->ir < 0) { p->ir = 0; orc__locate_angles(G, p); }
                else p->ir += 1;
                p->last_wall = W_RIN;
                if (p->ir >= G->nr) return;
                break;
            case W_RIN: p->ir -= 1; p->last_wall = W_ROUT; break;
            case W_TLO: p->itv -= 1; p->last_wall = W_THI; break;
            case W_THI: p->itv += 1; p->last_wall = W_TLO; break;
            case W_PLO: p->ip = (p->ip == 0) ? G->np - 1 : p->ip - 1; p->last_wall = W_PHI; break;
            case W_PHI: p->ip = (p->ip == G->np - 1) ? 0 : p->ip + 1; p->last_wall = W_PLO; break;
            default: return;
        }
    }
}

typedef struct {
    int nlam, ncell;
    const float* alpha;
    const float* S;
    double* I;
    double* W;
} RtCtx;

static void rt_seg(void* vctx, int c, double len) {
    RtCtx* X = (RtCtx*)vctx;
    for (int l = 0; l < X->nlam; ++l) {
        double a = (double)X->alpha[(size_t)l * X->ncell + c];
        double dt = a * len;
        double one_m_e = -expm1(-dt);
        X->I[l] += X->W[l] * (double)X->S[(size_t)l * X->ncell + c] * one_m_e;
        X->W[l] *= exp(-dt);
    }
}

typedef struct {
    int nlam, ncell;
    const float* alpha;
    double* tau;
} TauCtx;

static void tau_seg(void* vctx, int c, double len) {
    TauCtx* X = (TauCtx*)vctx;
    for (int l = 0; l < X->nlam; ++l) X->tau[l] += (double)X->alpha[(size_t)l * X->ncell + c] * len;
}

static void sub_uv(const Cam* C, int px, int py, int sub, int L, double* u, double* v) {
    int n = 1 << L;
    int a = sub % n, b = sub / n;
    double X = (double)(px - C->nx / 2) * C->d + (((double)a + 0.5) / (double)n - 0.5) * C->d;
    double Y = (double)(py - C->ny / 2) * C->d + (((double)b + 0.5) / (double)n - 0.5) * C->d;
    *u = X * C->cpa + Y * C->spa;
    *v = -X * C->spa + Y * C->cpa;
}

int orc_image(const orc_grid* grid, int nlam, const float* alpha, const float* S,
              const double* star_flux, const orc_camera* cam, double* image) {
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return 1; }
    Cam C;
    make_cam(cam, &C);
    double dth = min_theta_width(grid);
    int nx = cam->npix_x, ny = cam->npix_y;
    double* I = malloc(sizeof(double) * nlam);
    double* W = malloc(sizeof(double) * nlam);
    double* acc = malloc(sizeof(double) * nlam);
    for (int py = 0; py < ny; ++py)
        for (int px = 0; px < nx; ++px) {
            int L = refine_level(&G, cam, px, py, dth);
            int nsub = 1 << (2 * L);
            for (int l = 0; l < nlam; ++l) acc[l] = 0.0;
            for (int sub = 0; sub < nsub; ++sub) {
                double u, v;
                sub_uv(&C, px, py, sub, L, &u, &v);
                for (int l = 0; l < nlam; ++l) { I[l] = 0.0; W[l] = 1.0; }
                Pkt p;
                if (ray_start(&G, &C, u, v, &p)) {
                    RtCtx X = {nlam, G.ncell, alpha, S, I, W};
                    ray_walk(&G, &p, rt_seg, &X);
                }
                for (int l = 0; l < nlam; ++l) acc[l] += I[l];
            }
            for (int l = 0; l < nlam; ++l)
                image[((size_t)l * ny + py) * nx + px] = acc[l] / (double)nsub;
        }
    if (!cam->nostar && star_flux) {
        /* star: attenuation from the origin towards the observer */
        double* tau = calloc(nlam, sizeof(double));
        Pkt p;
        memset(&p, 0, sizeof(p));
        p.kx = (float)C.o[0]; p.ky = (float)C.o[1]; p.kz = (float)C.o[2];
        p.ir = -1;
        p.last_wall = W_NONE;
        TauCtx X = {nlam, G.ncell, alpha, tau};
        ray_walk(&G, &p, tau_seg, &X);
        double pc = 3.085677581e18;
        double omega = (cam->pixel_cm / pc) * (cam->pixel_cm / pc);
        int cx = nx / 2, cy = ny / 2;
        for (int l = 0; l < nlam; ++l)
            image[((size_t)l * ny + cy) * nx + cx] += star_flux[l] * exp(-tau[l]) / omega;
        free(tau);
    }
    free(I); free(W); free(acc);
    orc__free_geo(&G);
    return 0;
}

typedef struct {
    int* cells;
    double* lengths;
    int n, cap;
} SegCtx;

static void seg_collect(void* vctx, int c, double len) {
    SegCtx* X = (SegCtx*)vctx;
    if (X->n < X->cap) {
        X->cells[X->n] = c;
        X->lengths[X->n] = len;
    }
    X->n += 1;
}

int orc_ray_segments(const orc_grid* grid, const orc_camera* cam, int px, int py, int sub,
                     int level, int* cells, double* lengths, int cap) {
    Geo G;
    if (orc__make_geo(grid, &G)) { orc__free_geo(&G); return -1; }
    Cam C;
    make_cam(cam, &C);
    Pkt p;
    SegCtx X = {cells, lengths, 0, cap};
    if (sub < 0) {
        /* the star's line of sight: from the origin towards the observer */
        memset(&p, 0, sizeof(p));
        p.kx = (float)C.o[0]; p.ky = (float)C.o[1]; p.kz = (float)C.o[2];
        p.ir = -1;
        p.last_wall = W_NONE;
        ray_walk(&G, &p, seg_collect, &X);
    } else {
        double u, v;
        sub_uv(&C, px, py, sub, level, &u, &v);
        if (ray_start(&G, &C, u, v, &p)) ray_walk(&G, &p, seg_collect, &X);
    }
    orc__free_geo(&G);
    return X.n;
}
