/*
 * Grid geometry shared by the thermal Monte Carlo and the ray-tracing oracle
 * (test infrastructure only, see mcrt_oracle.h).
 */
#ifndef PDSPY_ORACLE_INTERNAL_H
#define PDSPY_ORACLE_INTERNAL_H
#include <stdint.h>

#include "mcrt_oracle.h"

/* double-single number: value = h + l, |l| <= ulp(h) / 2 */
typedef struct {
    float h, l;
} ds;

typedef struct {
    int nr, nt, np, ntv, mirror, ncell;
    const double* r;       /* [nr+1]            */
    double* mu;            /* [ntv+1] cos of the virtual theta walls  */
    double* sn;            /* [ntv+1] sin of the virtual theta walls  */
    double* cph; double* sph; const double* ph;  /* [np+1]           */
    double* Vr; double* Vt; double* Vp;
    float* rf; float* muf; float* snf; float* cphf; float* sphf;  /* float copies */
    float* rl; float* r2h; float* r2l; float* mu2h; float* mu2l;   /* double-single walls */
} Geo;

typedef struct {
    double x, y, z;    /* position, FP64 geometry          */
    ds sx, sy, sz;     /* position, double-single geometry */
    float kx, ky, kz;
    int ir, itv, ip;
    int lam;
    float tau;
    int last_wall;
    int cell_events;
    int64_t nevents;
    int64_t ncross;
    float dsafe;       /* lower bound of the distance to every wall of the cell */
    float dmax;        /* upper bound of the distance to the nearest wall (ORC_DMAX_UNKNOWN) */
    int fresh;         /* dsafe was computed at the current position */
    uint32_t ctr[4];   /* [draw block, packet id, model, pass tag] */
    uint32_t key[2];
    uint32_t buf[4];
    uint32_t draw;
    int64_t own_sc[4];  /* own deposits: (species, cell) keys, round-robin cache */
    int64_t own_u[4];   /* units this packet deposited there                   */
    int own_next;
} Pkt;

enum { W_NONE = 0, W_RIN = 1, W_ROUT = 2, W_TLO = 3, W_THI = 4, W_PLO = 5, W_PHI = 6 };

int orc__make_geo(const orc_grid* g, Geo* G);
void orc__free_geo(Geo* G);
double orc__next_wall(const Geo* G, const Pkt* p, int* wall_out);
void orc__locate_angles(const Geo* G, Pkt* p);
int orc__cell_index(const Geo* G, const Pkt* p);

/* Double-single geometry (geom_ds.c): the same walk with positions and walls in pairs of
 * floats, evaluated operation for operation like the GPU's default geometry. */
ds orc__next_wall_ds(const Geo* G, const Pkt* p, int* wall_out);  /* refined, as a pair */
float orc__wall_distance_ds(const Geo* G, const Pkt* p);
void orc__locate_angles_ds(const Geo* G, Pkt* p);
void orc__move_ds(Pkt* p, ds s, float kx, float ky, float kz);

#endif
