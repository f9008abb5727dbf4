// Shared constants and plain-old-data layouts of the thermal Monte Carlo (host + device).
//
// The table geometry below is part of the algorithm: reemission rows, inversion rows and
// the diffusion-time table of the modified random walk.  The CPU oracle uses the same
// values so that both implementations consume identical tables.
#pragma once
#include <stdint.h>

#define MC_NROW 128
#define MC_TROW_LO 1.0
#define MC_TROW_HI 1.0e4
#define MC_NINV 4096
#define MC_TINV_LO 1.0e-2
#define MC_TINV_HI 1.0e5
#define MC_NMRW 1024
#define MC_EUNIT_SHIFT 20
#define MC_MAX_SPEC 4
#define MC_MAX_EPOCH 24
#define MC_NSTAT 256
#define MC_LSTAT 32     // per-launch slots from here, MC_LSTRIDE each: (t_start, t_end,
                        // max events, parked, interactions, crossings, deposits)
#define MC_LSTRIDE 8
#define MC_MAX_LAUNCH 24
// static shared memory of the continuation kernel's batched walks: 17 fields x 32 lanes
// of 4 bytes per warp, 8 warps per block of at most 256 threads
#define MC_TAIL_SMEM (8 * 17 * 32 * 4)

// pdspy physical constants (pdspy/constants/physics.py:1-15).
#define MC_C_LIGHT 2.99792458e10
#define MC_H_PLANCK 6.6260755e-27
#define MC_K_BOLTZ 1.380658e-16
#define MC_PI 3.14159265358979323846

// Stats slots (int64) in the workspace.
enum {
    ST_PACKETS = 0, ST_KILLED, ST_ESCAPED, ST_CROSSINGS, ST_EVENTS, ST_ABSORB, ST_SCATTER,
    ST_MRW, ST_STATUS, ST_T0, ST_STOP, ST_LATE, ST_PARKED, ST_DRAINED
};

// Per-model device descriptor.  Offsets index the plan's double/float pools and the
// concatenated cell arrays ([model][spec][cell]).
struct McModel {
    int32_t nr, nt, np, ntv;     // cells; ntv = virtual theta cells (2 nt when mirrored)
    int32_t ncell, mirror;
    int64_t cell_off;            // first element of this model in [model][spec][cell]
    int32_t off_r, off_mu, off_sn, off_cph, off_sph, off_vr, off_vt, off_vp;  // dpool
    int32_t off_star;            // fpool offset of the stellar CDF [nlam]
    int32_t off_rf, off_muf, off_snf, off_cphf, off_sphf;  // fpool: float wall copies
    int32_t off_rl, off_r2h, off_r2l, off_mu2h, off_mu2l;  // fpool: double-single walls
    int32_t model_id;
    double q_unit;               // erg/s per fixed-point unit
    double lum;                  // erg/s
    int64_t nphot;
    int64_t bnd[MC_MAX_EPOCH + 1];
};
