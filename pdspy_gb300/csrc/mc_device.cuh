// Device building blocks of the thermal Monte Carlo: counter-based random numbers,
// the single-precision math the walk uses, direction sampling and table searches.
//
// Every expression is written out operation by operation and the translation unit is
// compiled with --fmad=false, so that each floating-point operation is one IEEE
// operation.  The CPU oracle evaluates the same sequence, which makes a GPU run and an
// oracle run with the same seed consume identical random numbers and take identical
// decisions.
#pragma once
#include <stdint.h>

#include "mc_common.h"

#define PHILOX_M0 0xD2511F53u
#define PHILOX_M1 0xCD9E8D57u
#define PHILOX_W0 0x9E3779B9u
#define PHILOX_W1 0xBB67AE85u

// Philox4x32-10 (Salmon, Moraes, Dror, Shaw, SC'11).
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint32_t k0, uint32_t k1) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t lo0 = PHILOX_M0 * c.x;
        uint32_t hi0 = __umulhi(PHILOX_M0, c.x);
        uint32_t lo1 = PHILOX_M1 * c.z;
        uint32_t hi1 = __umulhi(PHILOX_M1, c.z);
        uint4 n;
        n.x = hi1 ^ c.y ^ k0;
        n.y = lo1;
        n.z = hi0 ^ c.w ^ k1;
        n.w = lo0;
        c = n;
        k0 += PHILOX_W0;
        k1 += PHILOX_W1;
    }
    return c;
}

// Uniform in (0,1): 23 random bits as an odd multiple of 2^-24 (exact in float).
__device__ __forceinline__ float mc_u01(uint32_t x) {
    return (float)(((x >> 9) << 1) | 1u) * 5.9604644775390625e-08f;
}

// ln(x) for normal positive floats: x = 2^e m with m in (sqrt(1/2), sqrt(2)];
// ln m = 2 atanh(t), t = (m-1)/(m+1), by the atanh power series to t^9.
__device__ __forceinline__ float mc_logf(float x) {
    uint32_t bits = __float_as_uint(x);
    int e = (int)((bits >> 23) & 0xffu) - 127;
    float m = __uint_as_float((bits & 0x007fffffu) | 0x3f800000u);
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

// exp(-x) for x >= 0 (0 beyond x = 87): x = n ln2 + r with |r| <= ln2 / 2 (Cody & Waite's
// two-part ln2, hi part with 8 trailing zero bits so n * hi is exact), e^-r by its Taylor
// series to r^7 (truncation below 6e-9 relative), times 2^-n built from the exponent bits.
__device__ __forceinline__ float mc_expm(float x) {
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
    return p * __uint_as_float((uint32_t)(127 - n) << 23);
}

// (1 - exp(-x)) / x for x >= 0: its series to x^5 below 0.1 (truncation below 2e-10),
// the difference above.
__device__ __forceinline__ float mc_expm_frac(float x, float e) {
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

// Cube root of x in (0, 1]: a first guess from the exponent bits (one third of the
// biased exponent and mantissa, offset so the guess is within a few percent), then four
// Newton steps y <- (2 y + x / y^2) / 3.
__device__ __forceinline__ float mc_cbrt01(float x) {
    uint32_t b = __float_as_uint(x);
    float y = __uint_as_float(b / 3u + 709921077u);
#pragma unroll
    for (int i = 0; i < 4; ++i) y = (2.0f * y + x / (y * y)) * 0.333333343f;
    return y;
}

// sin and cos of 2 pi u, u in (0,1): nearest quarter turn plus Taylor series of sin (to
// x^9) and cos (to x^8) on |x| <= pi/4.
__device__ __forceinline__ void mc_sincospif2(float u, float& sn, float& cs) {
    float a = 2.0f * u;
    int n = (int)(a * 2.0f + 0.5f);
    float r = a - (float)n * 0.5f;
    float x = r * 3.14159265f;
    float x2 = x * x;
    float sp = 2.7557319e-06f;
    sp = sp * x2 - 1.9841270e-04f;
    sp = sp * x2 + 8.3333333e-03f;
    sp = sp * x2 - 1.6666667e-01f;
    float sx = x + x * (x2 * sp);
    float cp = 2.4801587e-05f;
    cp = cp * x2 - 1.3888889e-03f;
    cp = cp * x2 + 4.1666668e-02f;
    cp = cp * x2 - 0.5f;
    float cx = 1.0f + x2 * cp;
    switch (n & 3) {
        case 0: sn = sx; cs = cx; break;
        case 1: sn = cx; cs = -sx; break;
        case 2: sn = -sx; cs = -cx; break;
        default: sn = -cx; cs = sx; break;
    }
}

// Per-packet random numbers.  Every interaction of a packet owns its own Philox blocks:
// counter (n, packet, model, pass tag | stream << 24), key = seed, with n the index of the
// interaction in the packet's life.  Streams: 0 = albedo test, new optical depth, direction
// cosine, azimuth; 1 = reemission q', reemission row, reemission CDF, species; 2 = MRW
// diffusion time, jump cosine, jump azimuth; 3 (n = 0) = the emission.  A warp can
// therefore draw the numbers of future interactions without knowing what happened before
// them.
enum { MC_RS_EVENT = 0, MC_RS_SECOND = 1, MC_RS_MRW = 2, MC_RS_EMIT = 3 };

struct McRng {
    uint32_t pid, model, tag;
};

__device__ __forceinline__ uint4 mc_block(const McRng& r, uint32_t n, uint32_t stream, uint32_t k0,
                                          uint32_t k1) {
    return philox4x32_10(make_uint4(n, r.pid, r.model, r.tag | (stream << 24)), k0, k1);
}

// Rotate unit vector k by polar cosine mu and azimuth (cp, sp) about itself.
__device__ __forceinline__ void mc_rotate(float& kx, float& ky, float& kz, float mu, float cp,
                                          float sp) {
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    float ax = kx, ay = ky, az = kz;
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
    kx = nx * rn;
    ky = ny * rn;
    kz = nz * rn;
}

// Energy a packet has deposited itself, per (species, cell), in a four-entry cache
// (round-robin replacement).  The reemission temperature and the MRW mean opacities of a
// cell are taken at the epoch's snapshot plus the packet's own deposits there: in
// sequential Bjorkman & Wood a packet trapped in an optically thick cell heats the cell it
// reemits from, and the epoch snapshot alone cannot see deposits made after it was taken.
// The cache holds the last four cells, which covers a packet trapped at a wall or corner
// between cells.  Keys are species * ncell + cell within the model; units are the int64
// fixed-point deposits.  ver counts the deposits recorded (it keys per-cell caches of
// values derived from the cell temperature).
#define MC_OWN 4
struct McOwn {
    int32_t sc[MC_OWN];
    long long u[MC_OWN];
    int32_t next, ver;
};

__device__ __forceinline__ void own_init(McOwn& o) {
#pragma unroll
    for (int i = 0; i < MC_OWN; ++i) { o.sc[i] = -1; o.u[i] = 0; }
    o.next = 0;
    o.ver = 0;
}

__device__ __forceinline__ void own_add(McOwn& o, int sc, long long units) {
    o.ver += 1;
    bool hit = false;
#pragma unroll
    for (int i = 0; i < MC_OWN; ++i)
        if (o.sc[i] == sc) { o.u[i] += units; hit = true; }
    if (!hit) {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i)
            if (i == o.next) { o.sc[i] = sc; o.u[i] = units; }
        o.next = (o.next + 1) & (MC_OWN - 1);
    }
}

// The packet's own deposits in (species, cell) sc as energy per gram per second:
// (float) units * wq, with wq = (float)(q_unit / cell mass); 0 when not cached.
__device__ __forceinline__ float own_q(const McOwn& o, int sc, float wq) {
    long long u = 0;
#pragma unroll
    for (int i = 0; i < MC_OWN; ++i)
        if (o.sc[i] == sc) u = o.u[i];
    return u != 0 ? (float)u * wq : 0.0f;
}

// Upper bound of the distance to the nearest wall of the cell, kept along the walk: set
// from a computed wall distance D (which is a lower bound within a relative 5e-6), grown
// by every move (triangle inequality, rounded up), unknown after a crossing.
#define MC_DMAX_UNKNOWN 3.0e38f
__device__ __forceinline__ float mc_dmax_of(float D) { return D * 1.00001f; }
__device__ __forceinline__ float mc_dmax_after(float dmax, float step) {
    return dmax < MC_DMAX_UNKNOWN ? (dmax + step) * 1.000001f : MC_DMAX_UNKNOWN;
}

// Smallest index l with cdf[l] > u (cdf[n-1] == 1 > u).
__device__ __forceinline__ int mc_cdf_search(const float* cdf, int n, float u) {
    int lo = -1, hi = n - 1;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (cdf[mid] > u) hi = mid; else lo = mid;
    }
    return hi;
}

// Fractional reemission row of q on the increasing row table F[MC_NROW].
__device__ __forceinline__ void mc_row_search(const float* F, float q, int& j, float& w) {
    if (q < F[0]) {
        j = 0;
        w = 0.0f;
    } else if (q >= F[MC_NROW - 1]) {
        j = MC_NROW - 2;
        w = 1.0f;
    } else {
        int lo = 0, hi = MC_NROW - 1;
        while (hi - lo > 1) {
            int mid = lo + (hi - lo) / 2;
            if (F[mid] <= q) lo = mid; else hi = mid;
        }
        j = lo;
        w = (q - F[j]) / (F[j + 1] - F[j]);
        if (w < 0.0f) w = 0.0f;
        if (w > 1.0f) w = 1.0f;
    }
}
