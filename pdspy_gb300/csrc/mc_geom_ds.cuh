// Double-single geometry of the thermal Monte Carlo: packet positions, safety distances
// and wall-intersection roots in pairs of floats (hi + lo, 48-bit significand) on the
// FP32 pipe.
//
// Why not FP64: on GB300 every FP64 instruction occupies a sub-partition's FP64 unit for
// 64 cycles (a dependent DFMA or DADD takes 64 cycles even with one active lane, DDIV about
// 550 and DSQRT about 600), and the SM retires about 2 FP64 lane operations per cycle
// against 128 FP32 ones.  A packet walk is a dependent chain of geometry, so FP64 set
// both the latency of long random walks and the throughput of the bulk.  The pair
// arithmetic keeps the property FP64 was there for: the quantities that cancel near a
// wall (r^2 - R^2, the cone quadric z^2 - mu^2 r^2, the phi-plane offsets) are formed to
// about 2^-46 of their operands, so a packet sitting on a wall is still placed on the
// correct side to far below a mean free path.
//
// Root solves: each candidate wall is solved in single precision from the precise
// constant term (the stable quadratic forms), the earliest exit is selected, and that one
// root is refined by one Newton step whose residual is evaluated in double-single, which
// puts the crossing point on the wall to about 2^-46 of its radius.  The safety distance
// keeps the relative margin of the double-precision version (4e-6).
//
// The CPU oracle (oracle/mcrt_oracle.c) evaluates the same sequence of IEEE single
// operations, so the two implementations take identical decisions.
#pragma once
#include <stdint.h>

#include "mc_common.h"
#include "mc_device.cuh"
#include "mc_geom.cuh"

namespace pdgpu {

struct ds {
    float h, l;
};

// |a| >= |b| (or a == 0): exact sum as hi + lo.
__device__ __forceinline__ ds ds_fast2(float a, float b) {
    float s = a + b;
    float e = b - (s - a);
    return ds{s, e};
}
__device__ __forceinline__ ds ds_add(ds a, ds b) {
    float s = a.h + b.h;
    float v = s - a.h;
    float e = (a.h - (s - v)) + (b.h - v);
    e = e + (a.l + b.l);
    return ds_fast2(s, e);
}
__device__ __forceinline__ ds ds_neg(ds a) { return ds{-a.h, -a.l}; }
__device__ __forceinline__ ds ds_sub(ds a, ds b) { return ds_add(a, ds_neg(b)); }
__device__ __forceinline__ ds ds_prod(float a, float b) {
    float p = a * b;
    return ds{p, __fmaf_rn(a, b, -p)};
}
__device__ __forceinline__ ds ds_mulf(ds a, float b) {
    float p = a.h * b;
    float e = __fmaf_rn(a.h, b, -p);
    e = __fmaf_rn(a.l, b, e);
    return ds_fast2(p, e);
}
__device__ __forceinline__ ds ds_mul(ds a, ds b) {
    float p = a.h * b.h;
    float e = __fmaf_rn(a.h, b.h, -p);
    e = __fmaf_rn(a.h, b.l, e);
    e = __fmaf_rn(a.l, b.h, e);
    return ds_fast2(p, e);
}
__device__ __forceinline__ ds ds_sqr(ds a) {
    float p = a.h * a.h;
    float e = __fmaf_rn(a.h, a.h, -p);
    e = __fmaf_rn(a.h + a.h, a.l, e);
    return ds_fast2(p, e);
}
// a + s k (one coordinate of a move)
__device__ __forceinline__ ds ds_move(ds a, float s, float k) { return ds_add(a, ds_prod(s, k)); }
// a + (s.h + s.l) k, the lo term only when present
__device__ __forceinline__ ds ds_move2(ds a, ds s, float k) {
    ds r = ds_move(a, s.h, k);
    return s.l != 0.0f ? ds_add(r, ds_prod(s.l, k)) : r;
}

struct PktS {
    ds x, y, z;
    float dsafe;    // lower bound of the distance to every wall of the cell
    float dmax;     // upper bound of the distance to the nearest wall (3e38: unknown)
    int fresh;      // dsafe was computed at the current position
    float kx, ky, kz, tau;
    int ir, itv, ip, lam;
    int last_wall, cell_events;
    int nevents, ncross;
    int m, epoch;
    McRng rng;
};

// Float-pool wall tables of one model.  The geometry below reads walls through the
// accessors (sphere i: rh, r2; virtual cone j: mu, sn, mu2; phi half-plane k: cp, sp), so
// a walk can also run on a copy of its current cell's walls held in registers (WallsCell).
struct WallsS {
    const float *RH, *RL, *R2H, *R2L;    // sphere radii and squared radii (hi, lo)
    const float *MU, *SN, *MU2H, *MU2L;  // cone cos, sin and cos^2 (hi, lo), virtual index
    const float *CP, *SP;                // phi half-plane cos, sin
    __device__ __forceinline__ WallsS(const McModel& M, const float* __restrict__ fg)
        : RH(fg + M.off_rf), RL(fg + M.off_rl), R2H(fg + M.off_r2h), R2L(fg + M.off_r2l),
          MU(fg + M.off_muf), SN(fg + M.off_snf), MU2H(fg + M.off_mu2h), MU2L(fg + M.off_mu2l),
          CP(fg + M.off_cphf), SP(fg + M.off_sphf) {}
    __device__ __forceinline__ float rh(int i) const { return RH[i]; }
    __device__ __forceinline__ ds r2(int i) const { return ds{R2H[i], R2L[i]}; }
    __device__ __forceinline__ float mu(int j) const { return MU[j]; }
    __device__ __forceinline__ float sn(int j) const { return SN[j]; }
    __device__ __forceinline__ ds mu2(int j) const { return ds{MU2H[j], MU2L[j]}; }
    __device__ __forceinline__ float cp(int k) const { return CP[k]; }
    __device__ __forceinline__ float sp(int k) const { return SP[k]; }
};

// The walls of one cell (spheres ir and ir + 1, virtual cones itv and itv + 1, phi
// half-planes ip and ip + 1) copied into registers; the accessors take the same indices
// as WallsS and select the cached value, so the geometry computes identical results.
struct WallsCell {
    int i0, j0, k0;
    float rh0, rh1, mu0, mu1, sn0, sn1, cp0, cp1, sp0, sp1;
    ds r20, r21, mu20, mu21;
    __device__ __forceinline__ void load(const WallsS& W, int ir, int itv, int ip, int np) {
        i0 = ir; j0 = itv; k0 = ip;
        if (ir >= 0) { rh0 = W.rh(ir); r20 = W.r2(ir); } else { rh0 = 0.0f; r20 = ds{0.0f, 0.0f}; }
        rh1 = W.rh(ir + 1); r21 = W.r2(ir + 1);
        mu0 = W.mu(itv); sn0 = W.sn(itv); mu20 = W.mu2(itv);
        mu1 = W.mu(itv + 1); sn1 = W.sn(itv + 1); mu21 = W.mu2(itv + 1);
        if (np > 1) { cp0 = W.cp(ip); sp0 = W.sp(ip); cp1 = W.cp(ip + 1); sp1 = W.sp(ip + 1); }
        else { cp0 = sp0 = cp1 = sp1 = 0.0f; }
    }
    __device__ __forceinline__ float rh(int i) const { return i == i0 ? rh0 : rh1; }
    __device__ __forceinline__ ds r2(int i) const { return i == i0 ? r20 : r21; }
    __device__ __forceinline__ float mu(int j) const { return j == j0 ? mu0 : mu1; }
    __device__ __forceinline__ float sn(int j) const { return j == j0 ? sn0 : sn1; }
    __device__ __forceinline__ ds mu2(int j) const { return j == j0 ? mu20 : mu21; }
    __device__ __forceinline__ float cp(int k) const { return k == k0 ? cp0 : cp1; }
    __device__ __forceinline__ float sp(int k) const { return k == k0 ? sp0 : sp1; }
};

// Quantities shared by the wall candidates of one step.
struct FrameS {
    ds x, y, z, z2, r2, b;
    float kx, ky, kz, kk, bf, tol;
    int last;
};

template <class Wl>
__device__ __forceinline__ void frame_ds(const McModel& M, const Wl& W, const PktS& p,
                                         FrameS& f) {
    f.x = p.x; f.y = p.y; f.z = p.z;
    f.kx = p.kx; f.ky = p.ky; f.kz = p.kz;
    f.kk = (f.kx * f.kx + f.ky * f.ky) + f.kz * f.kz;
    ds rho2 = ds_add(ds_sqr(f.x), ds_sqr(f.y));
    f.z2 = ds_sqr(f.z);
    f.r2 = ds_add(rho2, f.z2);
    f.b = ds_add(ds_add(ds_mulf(f.x, f.kx), ds_mulf(f.y, f.ky)), ds_mulf(f.z, f.kz));
    f.bf = f.b.h;
    f.last = p.last_wall;
    float Ro = W.rh((p.ir < 0) ? 0 : p.ir + 1);
    f.tol = 1.0e-10f * Ro;
}

__device__ __forceinline__ bool accept_root_s(float s, int wall, int last, float tol, float& out) {
    if (wall == last) {
        if (s > tol) { out = s; return true; }
        return false;
    }
    if (s >= -tol) { out = s > 0.0f ? s : 0.0f; return true; }
    return false;
}

// Coefficients of the cone quadric Q(s) = A s^2 + 2 B s + C = z(s)^2 - mu^2 r(s)^2.
template <class Wl>
__device__ __forceinline__ void cone_coef(const Wl& W, const FrameS& f, int w, float& A,
                                          float& B, float& C) {
    ds mu2 = W.mu2(w);
    A = f.kz * f.kz - mu2.h * f.kk;
    B = ds_sub(ds_mulf(f.z, f.kz), ds_mul(mu2, f.b)).h;
    C = ds_sub(f.z2, ds_mul(mu2, f.r2)).h;
}

// Exit distance through wall candidate k (0 outer sphere, 1 inner sphere, 2 lower cone,
// 3 upper cone, 4 lower phi half-plane, 5 upper phi half-plane), before refinement.
template <class Wl>
__device__ inline bool candidate_ds(const McModel& M, const Wl& W, const PktS& p,
                                    const FrameS& f, int k, float& out) {
    const float kk = f.kk, bf = f.bf, tol = f.tol;
    const int last = f.last;
    if (k == 0) {
        int io = (p.ir < 0) ? 0 : p.ir + 1;
        float c = ds_sub(f.r2, W.r2(io)).h;
        float D = bf * bf - kk * c;
        if (D < 0.0f) D = 0.0f;
        float sq = sqrtf(D);
        float s = (bf <= 0.0f) ? (sq - bf) / kk : -c / (bf + sq);
        if (last == W_ROUT && s <= tol) return false;
        out = (s > 0.0f) ? s : 0.0f;
        return true;
    }
    if (p.ir < 0) return false;
    if (k == 1) {
        if (!(bf < 0.0f)) return false;
        float c = ds_sub(f.r2, W.r2(p.ir)).h;
        float D = bf * bf - kk * c;
        if (!(D >= 0.0f)) return false;
        float s = c / (sqrtf(D) - bf);
        return accept_root_s(s, W_RIN, last, tol, out);
    }
    if (k == 2 || k == 3) {
        const int side = k - 2;
        int w = p.itv + side;
        if (w == 0 || w == M.ntv) return false;
        int code = side ? W_THI : W_TLO;
        float mu = W.mu(w);
        float s = 0.0f;
        bool ok = false;
        if (mu == 0.0f) {
            if (side == 0 ? (f.kz > 0.0f) : (f.kz < 0.0f)) { s = -f.z.h / f.kz; ok = true; }
        } else {
            float A, B, C;
            cone_coef(W, f, w, A, B, C);
            bool want_plus = (side == 0) ? (mu > 0.0f) : (mu < 0.0f);
            float D = B * B - A * C;
            if (D >= 0.0f) {
                float sq = sqrtf(D);
                if (A == 0.0f) {
                    if (want_plus ? (B > 0.0f) : (B < 0.0f)) { s = -C / (2.0f * B); ok = true; }
                } else {
                    float q = (B >= 0.0f) ? -(B + sq) : (sq - B);
                    if (q != 0.0f) {
                        float sm, sp;
                        if (B >= 0.0f) { sm = q / A; sp = C / q; }
                        else { sp = q / A; sm = C / q; }
                        s = want_plus ? sp : sm;
                        ok = true;
                    }
                }
                if (ok) {
                    float zs = f.z.h + s * f.kz;
                    if (mu > 0.0f ? (zs < 0.0f) : (zs > 0.0f)) ok = false;
                }
            }
        }
        return ok && accept_root_s(s, code, last, tol, out);
    }
    if (M.np <= 1) return false;
    if (k == 4) {
        int k0 = p.ip;
        float g0 = ds_add(ds_mulf(f.x, -W.sp(k0)), ds_mulf(f.y, W.cp(k0))).h;
        float dg = -f.kx * W.sp(k0) + f.ky * W.cp(k0);
        if (!(dg < 0.0f)) return false;
        float s = -g0 / dg;
        float hx = f.x.h + s * f.kx, hy = f.y.h + s * f.ky;
        return hx * W.cp(k0) + hy * W.sp(k0) > 0.0f && accept_root_s(s, W_PLO, last, tol, out);
    }
    int k1 = p.ip + 1;
    float h0 = ds_add(ds_mulf(f.x, W.sp(k1)), ds_mulf(f.y, -W.cp(k1))).h;
    float dh = f.kx * W.sp(k1) - f.ky * W.cp(k1);
    if (!(dh < 0.0f)) return false;
    float s = -h0 / dh;
    float hx = f.x.h + s * f.kx, hy = f.y.h + s * f.ky;
    return hx * W.cp(k1) + hy * W.sp(k1) > 0.0f && accept_root_s(s, W_PHI, last, tol, out);
}

// One Newton step on the selected wall: the residual of the wall equation at x + s k in
// double-single over its single-precision derivative.  The step is taken only when it is
// a small correction (a root of another branch is never jumped to).  The refined distance
// is returned as a pair (s - correction): a single float cannot place the packet on the
// wall (its spacing at 1e12 cm is 1e5 cm).  The result is >= 0.
// Residual f and derivative f' of wall candidate k's equation at distance sd along the ray.
template <class Wl>
__device__ __forceinline__ void wall_residual(const McModel& M, const Wl& W, const PktS& p,
                                              const FrameS& f, int k, ds sd, float& fv,
                                              float& fd) {
    const float s = sd.h;
    ds X = ds_move2(f.x, sd, f.kx), Y = ds_move2(f.y, sd, f.ky), Z = ds_move2(f.z, sd, f.kz);
    fv = 0.0f;
    fd = 0.0f;
    if (k == 0 || k == 1) {
        int i = (k == 1) ? p.ir : ((p.ir < 0) ? 0 : p.ir + 1);
        ds r2 = ds_add(ds_add(ds_sqr(X), ds_sqr(Y)), ds_sqr(Z));
        fv = ds_sub(r2, W.r2(i)).h;
        fd = 2.0f * (f.bf + s * f.kk);
    } else if (k == 2 || k == 3) {
        int w = p.itv + (k - 2);
        if (W.mu(w) == 0.0f) {
            fv = Z.h;
            fd = f.kz;
        } else {
            float A, B, C;
            cone_coef(W, f, w, A, B, C);
            ds r2 = ds_add(ds_add(ds_sqr(X), ds_sqr(Y)), ds_sqr(Z));
            fv = ds_sub(ds_sqr(Z), ds_mul(W.mu2(w), r2)).h;
            fd = 2.0f * (B + A * s);
        }
    } else if (k == 4) {
        int k0 = p.ip;
        fv = ds_add(ds_mulf(X, -W.sp(k0)), ds_mulf(Y, W.cp(k0))).h;
        fd = -f.kx * W.sp(k0) + f.ky * W.cp(k0);
    } else {
        int k1 = p.ip + 1;
        fv = ds_add(ds_mulf(X, W.sp(k1)), ds_mulf(Y, -W.cp(k1))).h;
        fd = f.kx * W.sp(k1) - f.ky * W.cp(k1);
    }
}

// Newton refinement of candidate k's single-precision root s, the residual evaluated in
// pairs.  A first correction larger than 1e-6 s (a near-tangent crossing, where the
// single-precision root is poorly conditioned) is followed by a second step.
template <class Wl>
__device__ inline ds refine_ds(const McModel& M, const Wl& W, const PktS& p,
                               const FrameS& f, int k, float s) {
    float fv, fd;
    wall_residual(M, W, p, f, k, ds{s, 0.0f}, fv, fd);
    if (fd != 0.0f) {
        float d = fv / fd;
        if (fabsf(d) <= 1.0e-3f * s + f.tol) {
            ds r = ds_fast2(s, -d);
            if (fabsf(d) > 1.0e-6f * s && r.h > 0.0f) {
                wall_residual(M, W, p, f, k, r, fv, fd);
                if (fd != 0.0f) {
                    float d2 = fv / fd;
                    if (fabsf(d2) <= fabsf(d)) r = ds_add(r, ds{-d2, 0.0f});
                }
            }
            return r.h > 0.0f ? r : ds{0.0f, 0.0f};
        }
    }
    return ds{s > 0.0f ? s : 0.0f, 0.0f};
}

__device__ __forceinline__ int cand_wall_code(int k) {
    return k == 0 ? W_ROUT : k == 1 ? W_RIN : k == 2 ? W_TLO : k == 3 ? W_THI : k == 4 ? W_PLO : W_PHI;
}

// Distance to the wall through which the packet leaves its cell: the first candidate (in
// the order above) with the smallest exit distance, refined.
template <class Wl>
__device__ inline ds next_wall_ds(const McModel& M, const Wl& W, const PktS& p,
                                  int& wall_out) {
    FrameS f;
    frame_ds(M, W, p, f);
    float best = 3.0e38f;
    int bk = -1;
    const int nk = (p.ir < 0) ? 1 : (M.np > 1 ? 6 : 4);
    for (int k = 0; k < nk; ++k) {
        float s;
        if (candidate_ds(M, W, p, f, k, s) && s < best) {
            best = s;
            bk = k;
        }
    }
    if (bk < 0) {
        wall_out = W_NONE;
        return ds{3.0e38f, 0.0f};
    }
    wall_out = cand_wall_code(bk);
    return refine_ds(M, W, p, f, bk, best);
}

// The same wall solve for a packet inside the grid (ir >= 0) with a compile-time candidate
// count (4 without phi walls, 6 with): the candidates are independent, so unrolled they
// are evaluated side by side; the selection is the same (first smallest distance).
template <int NK, class Wl>
__device__ __forceinline__ ds next_wall_ds_n(const McModel& M, const Wl& W, const PktS& p,
                                             int& wall_out) {
    FrameS f;
    frame_ds(M, W, p, f);
    float sk[NK];
    bool ok[NK];
#pragma unroll
    for (int k = 0; k < NK; ++k) ok[k] = candidate_ds(M, W, p, f, k, sk[k]);
    float best = 3.0e38f;
    int bk = -1;
#pragma unroll
    for (int k = 0; k < NK; ++k)
        if (ok[k] && sk[k] < best) {
            best = sk[k];
            bk = k;
        }
    if (bk < 0) {
        wall_out = W_NONE;
        return ds{3.0e38f, 0.0f};
    }
    wall_out = cand_wall_code(bk);
    return refine_ds(M, W, p, f, bk, best);
}

// Virtual theta wall j lies at or below the packet's polar angle (cos theta_j >= z / r),
// decided from the sign of z^2 - mu_j^2 r^2 in double-single.
template <class Wl>
__device__ __forceinline__ bool mu_ge_ds(const Wl& W, int j, const ds& z, const ds& z2,
                                         const ds& r2) {
    float mu = W.mu(j);
    float Q = ds_sub(z2, ds_mul(W.mu2(j), r2)).h;
    if (mu >= 0.0f) return z.h <= 0.0f || Q <= 0.0f;
    return z.h < 0.0f && Q >= 0.0f;
}

// Azimuth of the packet at or beyond phi wall k: the half-turn (sin phi < 0, or sin 0 and
// cos < 0) and, within a half-turn, the sign of the plane function.
template <class Wl>
__device__ __forceinline__ bool phi_ge_ds(const Wl& W, int k, const ds& x, const ds& y) {
    int hp = (y.h < 0.0f || (y.h == 0.0f && x.h < 0.0f)) ? 1 : 0;
    float sw = W.sp(k), cw = W.cp(k);
    int hw = (sw < 0.0f || (sw == 0.0f && cw < 0.0f)) ? 1 : 0;
    if (hp != hw) return hp > hw;
    return ds_add(ds_mulf(x, -sw), ds_mulf(y, cw)).h >= 0.0f;
}

// Angular cell of a packet entering the grid through its inner sphere.
template <class Wl>
__device__ inline void locate_angles_ds(const McModel& M, const Wl& W, PktS& p) {
    ds z2 = ds_sqr(p.z);
    ds r2 = ds_add(ds_add(ds_sqr(p.x), ds_sqr(p.y)), z2);
    int lo = 0, hi = M.ntv;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (mu_ge_ds(W, mid, p.z, z2, r2)) lo = mid; else hi = mid;
    }
    p.itv = lo;
    if (M.np > 1) {
        int a = 0, b = M.np;
        while (b - a > 1) {
            int mid = a + (b - a) / 2;
            if (phi_ge_ds(W, mid, p.x, p.y)) a = mid; else b = mid;
        }
        p.ip = a;
    } else {
        p.ip = 0;
    }
}

__device__ __forceinline__ int cell_of_s(const McModel& M, const PktS& p) {
    int it = (p.itv < M.nt) ? p.itv : (2 * M.nt - 1 - p.itv);
    return (p.ir * M.nt + it) * M.np + p.ip;
}

// Lower bound of the distance from the packet to every wall of its cell (the safety
// distance and the MRW sphere radius).  The cancelling differences are formed in
// double-single, the non-cancelling factors (r + R, |rho cos| + |z sin|) in single
// precision; relative margin 4e-6.
template <class Wl>
__device__ inline float wall_distance_ds(const McModel& M, const Wl& W, const PktS& p) {
    ds x2 = ds_sqr(p.x), y2 = ds_sqr(p.y), z2 = ds_sqr(p.z);
    ds rho2 = ds_add(x2, y2);
    ds r2 = ds_add(rho2, z2);
    float rf = sqrtf(r2.h);
    float d = ds_sub(r2, W.r2(p.ir)).h / (rf + W.rh(p.ir));
    float d2 = ds_sub(W.r2(p.ir + 1), r2).h / (rf + W.rh(p.ir + 1));
    if (d2 < d) d = d2;
    float rhof = sqrtf(rho2.h);
    float zf = p.z.h;
    for (int side = 0; side < 2; ++side) {
        int w = p.itv + side;
        if (w == 0 || w == M.ntv) continue;
        float a = rhof * W.mu(w);
        float b = zf * W.sn(w);
        float dt;
        if ((a > 0.0f) == (b > 0.0f)) {
            float num = ds_sub(ds_mul(W.mu2(w), r2), z2).h;
            float den = fabsf(a) + fabsf(b);
            dt = den > 0.0f ? fabsf(num) / den : 0.0f;
        } else {
            dt = fabsf(a) + fabsf(b);
        }
        if (dt < d) d = dt;
    }
    if (M.np > 1) {
        int k0 = p.ip, k1 = p.ip + 1;
        float d0 = fabsf(ds_add(ds_mulf(p.x, -W.sp(k0)), ds_mulf(p.y, W.cp(k0))).h);
        float d1 = fabsf(ds_add(ds_mulf(p.x, W.sp(k1)), ds_mulf(p.y, -W.cp(k1))).h);
        if (d0 < d) d = d0;
        if (d1 < d) d = d1;
    }
    float m = d * (1.0f - 4.0e-6f);
    return m > 0.0f ? m : 0.0f;
}

// The same lower bound computed by a whole warp, one wall per lane (0 inner sphere, 1 outer
// sphere, 2-3 cones, 4-5 phi half-planes) and reduced with min, which gives exactly the
// value of wall_distance_ds.  Every lane returns the result.
template <class Wl>
__device__ inline float wall_distance_ds_warp(const McModel& M, const Wl& W, const PktS& p,
                                              int lane) {
    float d = 3.0e38f;
    if (lane < 6) {
        ds x2 = ds_sqr(p.x), y2 = ds_sqr(p.y), z2 = ds_sqr(p.z);
        ds rho2 = ds_add(x2, y2);
        ds r2 = ds_add(rho2, z2);
        if (lane < 2) {
            float rf = sqrtf(r2.h);
            if (lane == 0) d = ds_sub(r2, W.r2(p.ir)).h / (rf + W.rh(p.ir));
            else d = ds_sub(W.r2(p.ir + 1), r2).h / (rf + W.rh(p.ir + 1));
        } else if (lane < 4) {
            int w = p.itv + (lane - 2);
            if (w != 0 && w != M.ntv) {
                float rhof = sqrtf(rho2.h);
                float a = rhof * W.mu(w);
                float b = p.z.h * W.sn(w);
                if ((a > 0.0f) == (b > 0.0f)) {
                    float num = ds_sub(ds_mul(W.mu2(w), r2), z2).h;
                    float den = fabsf(a) + fabsf(b);
                    d = den > 0.0f ? fabsf(num) / den : 0.0f;
                } else {
                    d = fabsf(a) + fabsf(b);
                }
            }
        } else if (M.np > 1) {
            if (lane == 4) {
                int k0 = p.ip;
                d = fabsf(ds_add(ds_mulf(p.x, -W.sp(k0)), ds_mulf(p.y, W.cp(k0))).h);
            } else {
                int k1 = p.ip + 1;
                d = fabsf(ds_add(ds_mulf(p.x, W.sp(k1)), ds_mulf(p.y, -W.cp(k1))).h);
            }
        }
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) {
        float e = __shfl_xor_sync(0xffffffffu, d, o);
        if (e < d) d = e;
    }
    d = __shfl_sync(0xffffffffu, d, 0);
    float m = d * (1.0f - 4.0e-6f);
    return m > 0.0f ? m : 0.0f;
}

}  // namespace pdgpu
