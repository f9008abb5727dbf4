// Device geometry of the spherical grid shared by the thermal Monte Carlo and the ray
// tracer: wall-intersection root solves in double precision, angle location and the
// cell index of a packet or ray.
//
// Walls are spheres r = r_i, cones theta = theta_j (virtual full-sphere index for grids
// mirrored about the equator) and half-planes phi = phi_k.  The exit root of each quadric
// is selected by the sign of the quadric's derivative, so the root that leaves the
// current cell is taken and the wall just entered (last_wall) is never re-crossed at
// zero distance.
#pragma once
#include <stdint.h>

#include "mc_common.h"
#include "mc_device.cuh"

namespace pdgpu {

enum { W_NONE = 0, W_RIN = 1, W_ROUT = 2, W_TLO = 3, W_THI = 4, W_PLO = 5, W_PHI = 6 };

struct Pkt {
    double x, y, z;
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


__device__ __forceinline__ bool accept_root(double s, int wall, int last, double tol, double& out) {
    if (wall == last) {
        if (s > tol) { out = s; return true; }
        return false;
    }
    if (s >= -tol) { out = s > 0.0 ? s : 0.0; return true; }
    return false;
}

// Quantities shared by the wall candidates of one step.
struct WallFrame {
    double x, y, z, kx, ky, kz, kk, r2, b, tol;
    int last;
};

__device__ __forceinline__ void wall_frame(const McModel& M, const double* __restrict__ dp,
                                           const Pkt& p, WallFrame& f) {
    const double* R = dp + M.off_r;
    f.x = p.x; f.y = p.y; f.z = p.z;
    f.kx = (double)p.kx; f.ky = (double)p.ky; f.kz = (double)p.kz;
    f.kk = f.kx * f.kx + f.ky * f.ky + f.kz * f.kz;
    f.r2 = f.x * f.x + f.y * f.y + f.z * f.z;
    f.b = f.x * f.kx + f.y * f.ky + f.z * f.kz;
    f.last = p.last_wall;
    double Ro = (p.ir < 0) ? R[0] : R[p.ir + 1];
    f.tol = 1.0e-10 * Ro;
}

// Exit distance through wall candidate k (0 outer sphere, 1 inner sphere, 2 lower cone,
// 3 upper cone, 4 lower phi half-plane, 5 upper phi half-plane), FP64.  Returns false if
// the packet cannot leave through that wall.
__device__ inline bool wall_candidate(const McModel& M, const double* __restrict__ dp,
                                      const Pkt& p, const WallFrame& f, int k, double& out) {
    const double x = f.x, y = f.y, z = f.z, kx = f.kx, ky = f.ky, kz = f.kz;
    const double kk = f.kk, r2 = f.r2, b = f.b, tol = f.tol;
    const int last = f.last;
    const double* R = dp + M.off_r;
    if (k == 0) {
        double Ro = (p.ir < 0) ? R[0] : R[p.ir + 1];
        double c = r2 - Ro * Ro;
        double D = b * b - kk * c;
        if (D < 0.0) D = 0.0;
        double sq = sqrt(D);
        double s = (b <= 0.0) ? (sq - b) / kk : -c / (b + sq);
        if (last == W_ROUT && s <= tol) return false;
        out = (s > 0.0) ? s : 0.0;
        return true;
    }
    if (p.ir < 0) return false;
    if (k == 1) {
        if (!(b < 0.0)) return false;
        double Ri = R[p.ir];
        double c = r2 - Ri * Ri;
        double D = b * b - kk * c;
        if (!(D >= 0.0)) return false;
        double s = c / (sqrt(D) - b);
        return accept_root(s, W_RIN, last, tol, out);
    }
    if (k == 2 || k == 3) {
        const int side = k - 2;
        int w = p.itv + side;
        if (w == 0 || w == M.ntv) return false;
        int code = side ? W_THI : W_TLO;
        double mu = dp[M.off_mu + w];
        double s = 0.0;
        bool ok = false;
        if (mu == 0.0) {
            if (side == 0 ? (kz > 0.0) : (kz < 0.0)) { s = -z / kz; ok = true; }
        } else {
            double mu2 = mu * mu;
            double A = kz * kz - mu2 * kk;
            double B = z * kz - mu2 * b;
            double C = z * z - mu2 * r2;
            bool want_plus = (side == 0) ? (mu > 0.0) : (mu < 0.0);
            double D = B * B - A * C;
            if (D >= 0.0) {
                double sq = sqrt(D);
                if (A == 0.0) {
                    if (want_plus ? (B > 0.0) : (B < 0.0)) { s = -C / (2.0 * B); ok = true; }
                } else {
                    double q = (B >= 0.0) ? -(B + sq) : (sq - B);
                    if (q != 0.0) {
                        double sm, sp;
                        if (B >= 0.0) { sm = q / A; sp = C / q; }
                        else { sp = q / A; sm = C / q; }
                        s = want_plus ? sp : sm;
                        ok = true;
                    }
                }
                if (ok) {
                    double zs = z + s * kz;
                    if (mu > 0.0 ? (zs < 0.0) : (zs > 0.0)) ok = false;
                }
            }
        }
        return ok && accept_root(s, code, last, tol, out);
    }
    if (M.np <= 1) return false;
    const double* CP = dp + M.off_cph;
    const double* SP = dp + M.off_sph;
    if (k == 4) {
        int k0 = p.ip;
        double g0 = -x * SP[k0] + y * CP[k0];
        double dg = -kx * SP[k0] + ky * CP[k0];
        if (!(dg < 0.0)) return false;
        double s = -g0 / dg;
        double hx = x + s * kx, hy = y + s * ky;
        return hx * CP[k0] + hy * SP[k0] > 0.0 && accept_root(s, W_PLO, last, tol, out);
    }
    int k1 = p.ip + 1;
    double h0 = x * SP[k1] - y * CP[k1];
    double dh = kx * SP[k1] - ky * CP[k1];
    if (!(dh < 0.0)) return false;
    double s = -h0 / dh;
    double hx = x + s * kx, hy = y + s * ky;
    return hx * CP[k1] + hy * SP[k1] > 0.0 && accept_root(s, W_PHI, last, tol, out);
}

__device__ __forceinline__ int wall_code(int k) {
    return k == 0 ? W_ROUT : k == 1 ? W_RIN : k == 2 ? W_TLO : k == 3 ? W_THI : k == 4 ? W_PLO : W_PHI;
}

// Distance to the wall through which the packet leaves its cell: the first candidate (in
// the order above) with the smallest exit distance.
__device__ inline double next_wall(const McModel& M, const double* __restrict__ dp, const Pkt& p,
                                   int& wall_out) {
    WallFrame f;
    wall_frame(M, dp, p, f);
    double best = 1.0e300;
    int bw = W_NONE;
    const int nk = (p.ir < 0) ? 1 : (M.np > 1 ? 6 : 4);
    for (int k = 0; k < nk; ++k) {
        double s;
        if (wall_candidate(M, dp, p, f, k, s) && s < best) {
            best = s;
            bw = wall_code(k);
        }
    }
    wall_out = bw;
    return best;
}

__device__ inline void locate_angles(const McModel& M, const double* __restrict__ dp, Pkt& p) {
    double x = p.x, y = p.y, z = p.z;
    double r = sqrt(x * x + y * y + z * z);
    double ct = z / r;
    const double* MU = dp + M.off_mu;
    int lo = 0, hi = M.ntv;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (MU[mid] >= ct) lo = mid; else hi = mid;
    }
    p.itv = lo;
    if (M.np > 1) {
        double ph = atan2(y, x);
        if (ph < 0.0) ph += 2.0 * MC_PI;
        const double* PH = dp + M.off_vp + M.np;  // phi edges follow the phi widths
        int a = 0, bnd = M.np;
        while (bnd - a > 1) {
            int mid = a + (bnd - a) / 2;
            if (PH[mid] <= ph) a = mid; else bnd = mid;
        }
        p.ip = a;
    } else {
        p.ip = 0;
    }
}

__device__ __forceinline__ int cell_of(const McModel& M, const Pkt& p) {
    int it = (p.itv < M.nt) ? p.itv : (2 * M.nt - 1 - p.itv);
    return (p.ir * M.nt + it) * M.np + p.ip;
}

// Lower bound of the distance from the packet to every wall of its cell (the safety
// distance and the MRW sphere radius).  The small differences that cancel near a wall
// (r^2 - R^2, the cone quadric rho^2 cos^2 - z^2 sin^2, the phi-plane offsets) are formed
// in double precision from the double position; only non-cancelling factors (r + R,
// |rho cos| + |z sin|) use single precision.  Relative error below 1e-6, relative margin
// 4e-6; no square root or division runs in double precision.
__device__ inline float wall_distance(const McModel& M, const double* __restrict__ dp,
                               const float* __restrict__ fg, const Pkt& p) {
    double x = p.x, y = p.y, z = p.z;
    double x2 = x * x, y2 = y * y, z2 = z * z;
    double rho2 = x2 + y2;
    double r2 = rho2 + z2;
    float rf = sqrtf((float)r2);
    const double* R = dp + M.off_r;
    const float* RF = fg + M.off_rf;
    double Ri = R[p.ir], Ro = R[p.ir + 1];
    float d = (float)(r2 - Ri * Ri) / (rf + RF[p.ir]);
    float d2 = (float)(Ro * Ro - r2) / (rf + RF[p.ir + 1]);
    if (d2 < d) d = d2;
    float rhof = sqrtf((float)rho2);
    float zf = (float)z;
    const double* MU = dp + M.off_mu;
    const double* SN = dp + M.off_sn;
    const float* MUF = fg + M.off_muf;
    const float* SNF = fg + M.off_snf;
    for (int side = 0; side < 2; ++side) {
        int w = p.itv + side;
        if (w == 0 || w == M.ntv) continue;
        float a = rhof * MUF[w];
        float b = zf * SNF[w];
        float dt;
        if ((a > 0.0f) == (b > 0.0f)) {
            double mu = MU[w], sn = SN[w];
            double num = rho2 * (mu * mu) - z2 * (sn * sn);
            float den = fabsf(a) + fabsf(b);
            dt = den > 0.0f ? fabsf((float)num) / den : 0.0f;
        } else {
            dt = fabsf(a) + fabsf(b);
        }
        if (dt < d) d = dt;
    }
    if (M.np > 1) {
        const double* CP = dp + M.off_cph;
        const double* SP = dp + M.off_sph;
        int k0 = p.ip, k1 = p.ip + 1;
        float d0 = (float)fabs(-x * SP[k0] + y * CP[k0]);
        float d1 = (float)fabs(x * SP[k1] - y * CP[k1]);
        if (d0 < d) d = d0;
        if (d1 < d) d = d1;
    }
    float m = d * (1.0f - 4.0e-6f);
    return m > 0.0f ? m : 0.0f;
}


}  // namespace pdgpu
