/*
 * Double-single geometry of the thermal Monte Carlo oracle (test infrastructure only, see
 * mcrt_oracle.h): packet positions, safety distances and wall-intersection roots in pairs
 * of floats (value = hi + lo).
 *
 * This is the geometry the GPU runs by default.  Every expression below is the same
 * sequence of IEEE single-precision operations (compiled with -ffp-contract=off; fused
 * multiply-adds only where fmaf is written), so a packet walk here and on the GPU takes
 * identical decisions.
 *
 *  - Pair arithmetic: exact two-sum and two-product (Knuth; Dekker with a fused
 *    multiply-add) followed by a renormalising fast two-sum.
 *  - Quantities that cancel near a wall are formed in pairs: r^2 - R^2 for spheres,
 *    z^2 - mu^2 r^2 for cones and -x sin(phi) + y cos(phi) for half-planes.
 *  - Each candidate wall is solved in single precision from the precise constant term
 *    (the numerically stable quadratic forms); the earliest exit is taken (first
 *    candidate on ties) and refined by one Newton step whose residual is evaluated in
 *    pairs, which places the crossing on the wall to about 2^-46 of its radius.
 *  - The safety distance keeps a relative margin of 4e-6.
 */
#include <math.h>

#include "mc_internal.h"

static inline ds ds_fast2(float a, float b) {
    ds r;
    float s = a + b;
    r.h = s;
    r.l = b - (s - a);
    return r;
}
static inline ds ds_add(ds a, ds b) {
    float s = a.h + b.h;
    float v = s - a.h;
    float e = (a.h - (s - v)) + (b.h - v);
    e = e + (a.l + b.l);
    return ds_fast2(s, e);
}
static inline ds ds_neg(ds a) {
    ds r;
    r.h = -a.h;
    r.l = -a.l;
    return r;
}
static inline ds ds_sub(ds a, ds b) { return ds_add(a, ds_neg(b)); }
static inline ds ds_prod(float a, float b) {
    ds r;
    float p = a * b;
    r.h = p;
    r.l = fmaf(a, b, -p);
    return r;
}
static inline ds ds_mulf(ds a, float b) {
    float p = a.h * b;
    float e = fmaf(a.h, b, -p);
    e = fmaf(a.l, b, e);
    return ds_fast2(p, e);
}
static inline ds ds_mul(ds a, ds b) {
    float p = a.h * b.h;
    float e = fmaf(a.h, b.h, -p);
    e = fmaf(a.h, b.l, e);
    e = fmaf(a.l, b.h, e);
    return ds_fast2(p, e);
}
static inline ds ds_sqr(ds a) {
    float p = a.h * a.h;
    float e = fmaf(a.h, a.h, -p);
    e = fmaf(a.h + a.h, a.l, e);
    return ds_fast2(p, e);
}
static inline ds ds_move(ds a, float s, float k) { return ds_add(a, ds_prod(s, k)); }
static inline ds R2(const Geo* G, int i) {
    ds r;
    r.h = G->r2h[i];
    r.l = G->r2l[i];
    return r;
}
static inline ds MU2(const Geo* G, int j) {
    ds r;
    r.h = G->mu2h[j];
    r.l = G->mu2l[j];
    return r;
}

/* a + (s.h + s.l) k, the lo term only when present */
static inline ds ds_move2(ds a, ds s, float k) {
    ds r = ds_move(a, s.h, k);
    return s.l != 0.0f ? ds_add(r, ds_prod(s.l, k)) : r;
}

void orc__move_ds(Pkt* p, ds s, float kx, float ky, float kz) {
    p->sx = ds_move2(p->sx, s, kx);
    p->sy = ds_move2(p->sy, s, ky);
    p->sz = ds_move2(p->sz, s, kz);
}

typedef struct {
    ds x, y, z, z2, r2, b;
    float kx, ky, kz, kk, bf, tol;
    int last;
} Frame;

static void frame(const Geo* G, const Pkt* p, Frame* f) {
    f->x = p->sx; f->y = p->sy; f->z = p->sz;
    f->kx = p->kx; f->ky = p->ky; f->kz = p->kz;
    f->kk = (f->kx * f->kx + f->ky * f->ky) + f->kz * f->kz;
    ds rho2 = ds_add(ds_sqr(f->x), ds_sqr(f->y));
    f->z2 = ds_sqr(f->z);
    f->r2 = ds_add(rho2, f->z2);
    f->b = ds_add(ds_add(ds_mulf(f->x, f->kx), ds_mulf(f->y, f->ky)), ds_mulf(f->z, f->kz));
    f->bf = f->b.h;
    f->last = p->last_wall;
    float Ro = G->rf[(p->ir < 0) ? 0 : p->ir + 1];
    f->tol = 1.0e-10f * Ro;
}

/* The wall the packet entered through needs a strictly positive distance; any other wall
 * accepts tiny negative roots (rounding) as zero. */
static int accept_root(float s, int wall, int last, float tol, float* out) {
    if (wall == last) {
        if (s > tol) { *out = s; return 1; }
        return 0;
    }
    if (s >= -tol) { *out = s > 0.0f ? s : 0.0f; return 1; }
    return 0;
}

/* Q(s) = A s^2 + 2 B s + C = z(s)^2 - mu^2 r(s)^2 */
static void cone_coef(const Geo* G, const Frame* f, int w, float* A, float* B, float* C) {
    ds mu2 = MU2(G, w);
    *A = f->kz * f->kz - mu2.h * f->kk;
    *B = ds_sub(ds_mulf(f->z, f->kz), ds_mul(mu2, f->b)).h;
    *C = ds_sub(f->z2, ds_mul(mu2, f->r2)).h;
}

/* Candidate k: 0 outer sphere, 1 inner sphere, 2 lower cone, 3 upper cone, 4 lower and
 * 5 upper phi half-plane. */
static int candidate(const Geo* G, const Pkt* p, const Frame* f, int k, float* out) {
    const float kk = f->kk, bf = f->bf, tol = f->tol;
    const int last = f->last;
    if (k == 0) {
        int io = (p->ir < 0) ? 0 : p->ir + 1;
        float c = ds_sub(f->r2, R2(G, io)).h;
        float D = bf * bf - kk * c;
        if (D < 0.0f) D = 0.0f;
        float sq = sqrtf(D);
        float s = (bf <= 0.0f) ? (sq - bf) / kk : -c / (bf + sq);
        if (last == W_ROUT && s <= tol) return 0;
        *out = (s > 0.0f) ? s : 0.0f;
        return 1;
    }
    if (p->ir < 0) return 0;
    if (k == 1) {
        if (!(bf < 0.0f)) return 0;
        float c = ds_sub(f->r2, R2(G, p->ir)).h;
        float D = bf * bf - kk * c;
        if (!(D >= 0.0f)) return 0;
        float s = c / (sqrtf(D) - bf);
        return accept_root(s, W_RIN, last, tol, out);
    }
    if (k == 2 || k == 3) {
        int side = k - 2;
        int w = p->itv + side;
        if (w == 0 || w == G->ntv) return 0;
        int code = side ? W_THI : W_TLO;
        float mu = G->muf[w];
        float s = 0.0f;
        int ok = 0;
        if (mu == 0.0f) {
            if (side == 0 ? (f->kz > 0.0f) : (f->kz < 0.0f)) { s = -f->z.h / f->kz; ok = 1; }
        } else {
            float A, B, C;
            cone_coef(G, f, w, &A, &B, &C);
            int want_plus = (side == 0) ? (mu > 0.0f) : (mu < 0.0f);
            float D = B * B - A * C;
            if (D >= 0.0f) {
                float sq = sqrtf(D);
                if (A == 0.0f) {
                    if (want_plus ? (B > 0.0f) : (B < 0.0f)) { s = -C / (2.0f * B); ok = 1; }
                } else {
                    float q = (B >= 0.0f) ? -(B + sq) : (sq - B);
                    if (q != 0.0f) {
                        float sm, sp;
                        if (B >= 0.0f) { sm = q / A; sp = C / q; }
                        else { sp = q / A; sm = C / q; }
                        s = want_plus ? sp : sm;
                        ok = 1;
                    }
                }
                if (ok) {
                    float zs = f->z.h + s * f->kz;
                    if (mu > 0.0f ? (zs < 0.0f) : (zs > 0.0f)) ok = 0;
                }
            }
        }
        return ok && accept_root(s, code, last, tol, out);
    }
    if (G->np <= 1) return 0;
    if (k == 4) {
        int k0 = p->ip;
        float g0 = ds_add(ds_mulf(f->x, -G->sphf[k0]), ds_mulf(f->y, G->cphf[k0])).h;
        float dg = -f->kx * G->sphf[k0] + f->ky * G->cphf[k0];
        if (!(dg < 0.0f)) return 0;
        float s = -g0 / dg;
        float hx = f->x.h + s * f->kx, hy = f->y.h + s * f->ky;
        return hx * G->cphf[k0] + hy * G->sphf[k0] > 0.0f && accept_root(s, W_PLO, last, tol, out);
    }
    int k1 = p->ip + 1;
    float h0 = ds_add(ds_mulf(f->x, G->sphf[k1]), ds_mulf(f->y, -G->cphf[k1])).h;
    float dh = f->kx * G->sphf[k1] - f->ky * G->cphf[k1];
    if (!(dh < 0.0f)) return 0;
    float s = -h0 / dh;
    float hx = f->x.h + s * f->kx, hy = f->y.h + s * f->ky;
    return hx * G->cphf[k1] + hy * G->sphf[k1] > 0.0f && accept_root(s, W_PHI, last, tol, out);
}

/* One Newton step on the selected wall (taken only when it is a small correction).  The
 * refined distance is a pair (s - correction): one float cannot place the packet on the
 * wall (its spacing at 1e12 cm is 1e5 cm). */
/* Residual f and derivative f' of wall candidate k's equation at distance sd. */
static void residual(const Geo* G, const Pkt* p, const Frame* f, int k, ds sd, float* fv_out,
                     float* fd_out) {
    const float s = sd.h;
    ds X = ds_move2(f->x, sd, f->kx), Y = ds_move2(f->y, sd, f->ky), Z = ds_move2(f->z, sd, f->kz);
    float fv = 0.0f, fd = 0.0f;
    if (k == 0 || k == 1) {
        int i = (k == 1) ? p->ir : ((p->ir < 0) ? 0 : p->ir + 1);
        ds r2 = ds_add(ds_add(ds_sqr(X), ds_sqr(Y)), ds_sqr(Z));
        fv = ds_sub(r2, R2(G, i)).h;
        fd = 2.0f * (f->bf + s * f->kk);
    } else if (k == 2 || k == 3) {
        int w = p->itv + (k - 2);
        if (G->muf[w] == 0.0f) {
            fv = Z.h;
            fd = f->kz;
        } else {
            float A, B, C;
            cone_coef(G, f, w, &A, &B, &C);
            ds r2 = ds_add(ds_add(ds_sqr(X), ds_sqr(Y)), ds_sqr(Z));
            fv = ds_sub(ds_sqr(Z), ds_mul(MU2(G, w), r2)).h;
            fd = 2.0f * (B + A * s);
        }
    } else if (k == 4) {
        int k0 = p->ip;
        fv = ds_add(ds_mulf(X, -G->sphf[k0]), ds_mulf(Y, G->cphf[k0])).h;
        fd = -f->kx * G->sphf[k0] + f->ky * G->cphf[k0];
    } else {
        int k1 = p->ip + 1;
        fv = ds_add(ds_mulf(X, G->sphf[k1]), ds_mulf(Y, -G->cphf[k1])).h;
        fd = f->kx * G->sphf[k1] - f->ky * G->cphf[k1];
    }
    *fv_out = fv;
    *fd_out = fd;
}

/* Newton refinement of candidate k's single-precision root s (residual in pairs); a first
 * correction above 1e-6 s (near-tangent crossing) is followed by a second step. */
static ds refine(const Geo* G, const Pkt* p, const Frame* f, int k, float s) {
    float fv, fd;
    ds r, s0 = {s, 0.0f};
    residual(G, p, f, k, s0, &fv, &fd);
    if (fd != 0.0f) {
        float d = fv / fd;
        if (fabsf(d) <= 1.0e-3f * s + f->tol) {
            r = ds_fast2(s, -d);
            if (fabsf(d) > 1.0e-6f * s && r.h > 0.0f) {
                residual(G, p, f, k, r, &fv, &fd);
                if (fd != 0.0f) {
                    float d2 = fv / fd;
                    ds c = {-d2, 0.0f};
                    if (fabsf(d2) <= fabsf(d)) r = ds_add(r, c);
                }
            }
            if (!(r.h > 0.0f)) { r.h = 0.0f; r.l = 0.0f; }
            return r;
        }
    }
    r.h = s > 0.0f ? s : 0.0f;
    r.l = 0.0f;
    return r;
}

static const int k_code[6] = {W_ROUT, W_RIN, W_TLO, W_THI, W_PLO, W_PHI};

ds orc__next_wall_ds(const Geo* G, const Pkt* p, int* wall_out) {
    Frame f;
    frame(G, p, &f);
    float best = 3.0e38f;
    int bk = -1;
    int nk = (p->ir < 0) ? 1 : (G->np > 1 ? 6 : 4);
    for (int k = 0; k < nk; ++k) {
        float s;
        if (candidate(G, p, &f, k, &s) && s < best) {
            best = s;
            bk = k;
        }
    }
    if (bk < 0) {
        ds none = {3.0e38f, 0.0f};
        *wall_out = W_NONE;
        return none;
    }
    *wall_out = k_code[bk];
    return refine(G, p, &f, bk, best);
}

/* cos(theta_j) >= z / r, from the sign of z^2 - mu_j^2 r^2 */
static int mu_ge(const Geo* G, int j, ds z, ds z2, ds r2) {
    float mu = G->muf[j];
    float Q = ds_sub(z2, ds_mul(MU2(G, j), r2)).h;
    if (mu >= 0.0f) return z.h <= 0.0f || Q <= 0.0f;
    return z.h < 0.0f && Q >= 0.0f;
}

/* azimuth at or beyond phi wall k: half-turn first, then the plane function's sign */
static int phi_ge(const Geo* G, int k, ds x, ds y) {
    int hp = (y.h < 0.0f || (y.h == 0.0f && x.h < 0.0f)) ? 1 : 0;
    float sw = G->sphf[k], cw = G->cphf[k];
    int hw = (sw < 0.0f || (sw == 0.0f && cw < 0.0f)) ? 1 : 0;
    if (hp != hw) return hp > hw;
    return ds_add(ds_mulf(x, -sw), ds_mulf(y, cw)).h >= 0.0f;
}

void orc__locate_angles_ds(const Geo* G, Pkt* p) {
    ds z2 = ds_sqr(p->sz);
    ds r2 = ds_add(ds_add(ds_sqr(p->sx), ds_sqr(p->sy)), z2);
    int lo = 0, hi = G->ntv;
    while (hi - lo > 1) {
        int mid = lo + (hi - lo) / 2;
        if (mu_ge(G, mid, p->sz, z2, r2)) lo = mid; else hi = mid;
    }
    p->itv = lo;
    if (G->np > 1) {
        int a = 0, b = G->np;
        while (b - a > 1) {
            int mid = a + (b - a) / 2;
            if (phi_ge(G, mid, p->sx, p->sy)) a = mid; else b = mid;
        }
        p->ip = a;
    } else {
        p->ip = 0;
    }
}

float orc__wall_distance_ds(const Geo* G, const Pkt* p) {
    ds x2 = ds_sqr(p->sx), y2 = ds_sqr(p->sy), z2 = ds_sqr(p->sz);
    ds rho2 = ds_add(x2, y2);
    ds r2 = ds_add(rho2, z2);
    float rf = sqrtf(r2.h);
    float d = ds_sub(r2, R2(G, p->ir)).h / (rf + G->rf[p->ir]);
    float d2 = ds_sub(R2(G, p->ir + 1), r2).h / (rf + G->rf[p->ir + 1]);
    if (d2 < d) d = d2;
    float rhof = sqrtf(rho2.h);
    float zf = p->sz.h;
    for (int side = 0; side < 2; ++side) {
        int w = p->itv + side;
        if (w == 0 || w == G->ntv) continue;
        float a = rhof * G->muf[w];
        float b = zf * G->snf[w];
        float dt;
        if ((a > 0.0f) == (b > 0.0f)) {
            float num = ds_sub(ds_mul(MU2(G, w), r2), z2).h;
            float den = fabsf(a) + fabsf(b);
            dt = den > 0.0f ? fabsf(num) / den : 0.0f;
        } else {
            dt = fabsf(a) + fabsf(b);
        }
        if (dt < d) d = dt;
    }
    if (G->np > 1) {
        int k0 = p->ip, k1 = p->ip + 1;
        float d0 = fabsf(ds_add(ds_mulf(p->sx, -G->sphf[k0]), ds_mulf(p->sy, G->cphf[k0])).h);
        float d1 = fabsf(ds_add(ds_mulf(p->sx, G->sphf[k1]), ds_mulf(p->sy, -G->cphf[k1])).h);
        if (d0 < d) d = d0;
        if (d1 < d) d = d1;
    }
    float m = d * (1.0f - 4.0e-6f);
    return m > 0.0f ? m : 0.0f;
}
