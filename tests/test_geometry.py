"""Wall solves of the walk (double-single, the GPU's default, and FP64) against exact
intersections computed with mpmath at 50 digits, on random rays and on the special cases
of a spherical grid: rays through the pole, in the equatorial plane, near-tangent to a
sphere, on mirrored and full theta grids with phi walls.  The GPU evaluates the same
operations (bit-exact with the oracle), so this pins its geometry too."""
import math

import numpy as np
import pytest

mpmath = pytest.importorskip("mpmath")
from oracle import orc  # noqa: E402

mp = mpmath.mp
mp.dps = 50
AU = 1.495978707e13
W_RIN, W_ROUT, W_TLO, W_THI, W_PLO, W_PHI = 1, 2, 3, 4, 5, 6


def grid(mirror, nphi):
    r = np.logspace(-1, 2, 7) * AU
    t = np.linspace(0.0, np.pi / 2 if mirror else np.pi, 7)
    p = np.linspace(0.0, 2 * np.pi, nphi + 1)
    return r, t, p


def virtual_mu(t, mirror):
    nt = len(t) - 1
    mu = [mpmath.cos(mpf_(x)) for x in t]
    mu[0] = mpmath.mpf(1)
    for j, x in enumerate(t):
        if abs(x - np.pi / 2) < 1e-12:
            mu[j] = mpmath.mpf(0)
    if mirror:
        return mu + [-mu[nt - j] for j in range(1, nt + 1)]
    mu[-1] = mpmath.mpf(-1)
    return mu


def mpf_(x):
    return mpmath.mpf(float(x))


def exact_exit(pos, k, r, mu, ph, ir, itv, ip):
    """All (distance, wall) intersections of the ray with the cell's bounding surfaces
    (correct cone nappe and phi half-plane), ascending."""
    x, y, z = (mpf_(v) for v in pos)
    kx, ky, kz = (mpf_(np.float32(v)) for v in k)
    kk = kx * kx + ky * ky + kz * kz
    r2 = x * x + y * y + z * z
    b = x * kx + y * ky + z * kz
    out = []
    Ro = mpf_(r[ir + 1])
    out.append(((-b + mpmath.sqrt(b * b - kk * (r2 - Ro * Ro))) / kk, W_ROUT))
    Ri = mpf_(r[ir])
    disc = b * b - kk * (r2 - Ri * Ri)
    if disc >= 0:
        s = (-b - mpmath.sqrt(disc)) / kk
        if s > 0:
            out.append((s, W_RIN))
    ntv = len(mu) - 1
    for side, code in ((0, W_TLO), (1, W_THI)):
        w = itv + side
        if w == 0 or w == ntv:
            continue
        m = mu[w]
        if m == 0:
            if kz != 0 and -z / kz > 0:
                out.append((-z / kz, code))
            continue
        A = kz * kz - m * m * kk
        B = z * kz - m * m * b
        Cc = z * z - m * m * r2
        roots = []
        if abs(A) < mpmath.mpf(10) ** -40:
            if B != 0:
                roots.append(-Cc / (2 * B))
        else:
            d = B * B - A * Cc
            if d >= 0:
                roots += [(-B - mpmath.sqrt(d)) / A, (-B + mpmath.sqrt(d)) / A]
        for s in roots:
            if s > 0 and (z + s * kz) * m > 0:
                out.append((s, code))
    if len(ph) > 2:
        for kidx, code in ((ip, W_PLO), (ip + 1, W_PHI)):
            c, sn = mpmath.cos(mpf_(ph[kidx])), mpmath.sin(mpf_(ph[kidx]))
            g0 = -x * sn + y * c
            dg = -kx * sn + ky * c
            if dg != 0:
                s = -g0 / dg
                if s > 0 and (x + s * kx) * c + (y + s * ky) * sn > 0:
                    out.append((s, code))
    return sorted(out, key=lambda t_: t_[0])


def random_rays(mirror, nphi, n, seed):
    r, t, p = grid(mirror, nphi)
    nt = len(t) - 1
    rng = np.random.default_rng(seed)
    rays = []
    for _ in range(n):
        ir = int(rng.integers(0, len(r) - 1))
        it = int(rng.integers(0, nt))
        ip = int(rng.integers(0, len(p) - 1))
        f = rng.uniform(0.02, 0.98, 3)
        rr = r[ir] * (r[ir + 1] / r[ir]) ** f[0]
        th = t[it] + f[1] * (t[it + 1] - t[it])
        ph = p[ip] + f[2] * (p[ip + 1] - p[ip])
        itv = it
        if mirror and rng.random() < 0.5:
            th = np.pi - th
            itv = 2 * nt - 1 - it
        pos = [rr * math.sin(th) * math.cos(ph), rr * math.sin(th) * math.sin(ph), rr * math.cos(th)]
        d = rng.normal(size=3)
        d = (d / np.linalg.norm(d)).astype(np.float32)
        rays.append((pos, d, ir, itv, ip))
    return (r, t, p), rays


def check(geo, rays, fp64, rel=1e-9, walls=None):
    r, t, p = geo
    mirror = abs(t[-1] - np.pi / 2) < 1e-12
    mu = virtual_mu(t, mirror)
    worst = 0.0
    for pos, d, ir, itv, ip in rays:
        ex = exact_exit(pos, d, r, mu, p, ir, itv, ip)
        got, wall = orc.wall_solve(r, t, p, pos, d, ir, itv, ip, 0, fp64=fp64)
        scale = float(r[ir + 1])
        best, bw = ex[0]
        err = abs(got - float(best)) / scale
        worst = max(worst, err)
        tie = len(ex) > 1 and float(ex[1][0] - best) / scale < rel
        assert err < rel, (pos, d, ir, itv, ip, got, float(best), wall, bw)
        assert wall == bw or tie, (pos, d, ir, itv, ip, wall, bw, ex[:3])
        if walls is not None:
            walls.append(bw)
    return worst


@pytest.mark.parametrize("mirror,nphi", [(False, 1), (True, 1), (False, 8), (True, 8)])
@pytest.mark.parametrize("fp64", [False, True])
def test_random_rays(mirror, nphi, fp64):
    geo, rays = random_rays(mirror, nphi, 300, seed=11 + nphi + 2 * mirror)
    walls = []
    worst = check(geo, rays, fp64, walls=walls)
    assert worst < 1e-9
    # every kind of wall is exercised
    kinds = {W_RIN, W_ROUT, W_TLO, W_THI} | ({W_PLO, W_PHI} if nphi > 1 else set())
    assert kinds <= set(walls)


@pytest.mark.parametrize("fp64", [False, True])
def test_pole_equator_and_tangent_rays(fp64):
    r, t, p = grid(False, 8)
    nt = len(t) - 1
    rays = []
    # along the pole axis, from a point just off it, up and down
    for kz in (1.0, -1.0):
        pos = [1e-6 * r[2], 2e-6 * r[2], 0.5 * (r[2] + r[3]) * kz]
        ip = int(np.searchsorted(p, math.atan2(pos[1], pos[0]) % (2 * np.pi)) - 1)
        itv = 0 if kz > 0 else nt - 1
        rays.append((pos, np.array([0.0, 0.0, kz], np.float32), 2, itv, ip))
    # in the equatorial plane, just above it, moving parallel to it (never meets z = 0)
    for ang in (0.3, 1.9, 4.0):
        rr = 0.5 * (r[3] + r[4])
        pos = [rr * math.cos(ang), rr * math.sin(ang), 1e-7 * rr]
        d = np.array([-math.sin(ang + 0.2), math.cos(ang + 0.2), 0.0], np.float32)
        ip = int(np.searchsorted(p, ang % (2 * np.pi)) - 1)
        rays.append((pos, d, 3, nt // 2 - 1, ip))
    walls = []
    check((r, t, p), rays, fp64, walls=walls)
    assert walls[0] == W_ROUT and walls[1] == W_ROUT      # pole rays leave through spheres
    # near-tangent to the inner sphere of shell 3 (no phi walls; the ray stays between the
    # 30 and 60 degree cones until it passes its closest approach R (1 +- 1e-6))
    r, t, p = grid(False, 1)
    tangent = []
    for eps in (1e-6, -1e-6):
        R = r[3] * (1 + eps)
        pos = [1.2 * r[3], 0.6 * R, 0.8 * R]
        tangent.append((pos, np.array([-1.0, 0.0, 0.0], np.float32), 3, 1, 0))
    tw = []
    check((r, t, p), tangent, fp64, walls=tw)
    assert tw == [W_THI, W_RIN]

