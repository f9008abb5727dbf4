// Host-side preparation of a spherical grid for the device geometry in mc_geom.cuh:
// validation of the edges and the double/float wall tables and cell-volume factors.
//
// Grids follow pdspy's Grid.set_spherical_grid (pdspy/modeling/Grid.py:71-80): r edges
// (here in cm), theta edges over [0, pi] or [0, pi/2] (mirrored about the equator, the
// convention pdspy's YSOModel uses with RADMC-3D, YSOModel.py:47-63) and phi edges over
// [0, 2 pi].
#pragma once
#include <cmath>
#include <cstring>
#include <vector>

#include "mc_common.h"

namespace pdgpu {

// Validates one grid and appends its geometry to the pools; fills the geometry fields of
// M (counts, mirror flag, wall and volume offsets).  Returns false on invalid edges.
inline bool append_geometry(int nr, int nt, int np, const double* r_edges,
                            const double* theta_edges, const double* phi_edges, McModel& M,
                            std::vector<double>& dp, std::vector<float>& fp) {
    if (nr < 1 || nt < 1 || np < 1 || !r_edges || !theta_edges || !phi_edges) return false;
    if (!(r_edges[0] > 0.0)) return false;
    for (int i = 1; i <= nr; ++i)
        if (!(r_edges[i] > r_edges[i - 1])) return false;
    for (int i = 1; i <= nt; ++i)
        if (!(theta_edges[i] > theta_edges[i - 1])) return false;
    for (int i = 1; i <= np; ++i)
        if (!(phi_edges[i] > phi_edges[i - 1])) return false;
    double thmax = theta_edges[nt];
    if (std::fabs(theta_edges[0]) > 1e-12) return false;
    if (std::fabs(thmax - MC_PI) < 1e-9) M.mirror = 0;
    else if (std::fabs(thmax - 0.5 * MC_PI) < 1e-9) M.mirror = 1;
    else return false;
    if (np > 1 && (std::fabs(phi_edges[0]) > 1e-12 || std::fabs(phi_edges[np] - 2.0 * MC_PI) > 1e-9))
        return false;
    M.nr = nr; M.nt = nt; M.np = np;
    M.ntv = M.mirror ? 2 * nt : nt;
    M.ncell = nr * nt * np;
    M.off_r = (int)dp.size();
    for (int i = 0; i <= nr; ++i) dp.push_back(r_edges[i]);
    M.off_mu = (int)dp.size();
    dp.resize(dp.size() + M.ntv + 1);
    M.off_sn = (int)dp.size();
    dp.resize(dp.size() + M.ntv + 1);
    for (int j = 0; j <= nt; ++j) {
        double th = theta_edges[j];
        double mv = std::cos(th), sv = std::sin(th);
        if (std::fabs(th - 0.5 * MC_PI) < 1e-12) { mv = 0.0; sv = 1.0; }
        if (j == 0) { mv = 1.0; sv = 0.0; }
        if (!M.mirror && j == nt) { mv = -1.0; sv = 0.0; }
        dp[M.off_mu + j] = mv;
        dp[M.off_sn + j] = sv;
    }
    if (M.mirror)
        for (int j = 0; j < nt; ++j) {
            dp[M.off_mu + 2 * nt - j] = -dp[M.off_mu + j];
            dp[M.off_sn + 2 * nt - j] = dp[M.off_sn + j];
        }
    M.off_cph = (int)dp.size();
    for (int k = 0; k <= np; ++k) dp.push_back(std::cos(phi_edges[k]));
    M.off_sph = (int)dp.size();
    for (int k = 0; k <= np; ++k) dp.push_back(std::sin(phi_edges[k]));
    M.off_vr = (int)dp.size();
    for (int i = 0; i < nr; ++i) {
        double r0 = r_edges[i], r1 = r_edges[i + 1];
        dp.push_back((r1 * r1 * r1 - r0 * r0 * r0) / 3.0);
    }
    M.off_vt = (int)dp.size();
    for (int j = 0; j < nt; ++j) {
        double v = dp[M.off_mu + j] - dp[M.off_mu + j + 1];
        dp.push_back(M.mirror ? 2.0 * v : v);
    }
    M.off_vp = (int)dp.size();
    for (int k = 0; k < np; ++k) dp.push_back(phi_edges[k + 1] - phi_edges[k]);
    for (int k = 0; k <= np; ++k) dp.push_back(phi_edges[k]);  // edges follow the widths
    // single-precision copies of the walls for the safety distance
    M.off_rf = (int)fp.size();
    for (int i = 0; i <= nr; ++i) fp.push_back((float)dp[M.off_r + i]);
    M.off_muf = (int)fp.size();
    for (int j = 0; j <= M.ntv; ++j) fp.push_back((float)dp[M.off_mu + j]);
    M.off_snf = (int)fp.size();
    for (int j = 0; j <= M.ntv; ++j) fp.push_back((float)dp[M.off_sn + j]);
    M.off_cphf = (int)fp.size();
    for (int k = 0; k <= np; ++k) fp.push_back((float)dp[M.off_cph + k]);
    M.off_sphf = (int)fp.size();
    for (int k = 0; k <= np; ++k) fp.push_back((float)dp[M.off_sph + k]);
    // double-single walls: hi = nearest float, lo = nearest float of the remainder
    auto lo_part = [](double v) { return (float)(v - (double)(float)v); };
    M.off_rl = (int)fp.size();
    for (int i = 0; i <= nr; ++i) fp.push_back(lo_part(dp[M.off_r + i]));
    M.off_r2h = (int)fp.size();
    for (int i = 0; i <= nr; ++i) {
        double R = dp[M.off_r + i];
        fp.push_back((float)(R * R));
    }
    M.off_r2l = (int)fp.size();
    for (int i = 0; i <= nr; ++i) {
        double R = dp[M.off_r + i];
        fp.push_back(lo_part(R * R));
    }
    M.off_mu2h = (int)fp.size();
    for (int j = 0; j <= M.ntv; ++j) {
        double mu = dp[M.off_mu + j];
        fp.push_back((float)(mu * mu));
    }
    M.off_mu2l = (int)fp.size();
    for (int j = 0; j <= M.ntv; ++j) {
        double mu = dp[M.off_mu + j];
        fp.push_back(lo_part(mu * mu));
    }
    while (fp.size() % 4) fp.push_back(0.0f);
    return true;
}

}  // namespace pdgpu
