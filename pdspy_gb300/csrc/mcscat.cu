// Monochromatic Monte Carlo of the scattering source (GB300, sm_103a).
//
// Replaces the scattering Monte Carlo RADMC-3D runs inside "radmc3d image" and
// "radmc3d spectrum" when the dust scatters (pdspy/modeling/Model.py:515-577, :608-650;
// photon counts nphot_scat / nphot_spec and mc_scat_maxtauabs from
// pdspy/radmc3d/write.py:33-38, :141-142) and as "radmc3d mcscat" behind
// Model.run_scattering (Model.py:258-322).  The result is the mean intensity J of every
// cell at every camera wavelength; the isotropic scattering emissivity of the cell is
// sum_s rho_s ksca_s J (pdspy never passes an asymmetry parameter to RADMC-3D,
// Model.py:774-776, so scattering is isotropic on this path).
//
// Method (restated from the Monte Carlo literature: Lucy 1999 path-length estimator of
// J, absorption handled by continuous weighting):
//   - Packets of wavelength l carry eps_l = (L_star + L_dust) / N erg/s/Hz.  A packet
//     starts at the stars (at the origin, isotropic) with probability L_star / L_total,
//     else in a dust cell drawn from the cumulative thermal luminosity of the cells,
//     uniformly in the cell's volume, isotropic.
//   - Free paths are drawn in scattering optical depth.  Along a segment of length L in a
//     cell with absorption coefficient a the packet adds w (1 - e^-aL) / a to the cell's
//     path-length sum (w its surviving fraction) and w becomes w e^-aL.
//   - At the end of a free path it scatters isotropically.  It is dropped once the
//     absorption optical depth along its whole path exceeds maxtauabs (RADMC-3D's
//     mc_scat_maxtauabs), or after max_scatter scatterings.
//   - J = eps_l sum(w L_eff) / (4 pi V).
//
// Determinism.  The path-length sums are int64 fixed point with 2^32 units per radial
// width of the cell's shell, so the result does not depend on the order of the atomics;
// the cumulative luminosity of the cells is an integer prefix sum.  Random numbers are
// Philox4x32-10 blocks keyed by (seed; draw index, packet, wavelength, pass tag), and all
// arithmetic is written operation by operation (--fmad=false), so the CPU oracle
// reproduces J bit for bit.
//
// Execution.  One launch for all wavelengths: packets of every wavelength share one work
// queue that warps refill with one atomic per refill; geometry is the double-single walk
// of the thermal Monte Carlo (mc_geom_ds.cuh).  Walks are short (the absorption cut), so
// one packet per thread suffices.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/pdgpu.h"
#include "mc_common.h"
#include "mc_device.cuh"
#include "mc_geom_ds.cuh"
#include "mc_host.h"

namespace {
using namespace pdgpu;

constexpr uint32_t SC_TAG = 0x5Cu;   // pass tag of scattering packets
constexpr int SC_SRC_THREADS = 1024;
constexpr double SC_FOUR_PI = 4.0 * MC_PI;

enum { SS_PACKETS = 0, SS_ESCAPED, SS_DROPPED, SS_CAPPED, SS_SCATTER, SS_CROSS, SS_KILLED,
       SS_STATUS, SS_N = 16 };

struct ScLam {          // per wavelength, written by the source kernel
    double eps;         // packet energy, erg/s/Hz
    double lstar;       // stellar luminosity, erg/s/Hz
    double ldust;       // thermal dust luminosity represented by the cell table
    float pstar;        // probability that a packet starts at the stars
    int32_t pad;
};

struct ScParams {
    McModel M;
    const float* fp;       // float geometry pool
    const double* dp;      // double geometry pool
    const float* phf;      // [np+1] phi edges in turns
    const float* invdr;    // [nr] fixed-point units per cm of path: 2^32 / (R[i+1] - R[i])
    const float* kap;      // [nlam][2][ns]: kabs of every species, then ksca
    const float* rho;      // [ns][ncell]
    const float* cdf;      // [nlam][ncell]
    const ScLam* lam;
    unsigned long long* acc;   // [nlam][ncell]
    int64_t* stats;
    unsigned long long* queue;
    int64_t nphot, total;
    int32_t nlam, ns;
    uint32_t key0, key1;
    float maxtauabs;
    int32_t max_scatter;
};

// Thermal luminosity (erg/s/Hz) of cell c: 4 pi V_c emis_c.
__device__ __forceinline__ double sc_cell_lum(const McModel& M, const double* dp, const double* e,
                                              int c) {
    const int ir = c / (M.nt * M.np);
    const int it = (c / M.np) % M.nt;
    const int ip = c % M.np;
    const double V = (dp[M.off_vr + ir] * dp[M.off_vt + it]) * dp[M.off_vp + ip];
    return (e[c] * V) * SC_FOUR_PI;
}

__device__ __forceinline__ unsigned long long sc_units(double L, double Lmax, double scale) {
    if (!(L > 0.0) || !(Lmax > 0.0)) return 0ull;
    return (unsigned long long)(long long)((L / Lmax) * scale + 0.5);
}

// One block per wavelength: the cumulative distribution of the cells' thermal
// luminosity (integer units, scale 2^shift per the brightest cell), the stellar share and
// the packet energy.
__global__ void __launch_bounds__(SC_SRC_THREADS) sc_source_kernel(McModel M, const double* dp,
                                                                   const double* emis,
                                                                   const double* lstar,
                                                                   int ncell, double scale,
                                                                   int64_t nphot, float* cdf,
                                                                   ScLam* lam) {
    __shared__ double s_d[32];
    __shared__ unsigned long long s_u[32];
    __shared__ double s_max;
    __shared__ unsigned long long s_tot;
    const int l = blockIdx.x;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const int nw = blockDim.x >> 5;
    const double* e = emis ? emis + (size_t)l * ncell : nullptr;
    float* cl = cdf + (size_t)l * ncell;
    // brightest cell
    double mx = 0.0;
    if (e)
        for (int c = tid; c < ncell; c += blockDim.x) mx = fmax(mx, sc_cell_lum(M, dp, e, c));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = fmax(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    if (lane == 0) s_d[wid] = mx;
    __syncthreads();
    if (tid == 0) {
        double m = 0.0;
        for (int w = 0; w < nw; ++w) m = fmax(m, s_d[w]);
        s_max = m;
    }
    __syncthreads();
    const double Lmax = s_max;
    // total units
    unsigned long long t = 0;
    if (e)
        for (int c = tid; c < ncell; c += blockDim.x) t += sc_units(sc_cell_lum(M, dp, e, c), Lmax, scale);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) s_u[wid] = t;
    __syncthreads();
    if (tid == 0) {
        unsigned long long a = 0;
        for (int w = 0; w < nw; ++w) a += s_u[w];
        s_tot = a;
    }
    __syncthreads();
    const unsigned long long U = s_tot;
    // inclusive prefix, chunk by chunk
    unsigned long long carry = 0;
    for (int base = 0; base < ncell; base += blockDim.x) {
        const int c = base + tid;
        unsigned long long v = (e && c < ncell) ? sc_units(sc_cell_lum(M, dp, e, c), Lmax, scale) : 0ull;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(0xffffffffu, v, o);
            if (lane >= o) v += y;
        }
        __syncthreads();
        if (lane == 31) s_u[wid] = v;
        __syncthreads();
        if (wid == 0) {
            unsigned long long w = (lane < nw) ? s_u[lane] : 0ull;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long y = __shfl_up_sync(0xffffffffu, w, o);
                if (lane >= o) w += y;
            }
            s_u[lane] = w;
        }
        __syncthreads();
        const unsigned long long before = (wid > 0) ? s_u[wid - 1] : 0ull;
        if (c < ncell) cl[c] = U > 0 ? (float)((double)(carry + before + v) / (double)U) : 1.0f;
        carry += s_u[nw - 1];
    }
    if (tid == 0) {
        const double ls = lstar[l];
        const double ld = (double)U * (Lmax / scale);
        const double lt = ls + ld;
        ScLam r;
        r.lstar = ls;
        r.ldust = ld;
        r.pstar = lt > 0.0 ? (float)(ls / lt) : 1.0f;
        r.eps = lt / (double)nphot;
        r.pad = 0;
        lam[l] = r;
    }
}

struct ScCnt {
    long long escaped, dropped, capped, scatter, cross, killed;
};

// Start packet p (its rng set) of wavelength l.
__device__ __forceinline__ void sc_emit(PktS& p, const ScParams& P, const ScLam& L) {
    const McModel& M = P.M;
    const uint4 e0 = mc_block(p.rng, 0u, MC_RS_EMIT, P.key0, P.key1);
    const uint4 e1 = mc_block(p.rng, 1u, MC_RS_EMIT, P.key0, P.key1);
    p.tau = -mc_logf(mc_u01(e0.z));
    {
        float mu = 2.0f * mc_u01(e1.x) - 1.0f;
        float sn, cs;
        mc_sincospif2(mc_u01(e1.y), sn, cs);
        float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
        p.kx = st * cs; p.ky = st * sn; p.kz = mu;
    }
    p.last_wall = W_NONE;
    p.nevents = 0;
    p.ncross = 0;
    if (mc_u01(e0.x) < L.pstar) {
        p.x = ds{0.0f, 0.0f}; p.y = ds{0.0f, 0.0f}; p.z = ds{0.0f, 0.0f};
        p.ir = -1; p.itv = 0; p.ip = 0;
        return;
    }
    const uint4 e2 = mc_block(p.rng, 2u, MC_RS_EMIT, P.key0, P.key1);
    const int c = mc_cdf_search(P.cdf + (size_t)p.lam * M.ncell, M.ncell, mc_u01(e0.y));
    const int ir = c / (M.nt * M.np);
    const int it = (c / M.np) % M.nt;
    const int ip = c % M.np;
    const int itv = (M.mirror && mc_u01(e0.w) >= 0.5f) ? 2 * M.nt - 1 - it : it;
    const float* RF = P.fp + M.off_rf;
    const float* MUF = P.fp + M.off_muf;
    float t0 = RF[ir] / RF[ir + 1];
    float a = t0 * t0 * t0;
    float r = mc_cbrt01(a + mc_u01(e1.z) * (1.0f - a)) * RF[ir + 1];
    float m0 = MUF[itv + 1], m1 = MUF[itv];
    float mu = m0 + mc_u01(e1.w) * (m1 - m0);
    float uphi = mc_u01(e2.x);
    if (M.np > 1) uphi = P.phf[ip] + uphi * (P.phf[ip + 1] - P.phf[ip]);
    float sp, cp;
    mc_sincospif2(uphi, sp, cp);
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    float rs = r * st;
    p.x = ds{rs * cp, 0.0f};
    p.y = ds{rs * sp, 0.0f};
    p.z = ds{r * mu, 0.0f};
    p.ir = ir; p.itv = itv; p.ip = ip;
}

// One segment: to the next wall or to the next scattering.  Returns false when the packet
// has left the grid or was dropped.  w: surviving fraction, tabs: absorption depth so far.
__device__ __forceinline__ bool sc_step(PktS& p, float& w, float& tabs, const ScParams& P,
                                        ScCnt& cnt) {
    const McModel& M = P.M;
    const WallsS W(M, P.fp);
    const int ns = P.ns;
    const float* K = P.kap + (size_t)p.lam * 2 * ns;
    int c = -1;
    float aa = 0.0f, as = 0.0f;
    if (p.ir >= 0) {
        c = cell_of_s(M, p);
        for (int s = 0; s < ns; ++s) {
            const float r = __ldg(P.rho + (int64_t)s * M.ncell + c);
            aa = aa + r * K[s];
            as = as + r * K[ns + s];
        }
    }
    int wall = W_NONE;
    const ds sw = next_wall_ds(M, W, p, wall);
    const float tw = as * sw.h;
    const bool scat = tw > p.tau;
    ds sl = sw;
    if (scat) {
        const float se = p.tau / as;
        if (!(se > sw.h)) sl = ds{se, 0.0f};
    }
    const float len = sl.h;
    if (c >= 0 && len > 0.0f) {
        const float x = aa * len;
        const float att = mc_expm(x);
        const float d = w * (len * mc_expm_frac(x, att));
        float uf = d * P.invdr[p.ir] + 0.5f;
        if (uf >= 1.0f) {
            if (uf > 9.0e18f) uf = 9.0e18f;
            atomicAdd(P.acc + (int64_t)p.lam * M.ncell + c, (unsigned long long)(long long)uf);
        }
        w = w * att;
        tabs = tabs + x;
    }
    p.x = ds_move2(p.x, sl, p.kx);
    p.y = ds_move2(p.y, sl, p.ky);
    p.z = ds_move2(p.z, sl, p.kz);
    if (tabs > P.maxtauabs) {
        cnt.dropped += 1;
        return false;
    }
    if (scat) {
        const uint32_t n = (uint32_t)p.nevents;
        p.nevents += 1;
        cnt.scatter += 1;
        const uint4 b = mc_block(p.rng, n, MC_RS_EVENT, P.key0, P.key1);
        p.tau = -mc_logf(mc_u01(b.x));
        float mu = 2.0f * mc_u01(b.y) - 1.0f;
        float sn, cs;
        mc_sincospif2(mc_u01(b.z), sn, cs);
        float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
        p.kx = st * cs; p.ky = st * sn; p.kz = mu;
        p.last_wall = W_NONE;
        if (p.nevents >= P.max_scatter) {
            cnt.capped += 1;
            return false;
        }
        return true;
    }
    p.tau = p.tau - tw;
    p.ncross += 1;
    cnt.cross += 1;
    switch (wall) {
        case W_ROUT:
            if (p.ir < 0) { p.ir = 0; locate_angles_ds(M, W, p); }
            else p.ir += 1;
            p.last_wall = W_RIN;
            if (p.ir >= M.nr) {
                cnt.escaped += 1;
                return false;
            }
            break;
        case W_RIN: p.ir -= 1; p.last_wall = W_ROUT; break;
        case W_TLO: p.itv -= 1; p.last_wall = W_THI; break;
        case W_THI: p.itv += 1; p.last_wall = W_TLO; break;
        case W_PLO: p.ip = (p.ip == 0) ? M.np - 1 : p.ip - 1; p.last_wall = W_PHI; break;
        case W_PHI: p.ip = (p.ip == M.np - 1) ? 0 : p.ip + 1; p.last_wall = W_PLO; break;
        default: cnt.killed += 1; return false;
    }
    if (p.ncross > 100000000) {
        cnt.killed += 1;
        return false;
    }
    return true;
}

__device__ __forceinline__ long long sc_warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__global__ void __launch_bounds__(256, 3) sc_transport_kernel(ScParams P) {
    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    ScCnt cnt = {0, 0, 0, 0, 0, 0};
    PktS p;
    float w = 0.0f, tabs = 0.0f;
    bool active = false;
    bool queue_open = true;
    for (;;) {
        unsigned need = queue_open ? __ballot_sync(0xffffffffu, !active) : 0u;
        if (need) {
            const int n = __popc(need);
            unsigned long long basev = 0;
            if (lane == 0) basev = atomicAdd(P.queue, (unsigned long long)n);
            basev = __shfl_sync(0xffffffffu, basev, 0);
            if ((long long)basev + n >= P.total) queue_open = false;
            if (!active) {
                const long long g = (long long)basev + __popc(need & lt_mask);
                if (g < P.total) {
                    const int l = (int)(g / P.nphot);
                    p.lam = l;
                    p.rng.pid = (uint32_t)(g - (long long)l * P.nphot);
                    p.rng.model = (uint32_t)l;
                    p.rng.tag = SC_TAG;
                    sc_emit(p, P, P.lam[l]);
                    w = 1.0f;
                    tabs = 0.0f;
                    active = true;
                }
            }
        }
        if (!__any_sync(0xffffffffu, active)) break;
        if (active) active = sc_step(p, w, tabs, P, cnt);
    }
    const long long v[6] = {cnt.escaped, cnt.dropped, cnt.capped, cnt.scatter, cnt.cross, cnt.killed};
    const int slot[6] = {SS_ESCAPED, SS_DROPPED, SS_CAPPED, SS_SCATTER, SS_CROSS, SS_KILLED};
#pragma unroll
    for (int i = 0; i < 6; ++i) {
        const long long s = sc_warp_sum(v[i]);
        if (lane == 0 && s) atomicAdd((unsigned long long*)(P.stats + slot[i]), (unsigned long long)s);
    }
}

// J = eps_l (units / invdr) / (4 pi V).
__global__ void sc_finish_kernel(McModel M, const double* dp, const float* invdr, const ScLam* lam,
                                 const unsigned long long* acc, int nlam, double* J) {
    const int64_t n = (int64_t)nlam * M.ncell;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n;
         i += (int64_t)gridDim.x * blockDim.x) {
        const int l = (int)(i / M.ncell);
        const int c = (int)(i - (int64_t)l * M.ncell);
        const unsigned long long u = acc[i];
        double v = 0.0;
        if (u) {
            const int ir = c / (M.nt * M.np);
            const int it = (c / M.np) % M.nt;
            const int ip = c % M.np;
            const double V = (dp[M.off_vr + ir] * dp[M.off_vt + it]) * dp[M.off_vp + ip];
            v = (((double)(long long)u / (double)invdr[ir]) * lam[l].eps) / (SC_FOUR_PI * V);
        }
        J[i] = v;
    }
}

double planck_nu_host(double nu, double T) {
    double x = MC_H_PLANCK * nu / (MC_K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double pre = 2.0 * MC_H_PLANCK * nu * nu * nu / (MC_C_LIGHT * MC_C_LIGHT);
    return pre / expm1(x);
}

}  // namespace

struct pdgpu_scat_plan {
    McModel M;
    std::vector<double> dp;
    std::vector<float> fp, phf, invdr, kap;
    std::vector<double> lstar;
    int nlam, ns;
    pdgpu_scat_options o;
    double scale;
    size_t ws_dp, ws_fp, ws_phf, ws_invdr, ws_kap, ws_lstar, ws_lam, ws_cdf, ws_acc, ws_stats,
        ws_queue, ws_total;
    int nsm, grid, block;
    const void* uploaded_ws;
};

extern "C" {

pdgpu_status pdgpu_scat_plan_create(const pdgpu_model_desc* md, int32_t nlam, const double* lam_um,
                                    int32_t nspec, const double* kabs, const double* ksca,
                                    const pdgpu_scat_options* opts, pdgpu_scat_plan** out) {
    if (!out || !md || !lam_um || !kabs || !ksca || !opts) return PDGPU_INVALID_ARG;
    *out = nullptr;
    if (nlam < 1 || nspec < 1 || nspec > MC_MAX_SPEC || opts->nphot < 1) return PDGPU_INVALID_ARG;
    if (md->nstar < 0 || (md->nstar > 0 && (!md->star_radius_cm || !md->star_temperature)))
        return PDGPU_INVALID_ARG;
    if ((int64_t)nlam * opts->nphot > ((int64_t)1 << 40)) return PDGPU_INVALID_ARG;
    pdgpu_scat_plan* P = new (std::nothrow) pdgpu_scat_plan();
    if (!P) return PDGPU_INVALID_ARG;
    memset(&P->M, 0, sizeof(P->M));
    if (!append_geometry(md->nr, md->ntheta, md->nphi, md->r_edges_cm, md->theta_edges,
                         md->phi_edges, P->M, P->dp, P->fp)) {
        delete P;
        return PDGPU_INVALID_ARG;
    }
    const int nr = md->nr, np = md->nphi;
    for (int l = 0; l < nlam; ++l) {
        if (!(lam_um[l] > 0.0)) { delete P; return PDGPU_INVALID_ARG; }
        for (int s = 0; s < nspec; ++s)
            if (!(kabs[(size_t)s * nlam + l] >= 0.0) || !(ksca[(size_t)s * nlam + l] >= 0.0)) {
                delete P;
                return PDGPU_INVALID_ARG;
            }
    }
    P->nlam = nlam;
    P->ns = nspec;
    P->o = *opts;
    if (!(P->o.maxtauabs > 0.0f)) P->o.maxtauabs = 30.0f;
    if (P->o.max_scatter <= 0) P->o.max_scatter = 1000000;
    for (int k = 0; k <= np; ++k) P->phf.push_back((float)(md->phi_edges[k] / (2.0 * MC_PI)));
    for (int i = 0; i < nr; ++i)
        P->invdr.push_back((float)(4294967296.0 / (md->r_edges_cm[i + 1] - md->r_edges_cm[i])));
    P->kap.resize((size_t)nlam * 2 * nspec);
    for (int l = 0; l < nlam; ++l)
        for (int s = 0; s < nspec; ++s) {
            P->kap[((size_t)l * 2 + 0) * nspec + s] = (float)kabs[(size_t)s * nlam + l];
            P->kap[((size_t)l * 2 + 1) * nspec + s] = (float)ksca[(size_t)s * nlam + l];
        }
    P->lstar.assign(nlam, 0.0);
    for (int l = 0; l < nlam; ++l) {
        const double nu = MC_C_LIGHT / (lam_um[l] * 1.0e-4);
        double L = 0.0;
        for (int k = 0; k < md->nstar; ++k) {
            const double R = md->star_radius_cm[k];
            L = L + 4.0 * MC_PI * MC_PI * R * R * planck_nu_host(nu, md->star_temperature[k]);
        }
        P->lstar[l] = L;
    }
    // 2^shift units for the brightest cell keeps the sum over all cells below 2^62
    int lg = 0;
    while (((int64_t)1 << lg) < (int64_t)P->M.ncell) ++lg;
    P->scale = std::ldexp(1.0, std::min(40, 62 - lg));
    const int64_t ncl = (int64_t)nlam * P->M.ncell;
    size_t o = 0;
    auto place = [&](size_t bytes) {
        o = (o + 255) / 256 * 256;
        size_t at = o;
        o += bytes;
        return at;
    };
    P->ws_dp = place(P->dp.size() * sizeof(double));
    P->ws_fp = place(P->fp.size() * sizeof(float));
    P->ws_phf = place(P->phf.size() * sizeof(float));
    P->ws_invdr = place(P->invdr.size() * sizeof(float));
    P->ws_kap = place(P->kap.size() * sizeof(float));
    P->ws_lstar = place(P->lstar.size() * sizeof(double));
    P->ws_lam = place((size_t)nlam * sizeof(ScLam));
    P->ws_cdf = place((size_t)ncl * sizeof(float));
    P->ws_acc = place((size_t)ncl * sizeof(unsigned long long));
    P->ws_stats = place(SS_N * sizeof(int64_t));
    P->ws_queue = place(sizeof(unsigned long long));
    P->ws_total = (o + 255) / 256 * 256;
    P->uploaded_ws = nullptr;
    int dev = 0, nsm = 1;
    if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
    P->nsm = nsm > 0 ? nsm : 1;
    P->block = P->o.block_threads > 0 ? P->o.block_threads : 256;
    if (P->block % 32 || P->block > 256) P->block = 256;
    int occ = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, sc_transport_kernel, P->block, 0) != cudaSuccess || occ < 1)
        occ = 1;
    if (P->o.blocks_per_sm > 0 && P->o.blocks_per_sm < occ) occ = P->o.blocks_per_sm;
    int64_t g = (int64_t)occ * P->nsm;
    const int64_t need = ((int64_t)nlam * P->o.nphot + P->block - 1) / P->block;
    if (need < g) g = need;
    P->grid = (int)g;
    *out = P;
    return PDGPU_OK;
}

void pdgpu_scat_plan_destroy(pdgpu_scat_plan* plan) { delete plan; }

pdgpu_status pdgpu_scat_plan_info(const pdgpu_scat_plan* P, size_t* workspace_bytes, int64_t* ncell) {
    if (!P) return PDGPU_INVALID_ARG;
    if (workspace_bytes) *workspace_bytes = P->ws_total;
    if (ncell) *ncell = P->M.ncell;
    return PDGPU_OK;
}

pdgpu_status pdgpu_scat_plan_upload(pdgpu_scat_plan* P, void* ws, size_t bytes, void* stream) {
    if (!P) return PDGPU_INVALID_ARG;
    if (!ws || bytes < P->ws_total) return PDGPU_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char* w = (char*)ws;
    auto up = [&](size_t off, const void* src, size_t n) {
        return cudaMemcpyAsync(w + off, src, n, cudaMemcpyHostToDevice, st) == cudaSuccess;
    };
    if (!up(P->ws_dp, P->dp.data(), P->dp.size() * sizeof(double)) ||
        !up(P->ws_fp, P->fp.data(), P->fp.size() * sizeof(float)) ||
        !up(P->ws_phf, P->phf.data(), P->phf.size() * sizeof(float)) ||
        !up(P->ws_invdr, P->invdr.data(), P->invdr.size() * sizeof(float)) ||
        !up(P->ws_kap, P->kap.data(), P->kap.size() * sizeof(float)) ||
        !up(P->ws_lstar, P->lstar.data(), P->lstar.size() * sizeof(double)) ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    P->uploaded_ws = ws;
    return PDGPU_OK;
}

pdgpu_status pdgpu_scat_run(pdgpu_scat_plan* P, const float* rho, const double* emis, double* J,
                            void* ws, size_t bytes, void* stream) {
    if (!P || !rho || !J) return PDGPU_INVALID_ARG;
    if (!ws || bytes < P->ws_total || ws != P->uploaded_ws) return PDGPU_WORKSPACE;
    cudaStream_t st = (cudaStream_t)stream;
    char* w = (char*)ws;
    const int64_t ncl = (int64_t)P->nlam * P->M.ncell;
    if (cudaMemsetAsync(w + P->ws_acc, 0, (size_t)ncl * sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_stats, 0, SS_N * sizeof(int64_t), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_queue, 0, sizeof(unsigned long long), st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    const double* dp = (const double*)(w + P->ws_dp);
    sc_source_kernel<<<P->nlam, SC_SRC_THREADS, 0, st>>>(P->M, dp, emis, (const double*)(w + P->ws_lstar),
                                                         P->M.ncell, P->scale, P->o.nphot,
                                                         (float*)(w + P->ws_cdf), (ScLam*)(w + P->ws_lam));
    ScParams S;
    memset(&S, 0, sizeof(S));
    S.M = P->M;
    S.fp = (const float*)(w + P->ws_fp);
    S.dp = dp;
    S.phf = (const float*)(w + P->ws_phf);
    S.invdr = (const float*)(w + P->ws_invdr);
    S.kap = (const float*)(w + P->ws_kap);
    S.rho = rho;
    S.cdf = (const float*)(w + P->ws_cdf);
    S.lam = (const ScLam*)(w + P->ws_lam);
    S.acc = (unsigned long long*)(w + P->ws_acc);
    S.stats = (int64_t*)(w + P->ws_stats);
    S.queue = (unsigned long long*)(w + P->ws_queue);
    S.nphot = P->o.nphot;
    S.total = (int64_t)P->nlam * P->o.nphot;
    S.nlam = P->nlam;
    S.ns = P->ns;
    S.key0 = (uint32_t)(P->o.seed & 0xffffffffu);
    S.key1 = (uint32_t)(P->o.seed >> 32);
    S.maxtauabs = P->o.maxtauabs;
    S.max_scatter = P->o.max_scatter;
    sc_transport_kernel<<<P->grid, P->block, 0, st>>>(S);
    int fg = (int)std::min<int64_t>((ncl + 255) / 256, (int64_t)P->nsm * 8);
    if (fg < 1) fg = 1;
    sc_finish_kernel<<<fg, 256, 0, st>>>(P->M, dp, S.invdr, S.lam, S.acc, P->nlam, J);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_scat_plan_stats(pdgpu_scat_plan* P, const void* ws, void* stream,
                                   pdgpu_scat_stats* out) {
    if (!P || !ws || !out) return PDGPU_INVALID_ARG;
    int64_t s[SS_N];
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(s, (const char*)ws + P->ws_stats, sizeof(s), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    memset(out, 0, sizeof(*out));
    out->packets = (int64_t)P->nlam * P->o.nphot;
    out->escaped = s[SS_ESCAPED];
    out->dropped = s[SS_DROPPED];
    out->capped = s[SS_CAPPED] + s[SS_KILLED];
    out->scatterings = s[SS_SCATTER];
    out->crossings = s[SS_CROSS];
    out->status = (int32_t)s[SS_STATUS];
    return PDGPU_OK;
}

}  // extern "C"
