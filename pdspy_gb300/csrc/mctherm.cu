// Thermal Monte Carlo photon transport on spherical grids (GB300, sm_103a).
//
// Replaces the "radmc3d mctherm" subprocess behind pdspy's Model.run_thermal
// (pdspy/modeling/Model.py:221-256, pdspy/radmc3d/run.py:9-38).  Methods: Bjorkman &
// Wood 2001 immediate reemission with integer energy counting, made order-independent
// by epochs (below); the modified random walk of Min et al. 2009 / Robitaille 2010;
// Philox4x32-10 random numbers keyed by (seed; draw block, packet, model, pass).
//
// Execution model.  One persistent kernel per epoch.  Each thread owns one packet at a
// time; its whole state lives in registers (structure-of-arrays across the warp).  When
// packets finish, the warp refills the free lanes with one warp-aggregated atomicAdd on
// the epoch's work counter (ballot + popc + shfl), so the queue is read with one
// atomic per refill instead of one per packet.  Models of a batched plan are
// interleaved in the same queue.  Opacity, reemission-row, reemission-CDF and MRW tables
// are staged in shared memory when they fit.  Absorbed energy is accumulated in int64
// fixed point (2^20 units per packet) with atomicAdd, so the sum does not depend on the
// order of the atomics and a run is bit-reproducible for a given seed.
//
// Deterministic B&W.  Packets [b_k, b_{k+1}) form epoch k; sizes double from epoch to
// epoch.  In epoch k the reemission temperature of an absorption in cell c is taken at
// q' = q_lo + u * q_span (energy absorbed per gram per second), with q_lo from the
// energy absorbed in earlier epochs and q_span = q_lo (b_{k+1}/b_k - 1) its expected
// growth over the epoch.  The first epoch runs npilot pilot passes that estimate its own
// span.
//
// Precision.  Radiative quantities (optical depths, opacities, random numbers, reemission
// sampling) are FP32.  The packet position, the safety distance and the wall-intersection
// roots use double-single arithmetic on the FP32 pipe (mc_geom_ds.cuh explains why FP64 is
// not used for them on GB300); the same kernels instantiated with FP64 geometry
// (mc_geom.cuh) are selected by pdgpu_mc_options.fp64_walls and serve as the precision
// reference.  The energy -> temperature inversion is FP64 (once per cell).
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <new>
#include <vector>
#include <type_traits>

#include "../../include/pdgpu.h"
#include "mc_common.h"
#include "mc_device.cuh"
#include "mc_geom.cuh"
#include "mc_geom_ds.cuh"
#include "mc_host.h"

namespace {
using namespace pdgpu;

// Saved state of a parked packet (its random numbers follow from the packet id and its
// interaction count).  pos holds the position bits of either geometry.
struct __align__(16) ParkRec {
    uint64_t pos[3];
    long long own_u[MC_OWN];
    float dsafe, kx, ky, kz, tau;
    int ir, itv, ip, lam;
    int last_wall, cell_events, nevents, ncross;
    int m, epoch;
    uint32_t pid, model, tag, spare;   // spare: bits of dmax
    int own_sc[MC_OWN];
    int own_next, own_ver, fresh, pad;
};

struct DustTabs {       // pointers into the staged (shared or global) dust tables
    const float* kabs;  // [ns][nl]
    const float* ksca;
    const float* kext;
    const float* g;
    const float* F;     // [ns][NROW]
    const float* cdf;   // [ns][NROW][nl]
    const float* kP;    // [ns][NROW]
    const float* kR;
    const float* mrw;   // [NMRW]
};

struct McParams {
    const float* fpool;
    const double* dpool;
    const McModel* models;
    const int64_t* cum;          // [nm+1] prefix of this epoch's packet counts
    const float* rho;            // [model][spec][cell]
    const float* wq;             // [model][spec][cell] (float)(q_unit / cell mass)
    int64_t* E;                  // deposits of a packet's first late_after events
    int64_t* Elate;              // deposits of its later events
    const float2* q;             // (q_lo, q_span) per [epoch][model][spec][cell]
    int64_t qstride;             // cells per epoch snapshot
    int64_t late_after;          // 0: all deposits go to E
    ParkRec* park_out;           // phase 0: packets parked after late_after events;
    unsigned long long* park_out_count;   // phase 1: packets drained for phase 2
    int64_t park_out_cap;
    const ParkRec* park_in;      // phases 1 and 2: the packets to resume
    const unsigned long long* park_in_count;
    int64_t park_in_cap;
    unsigned long long* inflight;   // packets taken and not yet finished (when draining)
    int64_t drain_below;         // drain when fewer are in flight (0 = never)
    ParkRec* drain_out;          // drained packets, resumed one per warp
    unsigned long long* drain_out_count;
    int32_t pilot;               // pilot pass: packets stop after late_after events
    int32_t phase;               // 0: epoch launch; 1: parked packets, one per thread;
                                 // 2: drained packets, one per warp
    int32_t lslot;               // per-launch debug slot
    int64_t* escape;             // [nm][nl] or null
    int64_t* stats;              // [MC_NSTAT]
    unsigned long long* queue;   // work counter of this launch
    const volatile int32_t* abort_flag;
    int64_t deadline_ns;
    const int64_t* mdeadline;    // [nm] per-model deadline (ns from the run's start, 0 = none)
    int32_t* mstat;              // [nm] per-model status (0 = running/ok, else why it stopped)
    int32_t use_mdl;             // 1: per-model deadlines are set
    int64_t total;
    int32_t nm, ns, nl, epoch;
    uint32_t tag, key0, key1;
    int32_t mrw, mrw_trigger;
    int32_t mrw_eager_after;
    float mrw_gamma, mrw_tauthres;
    int32_t max_inter;
    int32_t dust_floats, use_smem;
    int32_t o_kabs, o_ksca, o_kext, o_g, o_F, o_cdf, o_kP, o_kR, o_mrw;
    int32_t count_stats;
    int32_t g_const;             // 1: every species has the one asymmetry g0 at every wavelength
    float g0;
};

struct Cnt {
    long long killed, escaped, crossings, events, absorb, scatter, mrw, late, parked, drained;
    int maxev;
};

// Geometry policies of the transport step.
//
// GeoS: double-single positions and walls (mc_geom_ds.cuh), the default.
// GeoD: the same walk with FP64 positions and walls (mc_geom.cuh), the precision reference.
// Each provides the packet type, the length type of a move, and the wall operations for a
// packet per thread (wall_lane) or per warp (wall_warp: candidate k on lane k, reduced with
// the serial tie-break, first candidate with the smallest distance).
struct GeoS {
    using Pkt = PktS;
    using len_t = ds;   // wall distances keep the Newton correction as the lo part
    static __device__ __forceinline__ ds of(float v) { return ds{v, 0.0f}; }
    static __device__ __forceinline__ float f(ds v) { return v.h; }
    static __device__ __forceinline__ bool gt(ds a, ds b) { return a.h > b.h; }
    static __device__ __forceinline__ int cell(const McModel& M, const Pkt& p) { return cell_of_s(M, p); }
    static __device__ __forceinline__ ds wall_lane(const McModel& M, const double*, const float* fp,
                                                   const Pkt& p, int& w) {
        WallsS W(M, fp);
        return next_wall_ds(M, W, p, w);
    }
    static __device__ __forceinline__ ds wall_warp(int lane, const McModel& M, const double*,
                                                   const float* fp, const Pkt& p, int& w) {
        return wall_warp_w(lane, M, WallsS(M, fp), p, w);
    }
    template <class Wl>
    static __device__ __forceinline__ ds wall_warp_w(int lane, const McModel& M, const Wl& W,
                                                     const Pkt& p, int& w) {
        FrameS f;
        frame_ds(M, W, p, f);
        const int nk = (p.ir < 0) ? 1 : (M.np > 1 ? 6 : 4);
        float s = 3.0e38f;
        int k = 64 + lane;
        if (lane < nk) {
            float v;
            if (candidate_ds(M, W, p, f, lane, v)) { s = v; k = lane; }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            float so = __shfl_xor_sync(0xffffffffu, s, o);
            int ko = __shfl_xor_sync(0xffffffffu, k, o);
            if (so < s || (so == s && ko < k)) { s = so; k = ko; }
        }
        s = __shfl_sync(0xffffffffu, s, 0);
        k = __shfl_sync(0xffffffffu, k, 0);
        if (k >= 64) { w = W_NONE; return ds{3.0e38f, 0.0f}; }
        w = cand_wall_code(k);
        return refine_ds(M, W, p, f, k, s);
    }
    static __device__ __forceinline__ float dist(const McModel& M, const double*, const float* fp,
                                                 const Pkt& p) {
        WallsS W(M, fp);
        return wall_distance_ds(M, W, p);
    }
    static __device__ __forceinline__ float dist_warp(int lane, const McModel& M, const double*,
                                                      const float* fp, const Pkt& p) {
        WallsS W(M, fp);
        return wall_distance_ds_warp(M, W, p, lane);
    }
    static __device__ __forceinline__ void locate(const McModel& M, const double*, const float* fp,
                                                  Pkt& p) {
        WallsS W(M, fp);
        locate_angles_ds(M, W, p);
    }
    static __device__ __forceinline__ void move(Pkt& p, ds s, float kx, float ky, float kz) {
        p.x = ds_move2(p.x, s, kx);
        p.y = ds_move2(p.y, s, ky);
        p.z = ds_move2(p.z, s, kz);
    }
    static __device__ __forceinline__ void origin(Pkt& p) {
        p.x = ds{0.0f, 0.0f}; p.y = ds{0.0f, 0.0f}; p.z = ds{0.0f, 0.0f};
    }
    static __device__ __forceinline__ uint64_t pack(ds v) {
        return (uint64_t)__float_as_uint(v.h) | ((uint64_t)__float_as_uint(v.l) << 32);
    }
    static __device__ __forceinline__ ds unpack(uint64_t b) {
        return ds{__uint_as_float((uint32_t)b), __uint_as_float((uint32_t)(b >> 32))};
    }
    static __device__ __forceinline__ void save(ParkRec& r, const Pkt& p) {
        r.pos[0] = pack(p.x); r.pos[1] = pack(p.y); r.pos[2] = pack(p.z);
    }
    static __device__ __forceinline__ void load(Pkt& p, const ParkRec& r) {
        p.x = unpack(r.pos[0]); p.y = unpack(r.pos[1]); p.z = unpack(r.pos[2]);
    }
};

struct GeoD {
    using Pkt = pdgpu::Pkt;
    using len_t = double;
    static __device__ __forceinline__ double of(float v) { return (double)v; }
    static __device__ __forceinline__ float f(double v) { return (float)v; }
    static __device__ __forceinline__ bool gt(double a, double b) { return a > b; }
    static __device__ __forceinline__ int cell(const McModel& M, const Pkt& p) { return cell_of(M, p); }
    static __device__ __forceinline__ double wall_lane(const McModel& M, const double* dp, const float*,
                                                       const Pkt& p, int& w) {
        return next_wall(M, dp, p, w);
    }
    static __device__ __forceinline__ double wall_warp(int lane, const McModel& M, const double* dp,
                                                       const float*, const Pkt& p, int& w) {
        WallFrame f;
        wall_frame(M, dp, p, f);
        const int nk = (p.ir < 0) ? 1 : (M.np > 1 ? 6 : 4);
        double s = 1.0e300;
        int k = 64 + lane;
        if (lane < nk) {
            double v;
            if (wall_candidate(M, dp, p, f, lane, v)) { s = v; k = lane; }
        }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
            double so = __shfl_xor_sync(0xffffffffu, s, o);
            int ko = __shfl_xor_sync(0xffffffffu, k, o);
            if (so < s || (so == s && ko < k)) { s = so; k = ko; }
        }
        s = __shfl_sync(0xffffffffu, s, 0);
        k = __shfl_sync(0xffffffffu, k, 0);
        w = (k < 64) ? wall_code(k) : W_NONE;
        return (k < 64) ? s : 1.0e300;
    }
    static __device__ __forceinline__ float dist(const McModel& M, const double* dp, const float* fp,
                                                 const Pkt& p) {
        return wall_distance(M, dp, fp, p);
    }
    static __device__ __forceinline__ float dist_warp(int, const McModel& M, const double* dp,
                                                      const float* fp, const Pkt& p) {
        return wall_distance(M, dp, fp, p);
    }
    static __device__ __forceinline__ void locate(const McModel& M, const double* dp, const float*,
                                                  Pkt& p) {
        locate_angles(M, dp, p);
    }
    static __device__ __forceinline__ void move(Pkt& p, double s, float kx, float ky, float kz) {
        p.x = fma(s, (double)kx, p.x);
        p.y = fma(s, (double)ky, p.y);
        p.z = fma(s, (double)kz, p.z);
    }
    static __device__ __forceinline__ void origin(Pkt& p) { p.x = 0.0; p.y = 0.0; p.z = 0.0; }
    static __device__ __forceinline__ void save(ParkRec& r, const Pkt& p) {
        r.pos[0] = (uint64_t)__double_as_longlong(p.x);
        r.pos[1] = (uint64_t)__double_as_longlong(p.y);
        r.pos[2] = (uint64_t)__double_as_longlong(p.z);
    }
    static __device__ __forceinline__ void load(Pkt& p, const ParkRec& r) {
        p.x = __longlong_as_double((long long)r.pos[0]);
        p.y = __longlong_as_double((long long)r.pos[1]);
        p.z = __longlong_as_double((long long)r.pos[2]);
    }
};

// Uniforms (and the quantities derived from them alone) of one interaction, by stream.
struct EvR {
    float ua, tn, umu, cs, sn;   // albedo test, new optical depth, cosine, azimuth sin/cos
};
struct SecR {
    float uq, urow, ucdf, us;    // reemission q', row and CDF picks, species pick
};
struct MrwR {
    float uy, jmu, jcs, jsn;     // diffusion time, jump cosine and azimuth
};

__device__ __forceinline__ EvR ev_of(uint4 b) {
    EvR r;
    r.ua = mc_u01(b.x);
    r.tn = -mc_logf(mc_u01(b.y));
    r.umu = mc_u01(b.z);
    mc_sincospif2(mc_u01(b.w), r.sn, r.cs);
    return r;
}
__device__ __forceinline__ SecR sec_of(uint4 b) {
    SecR r;
    r.uq = mc_u01(b.x); r.urow = mc_u01(b.y); r.ucdf = mc_u01(b.z); r.us = mc_u01(b.w);
    return r;
}
__device__ __forceinline__ MrwR mrw_of(uint4 b) {
    MrwR r;
    r.uy = mc_u01(b.x);
    r.jmu = 2.0f * mc_u01(b.y) - 1.0f;
    mc_sincospif2(mc_u01(b.z), r.jsn, r.jcs);
    return r;
}

template <class Pol>
__device__ __forceinline__ int reemit_lambda(Pol& pol, const DustTabs& T, int nl, float2 q, int s,
                                             float uq, float urow, float ucdf, float own);

// Henyey-Greenstein scattering cosine for asymmetry g from the uniform umu (isotropic
// below |g| = 1e-4).
__device__ __forceinline__ float hg_mu(float g, float umu) {
    float mu;
    if (fabsf(g) < 1.0e-4f) {
        mu = 2.0f * umu - 1.0f;
    } else {
        float t = (1.0f - g * g) / (1.0f - g + 2.0f * g * umu);
        mu = (1.0f + g * g - t * t) / (2.0f * g);
        if (mu < -1.0f) mu = -1.0f;
        if (mu > 1.0f) mu = 1.0f;
    }
    return mu;
}

// Isotropic direction from an interaction's cosine and azimuth uniforms.
__device__ __forceinline__ void iso_of(const EvR& ev, float& kx, float& ky, float& kz) {
    float mu = 2.0f * ev.umu - 1.0f;
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    kx = st * ev.cs; ky = st * ev.sn; kz = mu;
}

// Execution policies of the transport step.
//
// LanePol: one packet per thread (the epoch launches and the first continuation stage).
// WarpPol: one packet per warp, its state replicated in all 32 lanes (the last, longest
// walks, whose sequential chains set the run time), organised for latency: the random
// numbers of the next 32 interactions are drawn at once (lane l holds interaction n0 + l,
// an interaction reads its values with shuffles), the cell's Rosseland and Planck means
// are kept while the packet stays in the cell, table searches count entries with ballots,
// and wall candidates and wall distances are computed one wall per lane.  Every result is
// identical to the per-thread code; memory side effects are issued by lane 0.
struct LanePol {
    // the packet's own-deposit cache (McOwn) in shared memory, structure of arrays over the
    // block's threads: keys [MC_OWN][nthr], units [MC_OWN][nthr], next [nthr]
    int* osc;
    long long* ou;
    int* onext;
    int tid, nthr;
    __device__ __forceinline__ void own_reset() {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i) { osc[i * nthr + tid] = -1; ou[i * nthr + tid] = 0; }
        onext[tid] = 0;
    }
    __device__ __forceinline__ void own_add(int sc, long long units) {
        bool hit = false;
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i)
            if (osc[i * nthr + tid] == sc) { ou[i * nthr + tid] += units; hit = true; }
        if (!hit) {
            const int nx = onext[tid];
            osc[nx * nthr + tid] = sc;
            ou[nx * nthr + tid] = units;
            onext[tid] = (nx + 1) & (MC_OWN - 1);
        }
    }
    __device__ __forceinline__ float own_q(int sc, float wq) const {
        long long u = 0;
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i)
            if (osc[i * nthr + tid] == sc) u = ou[i * nthr + tid];
        return u != 0 ? (float)u * wq : 0.0f;
    }
    __device__ __forceinline__ int own_ver() const { return 0; }
    __device__ __forceinline__ void own_save(ParkRec& r) const {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i) { r.own_sc[i] = osc[i * nthr + tid]; r.own_u[i] = ou[i * nthr + tid]; }
        r.own_next = onext[tid];
        r.own_ver = 0;
    }
    __device__ __forceinline__ void own_load(const ParkRec& r) {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i) { osc[i * nthr + tid] = r.own_sc[i]; ou[i * nthr + tid] = r.own_u[i]; }
        onext[tid] = r.own_next;
    }
    __device__ __forceinline__ int cdf(const float* c, int n, float u) const {
        return mc_cdf_search(c, n, u);
    }
    __device__ __forceinline__ void row(const float* F, float q, int& j, float& w) const {
        mc_row_search(F, q, j, w);
    }
    template <class G>
    __device__ __forceinline__ typename G::len_t wall(const McModel& M, const double* dp,
                                                      const float* fp, const typename G::Pkt& p,
                                                      int& w) const {
        return G::wall_lane(M, dp, fp, p, w);
    }
    template <class G>
    __device__ __forceinline__ float dist(const McModel& M, const double* dp, const float* fp,
                                          const typename G::Pkt& p) const {
        return G::dist(M, dp, fp, p);
    }
    __device__ __forceinline__ EvR ev(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        return ev_of(mc_block(r, n, MC_RS_EVENT, k0, k1));
    }
    __device__ __forceinline__ SecR second(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        return sec_of(mc_block(r, n, MC_RS_SECOND, k0, k1));
    }
    __device__ __forceinline__ MrwR mrwd(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        return mrw_of(mc_block(r, n, MC_RS_MRW, k0, k1));
    }
    __device__ __forceinline__ void iso_dir(uint32_t, const EvR& ev, float& kx, float& ky,
                                            float& kz) const {
        iso_of(ev, kx, ky, kz);
    }
    __device__ __forceinline__ float hg(uint32_t, float g, float umu) const { return hg_mu(g, umu); }
    template <int NS>
    __device__ __forceinline__ int reemit(const DustTabs& T, int nl, float2 q, int s, const SecR& sb,
                                          float own, int, int, int, uint32_t);
    __device__ __forceinline__ bool cached(int, int, int, int, int) const { return false; }
    __device__ __forceinline__ void remember(int, int, int, int, int, float) {}
    // q per deposit unit of species s in cell c (wq0 = the model's [spec][cell] block)
    template <int NS>
    __device__ __forceinline__ float wq(const float* wq0, int ncell, int, int c, int s) const {
        return __ldg(wq0 + (int64_t)s * ncell + c);
    }
    __device__ __forceinline__ float cached_value(int) const { return 0.0f; }
    __device__ __forceinline__ bool leader() const { return true; }
    __device__ __forceinline__ unsigned long long bcast(unsigned long long v) const { return v; }
    // densities of cell c (rho0 = the model's [spec][cell] block)
    template <int NS>
    __device__ __forceinline__ void density(const float* rho0, int ncell, int, int c, float* rh) {
#pragma unroll
        for (int s = 0; s < NS; ++s) rh[s] = __ldg(rho0 + (int64_t)s * ncell + c);
    }
    // snapshot (q_lo, q_span) of species s in cell c (q0 = the epoch's [spec][cell] block)
    template <int NS>
    __device__ __forceinline__ float2 snap(const float2* q0, int ncell, int, int c, int, int s) {
        return q0[(int64_t)s * ncell + c];
    }
};

struct WarpPol {
    int lane;
    // random numbers of interactions n0 .. n0 + 31, lane l holding n0 + l
    bool rv, rmv;
    uint32_t n0;
    EvR re;
    SecR rs;
    MrwR rm;
    // derived per lane at the refill: the isotropic direction and, when every species has
    // one wavelength-independent asymmetry g0 (gconst), the Henyey-Greenstein cosine
    float ikx, iky, ikz, hgmu;
    int gconst;
    float g0;
    // reemission of lane l's interaction as if it were an absorption of species 0 in cell
    // (sk_m, sk_c) of epoch sk_e with the own deposits of when it was made (one-species
    // walks): bucket of the row table (0 below, 1 inside, 2 above), row index j and its
    // bounds, reemission row and wavelength bin
    int sk_m = -1, sk_c = -1, sk_e = -1;
    uint32_t sk_n0 = 0xffffffffu;
    int sp_case, sp_j, sp_row, sp_lam;
    float sp_Fj, sp_Fj1;
    // per-cell cache: (model, cell, epoch, own-deposit version) -> values by slot
    // (Rosseland, Planck per species)
    int cm, cc, ce, cv;
    unsigned cvalid;
    float cval[1 + MC_MAX_SPEC];
    // the packet's own-deposit cache, replicated in every lane
    McOwn own;
    __device__ __forceinline__ explicit WarpPol(int l, int gc, float g)
        : lane(l), rv(false), rmv(false), n0(0), gconst(gc), g0(g), cm(-1), cc(-1), ce(-1), cv(-1),
          cvalid(0u) { own_init(own); }
    __device__ __forceinline__ void own_reset() { own_init(own); }
    __device__ __forceinline__ void own_add(int sc, long long units) { ::own_add(own, sc, units); }
    __device__ __forceinline__ float own_q(int sc, float wq) const { return ::own_q(own, sc, wq); }
    __device__ __forceinline__ int own_ver() const { return own.ver; }
    __device__ __forceinline__ void own_save(ParkRec& r) const {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i) { r.own_sc[i] = own.sc[i]; r.own_u[i] = own.u[i]; }
        r.own_next = own.next;
        r.own_ver = own.ver;
    }
    __device__ __forceinline__ void own_load(const ParkRec& r) {
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i) { own.sc[i] = r.own_sc[i]; own.u[i] = r.own_u[i]; }
        own.next = r.own_next;
        own.ver = r.own_ver;
    }
    // number of entries <= u of a non-decreasing table == smallest index with c > u
    __device__ __forceinline__ int cdf(const float* c, int n, float u) const {
        if (n <= 128) {   // four independent loads, then the ballots (u < 1 < 2)
            const float v0 = lane < n ? c[lane] : 2.0f;
            const float v1 = 32 + lane < n ? c[32 + lane] : 2.0f;
            const float v2 = 64 + lane < n ? c[64 + lane] : 2.0f;
            const float v3 = 96 + lane < n ? c[96 + lane] : 2.0f;
            return (__popc(__ballot_sync(0xffffffffu, v0 <= u)) +
                    __popc(__ballot_sync(0xffffffffu, v1 <= u))) +
                   (__popc(__ballot_sync(0xffffffffu, v2 <= u)) +
                    __popc(__ballot_sync(0xffffffffu, v3 <= u)));
        }
        int cnt = 0;
        for (int b = 0; b < n; b += 32) {
            int l = b + lane;
            bool le = (l < n) && (c[l] <= u);
            cnt += __popc(__ballot_sync(0xffffffffu, le));
        }
        return cnt;
    }
    __device__ __forceinline__ void row(const float* F, float q, int& j, float& w) const {
        int cnt = 0;
#pragma unroll
        for (int b = 0; b < MC_NROW; b += 32) cnt += __popc(__ballot_sync(0xffffffffu, F[b + lane] <= q));
        if (cnt == 0) {
            j = 0;
            w = 0.0f;
        } else if (cnt == MC_NROW) {
            j = MC_NROW - 2;
            w = 1.0f;
        } else {
            j = cnt - 1;
            w = (q - F[j]) / (F[j + 1] - F[j]);
            if (w < 0.0f) w = 0.0f;
            if (w > 1.0f) w = 1.0f;
        }
    }
    // walls of the packet's current cell in registers (double-single geometry), reloaded
    // when (ir, itv, ip) changes
    int wir = -2, witv = -1, wip = -1;
    WallsCell wcell;
    __device__ __forceinline__ const WallsCell& cell_walls(const McModel& M, const float* fp,
                                                           const PktS& p) {
        if (p.ir != wir || p.itv != witv || p.ip != wip) {
            wcell.load(WallsS(M, fp), p.ir, p.itv, p.ip, M.np);
            wir = p.ir; witv = p.itv; wip = p.ip;
        }
        return wcell;
    }
    template <class G>
    __device__ __forceinline__ typename G::len_t wall(const McModel& M, const double* dp,
                                                      const float* fp, const typename G::Pkt& p,
                                                      int& w) {
        if constexpr (std::is_same<G, GeoS>::value) {
            return G::wall_warp_w(lane, M, cell_walls(M, fp, p), p, w);
        } else {
            return G::wall_warp(lane, M, dp, fp, p, w);
        }
    }
    template <class G>
    __device__ __forceinline__ float dist(const McModel& M, const double* dp, const float* fp,
                                          const typename G::Pkt& p) {
        if constexpr (std::is_same<G, GeoS>::value) {
            return wall_distance_ds_warp(M, cell_walls(M, fp, p), p, lane);
        } else {
            return G::dist_warp(lane, M, dp, fp, p);
        }
    }
    __device__ __forceinline__ int slot(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        if (!rv || n < n0 || n - n0 >= 32u) {
            n0 = n;
            const uint32_t m = n + (uint32_t)lane;
            re = ev_of(mc_block(r, m, MC_RS_EVENT, k0, k1));
            rs = sec_of(mc_block(r, m, MC_RS_SECOND, k0, k1));
            rmv = false;   // the MRW stream is drawn when a jump first needs it
            iso_of(re, ikx, iky, ikz);
            hgmu = gconst ? hg_mu(g0, re.umu) : 0.0f;
            rv = true;
        }
        return (int)(n - n0);
    }
    // random numbers of interactions n .. n + 31, lane l holding n + l
    __device__ __forceinline__ void refill_at(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        if (!rv || n0 != n) {
            rv = false;
            slot(r, n, k0, k1);
        }
    }
    __device__ __forceinline__ EvR ev(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        const int l = slot(r, n, k0, k1);
        EvR o;
        o.ua = __shfl_sync(0xffffffffu, re.ua, l);
        o.tn = __shfl_sync(0xffffffffu, re.tn, l);
        o.umu = __shfl_sync(0xffffffffu, re.umu, l);
        o.cs = __shfl_sync(0xffffffffu, re.cs, l);
        o.sn = __shfl_sync(0xffffffffu, re.sn, l);
        return o;
    }
    __device__ __forceinline__ SecR second(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        const int l = slot(r, n, k0, k1);
        SecR o;
        o.uq = __shfl_sync(0xffffffffu, rs.uq, l);
        o.urow = __shfl_sync(0xffffffffu, rs.urow, l);
        o.ucdf = __shfl_sync(0xffffffffu, rs.ucdf, l);
        o.us = __shfl_sync(0xffffffffu, rs.us, l);
        return o;
    }
    __device__ __forceinline__ MrwR mrwd(const McRng& r, uint32_t n, uint32_t k0, uint32_t k1) {
        const int l = slot(r, n, k0, k1);
        if (!rmv) {
            rm = mrw_of(mc_block(r, n0 + (uint32_t)lane, MC_RS_MRW, k0, k1));
            rmv = true;
        }
        MrwR o;
        o.uy = __shfl_sync(0xffffffffu, rm.uy, l);
        o.jmu = __shfl_sync(0xffffffffu, rm.jmu, l);
        o.jcs = __shfl_sync(0xffffffffu, rm.jcs, l);
        o.jsn = __shfl_sync(0xffffffffu, rm.jsn, l);
        return o;
    }
    __device__ __forceinline__ void iso_dir(uint32_t n, const EvR&, float& kx, float& ky, float& kz) const {
        const int l = (int)(n - n0);
        kx = __shfl_sync(0xffffffffu, ikx, l);
        ky = __shfl_sync(0xffffffffu, iky, l);
        kz = __shfl_sync(0xffffffffu, ikz, l);
    }
    __device__ __forceinline__ float hg(uint32_t n, float g, float umu) const {
        if (gconst) return __shfl_sync(0xffffffffu, hgmu, (int)(n - n0));
        return hg_mu(g, umu);
    }
    // Reemission wavelength of interaction n (an absorption of species s in cell c of model m,
    // epoch e): the same result as reemit_lambda.  One-species walks use the lanes'
    // speculative results, made for the whole block of 32 interactions at the first
    // absorption in a cell: the true q' (which includes every own deposit made since) is
    // checked against the speculative row bucket, and only the row decision is redone
    // when it stays inside it.
    template <int NS>
    __device__ __forceinline__ int reemit(const DustTabs& T, int nl, float2 q, int s, const SecR& sb,
                                          float own, int m, int c, int e, uint32_t n) {
        if (NS > 1) return reemit_lambda(*this, T, nl, q, s, sb.uq, sb.urow, sb.ucdf, own);
        if (m != sk_m || c != sk_c || e != sk_e || n0 != sk_n0) {
            float qq = q.x + rs.uq * q.y;
            qq = qq + own;
            int j;
            float w;
            mc_row_search(T.F, qq, j, w);
            sp_case = (qq < T.F[0]) ? 0 : (qq >= T.F[MC_NROW - 1]) ? 2 : 1;
            sp_j = j;
            sp_Fj = T.F[j];
            sp_Fj1 = T.F[j + 1];
            sp_row = j + ((rs.urow < w) ? 1 : 0);
            sp_lam = mc_cdf_search(T.cdf + (size_t)sp_row * nl, nl, rs.ucdf);
            sk_m = m; sk_c = c; sk_e = e; sk_n0 = n0;
        }
        const int l = (int)(n - n0);
        const int cs_ = __shfl_sync(0xffffffffu, sp_case, l);
        const int j = __shfl_sync(0xffffffffu, sp_j, l);
        const int row = __shfl_sync(0xffffffffu, sp_row, l);
        const int lam = __shfl_sync(0xffffffffu, sp_lam, l);
        const float Fj = __shfl_sync(0xffffffffu, sp_Fj, l);
        const float Fj1 = __shfl_sync(0xffffffffu, sp_Fj1, l);
        float qq = q.x + sb.uq * q.y;
        qq = qq + own;
        if (cs_ == 0) {
            if (qq < Fj) return lam;
        } else if (cs_ == 2) {
            if (qq >= Fj1) return lam;
        } else if (Fj <= qq && qq < Fj1) {
            float w = (qq - Fj) / (Fj1 - Fj);
            if (w < 0.0f) w = 0.0f;
            if (w > 1.0f) w = 1.0f;
            const int rt = j + ((sb.urow < w) ? 1 : 0);
            if (rt == row) return lam;
            return cdf(T.cdf + (size_t)rt * nl, nl, sb.ucdf);
        }
        return reemit_lambda(*this, T, nl, q, s, sb.uq, sb.urow, sb.ucdf, own);
    }
    __device__ __forceinline__ bool cached(int m, int c, int e, int v, int k) const {
        return cm == m && cc == c && ce == e && cv == v && ((cvalid >> k) & 1u);
    }
    __device__ __forceinline__ void remember(int m, int c, int e, int v, int k, float x) {
        if (cm != m || cc != c || ce != e || cv != v) { cm = m; cc = c; ce = e; cv = v; cvalid = 0u; }
        cval[k] = x;
        cvalid |= 1u << k;
    }
    __device__ __forceinline__ float cached_value(int k) const { return cval[k]; }
    __device__ __forceinline__ bool leader() const { return lane == 0; }
    // lane 0's value in every lane
    __device__ __forceinline__ unsigned long long bcast(unsigned long long v) const {
        return __shfl_sync(0xffffffffu, v, 0);
    }
    // densities, q per deposit unit and snapshots of the packet's cell, reloaded when the
    // cell changes
    int dm = -1, dc = -1, qm = -1, qc = -1, qe = -1, wm = -1, wc = -1;
    float drho[MC_MAX_SPEC];
    float dwq[MC_MAX_SPEC];
    float2 dq[MC_MAX_SPEC];
    template <int NS>
    __device__ __forceinline__ float wq(const float* wq0, int ncell, int m, int c, int s) {
        if (m != wm || c != wc) {
#pragma unroll
            for (int k = 0; k < NS; ++k) dwq[k] = __ldg(wq0 + (int64_t)k * ncell + c);
            wm = m;
            wc = c;
        }
        float v = dwq[0];
#pragma unroll
        for (int k = 1; k < NS; ++k)
            if (k == s) v = dwq[k];
        return v;
    }
    template <int NS>
    __device__ __forceinline__ void density(const float* rho0, int ncell, int m, int c, float* rh) {
        if (m != dm || c != dc) {
#pragma unroll
            for (int s = 0; s < NS; ++s) drho[s] = __ldg(rho0 + (int64_t)s * ncell + c);
            dm = m;
            dc = c;
        }
#pragma unroll
        for (int s = 0; s < NS; ++s) rh[s] = drho[s];
    }
    template <int NS>
    __device__ __forceinline__ float2 snap(const float2* q0, int ncell, int m, int c, int e, int s) {
        if (m != qm || c != qc || e != qe) {
#pragma unroll
            for (int k = 0; k < NS; ++k) dq[k] = q0[(int64_t)k * ncell + c];
            qm = m;
            qc = c;
            qe = e;
        }
        float2 v = dq[0];
#pragma unroll
        for (int k = 1; k < NS; ++k)
            if (k == s) v = dq[k];
        return v;
    }
};

template <class Pol>
__device__ __forceinline__ float row_interp(Pol& pol, const DustTabs& T, const float* tab, float q,
                                            int s) {
    // q: the cell's energy per gram per second (mid-epoch snapshot + the packet's own)
    int j;
    float w;
    pol.row(T.F + s * MC_NROW, q, j, w);
    return tab[j] + w * (tab[j + 1] - tab[j]);
}

// Reemission wavelength bin of species s from the cell's (q_lo, q_span) snapshot and the
// three uniforms of the interaction's second stream.
template <class Pol>
__device__ __forceinline__ int reemit_lambda(Pol& pol, const DustTabs& T, int nl, float2 q, int s,
                                             float uq, float urow, float ucdf, float own) {
    float qq = q.x + uq * q.y;
    qq = qq + own;
    int j;
    float w;
    pol.row(T.F + s * MC_NROW, qq, j, w);
    int row = j + ((urow < w) ? 1 : 0);
    return pol.cdf(T.cdf + ((size_t)s * MC_NROW + row) * nl, nl, ucdf);
}

template <int NS>
__device__ __forceinline__ int LanePol::reemit(const DustTabs& T, int nl, float2 q, int s,
                                               const SecR& sb, float own, int, int, int, uint32_t) {
    return reemit_lambda(*this, T, nl, q, s, sb.uq, sb.urow, sb.ucdf, own);
}

template <class G>
__device__ __forceinline__ void emit(typename G::Pkt& p, const DustTabs& T, const float* star_cdf,
                                     int nl, uint32_t k0, uint32_t k1) {
    const uint4 e = mc_block(p.rng, 0u, MC_RS_EMIT, k0, k1);
    float mu = 2.0f * mc_u01(e.x) - 1.0f;
    float sn, cs;
    mc_sincospif2(mc_u01(e.y), sn, cs);
    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
    p.kx = st * cs;
    p.ky = st * sn;
    p.kz = mu;
    p.lam = mc_cdf_search(star_cdf, nl, mc_u01(e.z));
    p.tau = -mc_logf(mc_u01(e.w));
    G::origin(p);
    p.dsafe = 0.0f;
    p.dmax = MC_DMAX_UNKNOWN;
    p.fresh = 1;
    p.ir = -1; p.itv = 0; p.ip = 0;
    p.last_wall = W_NONE;
    p.cell_events = 0;
    p.nevents = 0;
    p.ncross = 0;
}

template <class G, class Pol>
__device__ __forceinline__ void park_save(ParkRec& r, const typename G::Pkt& p, const Pol& pol) {
    G::save(r, p);
    r.dsafe = p.dsafe;
    r.kx = p.kx; r.ky = p.ky; r.kz = p.kz; r.tau = p.tau;
    r.ir = p.ir; r.itv = p.itv; r.ip = p.ip; r.lam = p.lam;
    r.last_wall = p.last_wall; r.cell_events = p.cell_events;
    r.nevents = p.nevents; r.ncross = p.ncross; r.m = p.m; r.epoch = p.epoch;
    r.pid = p.rng.pid; r.model = p.rng.model; r.tag = p.rng.tag;
    r.spare = __float_as_uint(p.dmax);
    r.fresh = p.fresh; r.pad = 0;
    pol.own_save(r);
}

template <class G, class Pol>
__device__ __forceinline__ void park_load(typename G::Pkt& p, const ParkRec& r, Pol& pol) {
    G::load(p, r);
    p.dsafe = r.dsafe;
    p.kx = r.kx; p.ky = r.ky; p.kz = r.kz; p.tau = r.tau;
    p.ir = r.ir; p.itv = r.itv; p.ip = r.ip; p.lam = r.lam;
    p.last_wall = r.last_wall; p.cell_events = r.cell_events;
    p.nevents = r.nevents; p.ncross = r.ncross; p.m = r.m; p.epoch = r.epoch;
    p.rng.pid = r.pid; p.rng.model = r.model; p.rng.tag = r.tag;
    p.dmax = __uint_as_float(r.spare);
    p.fresh = r.fresh;
    pol.own_load(r);
}

// One transport step: a wall crossing or an interaction.  Returns false when the packet
// has left the grid or was killed.
template <int NS, class Pol, class G>
__device__ __forceinline__ bool mc_step(typename G::Pkt& p, const McParams& P, const McModel& M,
                                        const DustTabs& T, Cnt& cnt, Pol& pol) {
    using len_t = typename G::len_t;
    const double* __restrict__ dp = P.dpool;
    const int nl = P.nl;
    const uint32_t k0 = P.key0, k1 = P.key1;
    int c = -1;
    float alpha = 0.0f;
    float rh[NS];
    const int64_t base = M.cell_off;
    if (p.ir >= 0) {
        c = G::cell(M, p);
        pol.template density<NS>(P.rho + base, M.ncell, p.m, c, rh);
#pragma unroll
        for (int s = 0; s < NS; ++s) alpha = alpha + rh[s] * T.kext[s * nl + p.lam];
    }
    // Safety distance: an interaction closer than the isotropic distance to the nearest
    // wall needs no wall solve (the common case in optically thick cells).
    bool full = true;
    len_t se = G::of(0.0f);
    float sef = 0.0f;
    if (alpha > 0.0f) {
        sef = p.tau / alpha;
        // a safety distance not computed here is refreshed before paying for a wall solve
        if (!(sef < p.dsafe) && !p.fresh) {
            const float D = pol.template dist<G>(M, dp, P.fpool, p);
            p.dsafe = 0.999999f * D;
            p.dmax = mc_dmax_of(D);
            p.fresh = 1;
        }
        if (sef < p.dsafe) { full = false; se = G::of(sef); }
    }
    int wall = W_NONE;
    len_t sw = G::of(0.0f);
    float tcell = 0.0f;
    bool is_event = true;
    if (full) {
        sw = pol.template wall<G>(M, dp, P.fpool, p, wall);
        tcell = alpha * G::f(sw);
        is_event = tcell > p.tau;
        if (is_event) {
            se = G::of(p.tau / alpha);
            if (G::gt(se, sw)) se = sw;
        }
    }
    if (is_event) {
        G::move(p, se, p.kx, p.ky, p.kz);
        p.dsafe = full ? 0.0f : p.dsafe - sef;
        p.fresh = 0;
        p.last_wall = W_NONE;
        const uint32_t n = (uint32_t)p.nevents;   // index of this interaction
        p.cell_events += 1;
        p.nevents += 1;
        cnt.events += 1;
        const bool late = P.late_after > 0 && p.nevents > P.late_after;
        int64_t* dep = late ? P.Elate : P.E;
        const float2* qa = P.q + (int64_t)p.epoch * P.qstride;
        const EvR ev = pol.ev(p.rng, n, k0, k1);
        p.dmax = mc_dmax_after(p.dmax, G::f(se));
        bool did_mrw = false;
        // MRW is considered after mrw_count_trigger events in one cell, and at every event
        // once the packet has made more than mrw_eager_after events (it is trapped).  It is
        // tried (the wall distance computed) only when the upper bound of that distance
        // allows a jump; a try also refreshes the safety distance.
        const bool cond = P.mrw && (p.cell_events >= P.mrw_trigger ||
                                    (P.mrw_eager_after > 0 && p.nevents > P.mrw_eager_after));
        bool tried = false;
        float Dw = 0.0f;
        float2 qv[NS];
        float aR = 0.0f;
        if (cond && 0.999f * p.dmax * alpha >= P.mrw_tauthres) {
#pragma unroll
            for (int s = 0; s < NS; ++s) qv[s] = pol.template snap<NS>(qa + base, M.ncell, p.m, c, p.epoch, s);
            if (pol.cached(p.m, c, p.epoch, pol.own_ver(), 0)) {
                aR = pol.cached_value(0);
            } else {
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    float qm = qv[s].x + 0.5f * qv[s].y;
                    qm = qm + pol.own_q(s * M.ncell + c, pol.template wq<NS>(P.wq + base, M.ncell, p.m, c, s));
                    aR = aR + rh[s] * row_interp(pol, T, T.kR + s * MC_NROW, qm, s);
                }
                pol.remember(p.m, c, p.epoch, pol.own_ver(), 0, aR);
            }
            tried = 0.999f * p.dmax * aR >= P.mrw_gamma;
        }
        if (tried) {
            Dw = pol.template dist<G>(M, dp, P.fpool, p);
            float R0f = 0.999f * Dw;
            len_t R0 = G::of(R0f);
            if (R0f * aR >= P.mrw_gamma && R0f * alpha >= P.mrw_tauthres) {
                did_mrw = true;
                const MrwR mb = pol.mrwd(p.rng, n, k0, k1);
                const SecR sb = pol.second(p.rng, n, k0, k1);
                float uy = mb.uy;
                float f = uy * (float)(MC_NMRW - 1);
                int i = (int)f;
                if (i > MC_NMRW - 2) i = MC_NMRW - 2;
                float w = f - (float)i;
                float yv = T.mrw[i] + w * (T.mrw[i + 1] - T.mrw[i]);
                float ell = 3.0f * aR * R0f * R0f * yv;
                float kp[NS];
                float aP = 0.0f;
#pragma unroll
                for (int s = 0; s < NS; ++s) {
                    if (pol.cached(p.m, c, p.epoch, pol.own_ver(), 1 + s)) {
                        kp[s] = pol.cached_value(1 + s);
                    } else {
                        float qm = qv[s].x + 0.5f * qv[s].y;
                        qm = qm + pol.own_q(s * M.ncell + c,
                                        pol.template wq<NS>(P.wq + base, M.ncell, p.m, c, s));
                        kp[s] = rh[s] * row_interp(pol, T, T.kP + s * MC_NROW, qm, s);
                        pol.remember(p.m, c, p.epoch, pol.own_ver(), 1 + s, kp[s]);
                    }
                    aP = aP + kp[s];
                    float units_f = kp[s] * ell * 1048576.0f + 0.5f;
                    if (units_f > 9.0e18f) units_f = 9.0e18f;
                    long long units = (long long)units_f;
                    if (units > 0) {
                        if (pol.leader())
                            atomicAdd((unsigned long long*)(dep + base + (int64_t)s * M.ncell + c),
                                      (unsigned long long)units);
                        pol.own_add(s * M.ncell + c, units);
                    }
                }
                float dx, dy, dz;
                {
                    float mu = mb.jmu;
                    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
                    dx = st * mb.jcs; dy = st * mb.jsn; dz = mu;
                }
                G::move(p, R0, dx, dy, dz);
                {
                    float mu = sqrtf(ev.umu);
                    float kx = dx, ky = dy, kz = dz;
                    mc_rotate(kx, ky, kz, mu, ev.cs, ev.sn);
                    p.kx = kx; p.ky = ky; p.kz = kz;
                }
                int sp = 0;
                if (NS > 1) {
                    float us = sb.us * aP;
                    float acc = 0.0f;
                    sp = NS - 1;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        acc = acc + kp[s];
                        if (us < acc) { sp = s; break; }
                    }
                }
                float2 qs = qv[0];
#pragma unroll
                for (int s = 1; s < NS; ++s)
                    if (s == sp) qs = qv[s];
                p.lam = reemit_lambda(pol, T, nl, qs, sp, sb.uq, sb.urow, sb.ucdf,
                                      pol.own_q(sp * M.ncell + c, pol.template wq<NS>(P.wq + base, M.ncell, p.m, c, sp)));
                p.tau = ev.tn;
                p.cell_events = 0;
                cnt.mrw += 1;
            }
        }
        if (!did_mrw) {
            float ua = ev.ua;
            float asca = 0.0f;
#pragma unroll
            for (int s = 0; s < NS; ++s) asca = asca + rh[s] * T.ksca[s * nl + p.lam];
            if (ua * alpha < asca) {
                int sp = 0;
                if (NS > 1) {
                    const SecR sb = pol.second(p.rng, n, k0, k1);
                    float us = sb.us * asca;
                    float acc = 0.0f;
                    sp = NS - 1;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        acc = acc + rh[s] * T.ksca[s * nl + p.lam];
                        if (us < acc) { sp = s; break; }
                    }
                }
                const float mu = pol.hg(n, T.g[sp * nl + p.lam], ev.umu);
                mc_rotate(p.kx, p.ky, p.kz, mu, ev.cs, ev.sn);
                cnt.scatter += 1;
            } else {
                const SecR sb = pol.second(p.rng, n, k0, k1);
                int sp = 0;
                if (NS > 1) {
                    float aabs = 0.0f;
#pragma unroll
                    for (int s = 0; s < NS; ++s) aabs = aabs + rh[s] * T.kabs[s * nl + p.lam];
                    float us = sb.us * aabs;
                    float acc = 0.0f;
                    sp = NS - 1;
#pragma unroll
                    for (int s = 0; s < NS; ++s) {
                        acc = acc + rh[s] * T.kabs[s * nl + p.lam];
                        if (us < acc) { sp = s; break; }
                    }
                }
                int64_t idx = base + (int64_t)sp * M.ncell + c;
                if (pol.leader()) atomicAdd((unsigned long long*)(dep + idx), 1ull << MC_EUNIT_SHIFT);
                pol.own_add(sp * M.ncell + c, 1ll << MC_EUNIT_SHIFT);
                const float2 qs = pol.template snap<NS>(qa + base, M.ncell, p.m, c, p.epoch, sp);
                p.lam = pol.template reemit<NS>(
                    T, nl, qs, sp, sb,
                    pol.own_q(sp * M.ncell + c, pol.template wq<NS>(P.wq + base, M.ncell, p.m, c, sp)),
                    p.m, c, p.epoch, n);
                pol.iso_dir(n, ev, p.kx, p.ky, p.kz);
                cnt.absorb += 1;
            }
            p.tau = ev.tn;
        }
        if (did_mrw) Dw = pol.template dist<G>(M, dp, P.fpool, p);
        if (did_mrw || tried) {
            p.dsafe = 0.999999f * Dw;
            p.dmax = mc_dmax_of(Dw);
            p.fresh = 1;
        }
        if (late) cnt.late += 1;
        if (p.nevents >= P.max_inter) {
            cnt.killed += 1;
            return false;
        }
        if (P.late_after > 0 && p.nevents == P.late_after && P.phase == 0) {
            if (P.pilot) return false;   // later deposits of pilot packets are discarded
            unsigned long long slot = 0;
            if (pol.leader()) slot = atomicAdd(P.park_out_count, 1ull);
            slot = pol.bcast(slot);
            if ((long long)slot < P.park_out_cap) {
                if (pol.leader()) {
                    ParkRec r;
                    park_save<G>(r, p, pol);
                    P.park_out[slot] = r;
                }
                cnt.parked += 1;
                return false;
            }
        }
        return true;
    }
    G::move(p, sw, p.kx, p.ky, p.kz);
    p.tau = p.tau - tcell;
    p.dsafe = 0.0f;          // on a wall: a wall solve is due, nothing to refresh
    p.dmax = MC_DMAX_UNKNOWN;
    p.fresh = 1;
    p.ncross += 1;
    cnt.crossings += 1;
    p.cell_events = 0;
    switch (wall) {
        case W_ROUT:
            if (p.ir < 0) { p.ir = 0; G::locate(M, dp, P.fpool, p); }
            else p.ir += 1;
            p.last_wall = W_RIN;
            if (p.ir >= M.nr) {
                cnt.escaped += 1;
                if (P.escape && pol.leader()) atomicAdd((unsigned long long*)(P.escape + (int64_t)p.m * nl + p.lam), 1ull);
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

__device__ __forceinline__ long long warp_sum(long long v) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}

__device__ __forceinline__ unsigned long long globaltimer() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// A model of a batched plan whose own deadline has passed is stopped: its status records
// PDGPU_TIMEOUT, its remaining packets are dropped, and the other models go on (the
// batched counterpart of one walker's radmc3d subprocess reaching its timelimit).
__device__ __forceinline__ bool model_live(const McParams& P, int m) {
    if (!P.use_mdl) return true;
    if (*(volatile const int32_t*)(P.mstat + m) != 0) return false;
    const long long dl = P.mdeadline[m];
    if (dl > 0 && (long long)globaltimer() - *(volatile const long long*)(P.stats + ST_T0) > dl) {
        atomicCAS(P.mstat + m, 0, (int32_t)PDGPU_TIMEOUT);
        return false;
    }
    return true;
}

template <int NS, class G>
__global__ void __launch_bounds__(256, 2) mc_transport_kernel(McParams P) {
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    int64_t* s_cum = reinterpret_cast<int64_t*>(sm + ((P.use_smem ? P.dust_floats : 0) + 3) / 4 * 4);
    __shared__ int s_stop;
    __shared__ long long s_total;
    if (threadIdx.x == 0) {
        s_stop = (*(volatile long long*)(P.stats + ST_STOP) != 0) ? 1 : 0;
        long long tot = P.total;
        if (P.phase == 1) {
            long long c = (long long)*(volatile const unsigned long long*)P.park_in_count;
            tot = c < P.park_in_cap ? c : P.park_in_cap;
        }
        s_total = tot;
        atomicMin((unsigned long long*)(P.stats + MC_LSTAT + MC_LSTRIDE * P.lslot), (unsigned long long)globaltimer());
    }
    const float* tab = P.fpool;
    if (P.use_smem) {
        const float4* src = reinterpret_cast<const float4*>(P.fpool);
        int n4 = (P.dust_floats + 3) / 4;
        for (int i = threadIdx.x; i < n4; i += blockDim.x) smem4[i] = __ldg(src + i);
        tab = sm;
    }
    for (int i = threadIdx.x; i <= P.nm; i += blockDim.x) s_cum[i] = P.cum[i];
    __syncthreads();
    const long long total = s_total;
    DustTabs T;
    T.kabs = tab + P.o_kabs; T.ksca = tab + P.o_ksca; T.kext = tab + P.o_kext; T.g = tab + P.o_g;
    T.F = tab + P.o_F; T.cdf = tab + P.o_cdf; T.kP = tab + P.o_kP; T.kR = tab + P.o_kR;
    T.mrw = tab + P.o_mrw;

    const int lane = threadIdx.x & 31;
    const unsigned lt_mask = (1u << lane) - 1u;
    Cnt cnt = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    typename G::Pkt p;
    bool active = false;
    unsigned iter = 0;
    LanePol lanepol;
    {
        // own-deposit caches of the block's threads, after the model prefix sums
        char* ob = reinterpret_cast<char*>(s_cum + P.nm + 1);
        lanepol.osc = reinterpret_cast<int*>(ob);
        lanepol.ou = reinterpret_cast<long long*>(ob + (size_t)MC_OWN * blockDim.x * sizeof(int));
        lanepol.onext = reinterpret_cast<int*>(ob + (size_t)MC_OWN * blockDim.x * (sizeof(int) + sizeof(long long)));
        lanepol.tid = threadIdx.x;
        lanepol.nthr = blockDim.x;
    }
    bool queue_open = true;
    for (;;) {
        if (s_stop) break;
        unsigned need = queue_open ? __ballot_sync(0xffffffffu, !active) : 0u;
        if (need) {
            int n = __popc(need);
            unsigned long long basev = 0;
            if (lane == 0) basev = atomicAdd(P.queue, (unsigned long long)n);
            basev = __shfl_sync(0xffffffffu, basev, 0);
            if ((long long)basev + n >= total) queue_open = false;
            bool got = false;
            if (!active) {
                long long g = (long long)basev + __popc(need & lt_mask);
                if (g < total) {
                    bool live = true;
                    if (P.phase == 1) {
                        park_load<G>(p, P.park_in[g], lanepol);
                        live = model_live(P, p.m);
                    } else {
                        int lo = 0, hi = P.nm;
                        while (hi - lo > 1) {
                            int mid = (lo + hi) >> 1;
                            if (s_cum[mid] <= g) lo = mid; else hi = mid;
                        }
                        const McModel& M = P.models[lo];
                        p.m = lo;
                        p.epoch = P.epoch;
                        p.rng.pid = (uint32_t)(M.bnd[P.epoch] + (g - s_cum[lo]));
                        p.rng.model = (uint32_t)M.model_id;
                        p.rng.tag = P.tag;
                        live = model_live(P, lo);
                        if (live) {
                            emit<G>(p, T, P.fpool + M.off_star, P.nl, P.key0, P.key1);
                            lanepol.own_reset();
                        }
                    }
                    active = live;
                    got = live;
                }
            }
            if (P.drain_below > 0) {
                int ng = __popc(__ballot_sync(0xffffffffu, got));
                if (lane == 0 && ng) atomicAdd(P.inflight, (unsigned long long)ng);
            }
        }
        if (!__any_sync(0xffffffffu, active)) {
            if (!queue_open) break;
            continue;   // every packet drawn belonged to stopped models: draw again
        }
        const bool was = active;
        // packets of a model that has reached its own deadline are dropped
        if (active && P.use_mdl && (iter & 4095u) == 4095u && !model_live(P, p.m)) active = false;
        if (active) {
            active = mc_step<NS, LanePol, G>(p, P, P.models[p.m], T, cnt, lanepol);
            if (!active && p.nevents > cnt.maxev) cnt.maxev = p.nevents;
        }
        if (P.drain_below > 0) {
            int nf = __popc(__ballot_sync(0xffffffffu, was && !active));
            if (lane == 0 && nf) atomicAdd(P.inflight, (unsigned long long)(-(long long)nf));
            // few packets left: hand them to the warp-per-packet launch (an epoch's walks
            // resume there with the epoch's snapshot and still park at late_after)
            if (!queue_open && (iter & 63u) == 63u) {
                int dr = 0;
                if (lane == 0)
                    dr = (long long)*(volatile unsigned long long*)P.inflight < P.drain_below;
                dr = __shfl_sync(0xffffffffu, dr, 0);
                if (dr) {
                    bool parked = false;
                    if (active) {
                        unsigned long long slot = atomicAdd(P.drain_out_count, 1ull);
                        if ((long long)slot < P.park_out_cap) {
                            ParkRec r;
                            park_save<G>(r, p, lanepol);
                            P.drain_out[slot] = r;
                            parked = true;
                            active = false;
                            cnt.drained += 1;
                        }
                    }
                    int np = __popc(__ballot_sync(0xffffffffu, parked));
                    if (lane == 0 && np) atomicAdd(P.inflight, (unsigned long long)(-(long long)np));
                    if (!__any_sync(0xffffffffu, active)) break;
                }
            }
        }
        if (((++iter) & 4095u) == 0u) {
            int stop = 0;
            if (lane == 0) {
                if (*(volatile long long*)(P.stats + ST_STOP) != 0) stop = 1;
                if (P.abort_flag && *P.abort_flag != 0) {
                    atomicCAS((unsigned long long*)(P.stats + ST_STATUS), 0ull, (unsigned long long)PDGPU_ABORTED);
                    stop = 1;
                }
                if (P.deadline_ns > 0) {
                    long long t0 = P.stats[ST_T0];
                    if ((long long)globaltimer() - t0 > P.deadline_ns) {
                        atomicCAS((unsigned long long*)(P.stats + ST_STATUS), 0ull, (unsigned long long)PDGPU_TIMEOUT);
                        stop = 1;
                    }
                }
                if (stop) atomicExch((unsigned long long*)(P.stats + ST_STOP), 1ull);
            }
            stop = __shfl_sync(0xffffffffu, stop, 0);
            if (stop) break;
        }
    }
    if (P.count_stats) {
        long long v[10] = {cnt.killed, cnt.escaped, cnt.crossings, cnt.events, cnt.absorb,
                           cnt.scatter, cnt.mrw, cnt.late, cnt.parked, cnt.drained};
        const int slot[10] = {ST_KILLED, ST_ESCAPED, ST_CROSSINGS, ST_EVENTS, ST_ABSORB, ST_SCATTER,
                              ST_MRW, ST_LATE, ST_PARKED, ST_DRAINED};
#pragma unroll
        for (int i = 0; i < 10; ++i) {
            long long s = warp_sum(v[i]);
            if (lane == 0 && s) atomicAdd((unsigned long long*)(P.stats + slot[i]), (unsigned long long)s);
        }
    }
    int mx = cnt.maxev;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
    long long pk = warp_sum(cnt.parked);
    const long long le = warp_sum(cnt.events), lc = warp_sum(cnt.crossings),
                    ld = warp_sum(cnt.absorb + cnt.mrw);
    if (lane == 0) {
        int64_t* L = P.stats + MC_LSTAT + MC_LSTRIDE * P.lslot;
        atomicMax((unsigned long long*)(L + 1), (unsigned long long)globaltimer());
        atomicMax((unsigned long long*)(L + 2), (unsigned long long)mx);
        if (pk) atomicAdd((unsigned long long*)(L + 3), (unsigned long long)pk);
        if (le) atomicAdd((unsigned long long*)(L + 4), (unsigned long long)le);
        if (lc) atomicAdd((unsigned long long*)(L + 5), (unsigned long long)lc);
        if (ld) atomicAdd((unsigned long long*)(L + 6), (unsigned long long)ld);
    }
}

// Fast path of the warp-per-packet walk for one dust species and the double-single
// geometry, written for the latency of one dependent chain: the cell's density, snapshot,
// q per deposit unit and walls are held in registers, every lane evaluates the geometry
// itself (straight-line code, no shuffles), and the random numbers, isotropic directions,
// scattering cosines and reemission wavelengths come from the lanes' precomputed values.
// It takes the same decisions in the same order as mc_step (safety-distance refresh, wall
// solve, interaction or crossing, MRW try and jump), so the result is identical; the rare
// cases (a packet inside the inner hole, an empty cell, the interaction cap) are left to
// mc_step before anything of the step is committed.
struct TailCell {
    int ir = -2, itv = -1, ip = -1, epoch = -1;
    int c;
    float rho, wq;
    float2 q;
};

__device__ __forceinline__ ds tail_wall(const McModel& M, const WallsCell& W, const PktS& p,
                                        int& wall) {
    return M.np > 1 ? next_wall_ds_n<6>(M, W, p, wall) : next_wall_ds_n<4>(M, W, p, wall);
}

// Runs steps of packet p until one must go to mc_step (returns 0), the budget of steps is
// spent (1) or the packet has left the grid or was killed (2).  steps counts the steps taken.
__device__ __forceinline__ int tail_fast_run(PktS& p, const McParams& P, const McModel& M,
                                             const DustTabs& T, Cnt& cnt, WarpPol& pol,
                                             TailCell& tc, int budget, int& steps) {
    const int nl = P.nl;
    const uint32_t k0 = P.key0, k1 = P.key1;
    const int64_t base = M.cell_off;
    const int lane = pol.lane;
    for (steps = 0; steps < budget; ++steps) {
        if (p.ir < 0) return 0;
        if (p.ir != tc.ir || p.itv != tc.itv || p.ip != tc.ip || p.epoch != tc.epoch) {
            tc.c = cell_of_s(M, p);
            tc.ir = p.ir; tc.itv = p.itv; tc.ip = p.ip; tc.epoch = p.epoch;
            tc.rho = __ldg(P.rho + base + tc.c);
            tc.wq = __ldg(P.wq + base + tc.c);
            tc.q = P.q[(int64_t)p.epoch * P.qstride + base + tc.c];
        }
        const WallsCell& W = pol.cell_walls(M, P.fpool, p);
        const int c = tc.c;
        const float rh = tc.rho;
        float alpha = 0.0f;
        alpha = alpha + rh * T.kext[p.lam];
        if (!(alpha > 0.0f)) return 0;
        if (p.nevents + 1 >= P.max_inter) return 0;
        // a walk resumed within its epoch parks at late_after: mc_step takes that step
        if (P.phase == 0 && P.late_after > 0 && p.nevents + 1 >= P.late_after) return 0;
        const float sef = p.tau / alpha;
        if (!(sef < p.dsafe) && !p.fresh) {
            const float D = wall_distance_ds(M, W, p);
            p.dsafe = 0.999999f * D;
            p.dmax = mc_dmax_of(D);
            p.fresh = 1;
        }
        const bool full = !(sef < p.dsafe);
        ds se = ds{sef, 0.0f};
        if (full) {
            int wall = W_NONE;
            const ds sw = tail_wall(M, W, p, wall);
            const float tcell = alpha * sw.h;
            if (!(tcell > p.tau)) {
                // crossing into the next cell
                p.x = ds_move2(p.x, sw, p.kx);
                p.y = ds_move2(p.y, sw, p.ky);
                p.z = ds_move2(p.z, sw, p.kz);
                p.tau = p.tau - tcell;
                p.dsafe = 0.0f;
                p.dmax = MC_DMAX_UNKNOWN;
                p.fresh = 1;
                p.ncross += 1;
                cnt.crossings += 1;
                p.cell_events = 0;
                switch (wall) {
                    case W_ROUT:
                        p.ir += 1;
                        p.last_wall = W_RIN;
                        if (p.ir >= M.nr) {
                            cnt.escaped += 1;
                            if (P.escape && lane == 0)
                                atomicAdd((unsigned long long*)(P.escape + (int64_t)p.m * nl + p.lam), 1ull);
                            return 2;
                        }
                        break;
                    case W_RIN: p.ir -= 1; p.last_wall = W_ROUT; break;
                    case W_TLO: p.itv -= 1; p.last_wall = W_THI; break;
                    case W_THI: p.itv += 1; p.last_wall = W_TLO; break;
                    case W_PLO: p.ip = (p.ip == 0) ? M.np - 1 : p.ip - 1; p.last_wall = W_PHI; break;
                    case W_PHI: p.ip = (p.ip == M.np - 1) ? 0 : p.ip + 1; p.last_wall = W_PLO; break;
                    default: cnt.killed += 1; return 2;
                }
                if (p.ncross > 100000000) {
                    cnt.killed += 1;
                    return 2;
                }
                continue;
            }
            se = ds{p.tau / alpha, 0.0f};
            if (se.h > sw.h) se = sw;
        }
        // the interaction
        p.x = ds_move2(p.x, se, p.kx);
        p.y = ds_move2(p.y, se, p.ky);
        p.z = ds_move2(p.z, se, p.kz);
        p.dsafe = full ? 0.0f : p.dsafe - sef;
        p.fresh = 0;
        p.last_wall = W_NONE;
        const uint32_t n = (uint32_t)p.nevents;
        p.cell_events += 1;
        p.nevents += 1;
        cnt.events += 1;
        const bool late = P.late_after > 0 && p.nevents > P.late_after;
        int64_t* dep = late ? P.Elate : P.E;
        const EvR ev = pol.ev(p.rng, n, k0, k1);
        p.dmax = mc_dmax_after(p.dmax, se.h);
        bool did_mrw = false;
        const bool cond = P.mrw && (p.cell_events >= P.mrw_trigger ||
                                    (P.mrw_eager_after > 0 && p.nevents > P.mrw_eager_after));
        bool tried = false;
        float Dw = 0.0f;
        float aR = 0.0f;
        if (cond && 0.999f * p.dmax * alpha >= P.mrw_tauthres) {
            if (pol.cached(p.m, c, p.epoch, pol.own_ver(), 0)) {
                aR = pol.cached_value(0);
            } else {
                float qm = tc.q.x + 0.5f * tc.q.y;
                qm = qm + pol.own_q(c, tc.wq);
                aR = aR + rh * row_interp(pol, T, T.kR, qm, 0);
                pol.remember(p.m, c, p.epoch, pol.own_ver(), 0, aR);
            }
            tried = 0.999f * p.dmax * aR >= P.mrw_gamma;
        }
        if (tried) {
            Dw = wall_distance_ds(M, W, p);
            const float R0f = 0.999f * Dw;
            if (R0f * aR >= P.mrw_gamma && R0f * alpha >= P.mrw_tauthres) {
                did_mrw = true;
                const MrwR mb = pol.mrwd(p.rng, n, k0, k1);
                const SecR sb = pol.second(p.rng, n, k0, k1);
                float f = mb.uy * (float)(MC_NMRW - 1);
                int i = (int)f;
                if (i > MC_NMRW - 2) i = MC_NMRW - 2;
                float w = f - (float)i;
                float yv = T.mrw[i] + w * (T.mrw[i + 1] - T.mrw[i]);
                float ell = 3.0f * aR * R0f * R0f * yv;
                float kp;
                if (pol.cached(p.m, c, p.epoch, pol.own_ver(), 1)) {
                    kp = pol.cached_value(1);
                } else {
                    float qm = tc.q.x + 0.5f * tc.q.y;
                    qm = qm + pol.own_q(c, tc.wq);
                    kp = rh * row_interp(pol, T, T.kP, qm, 0);
                    pol.remember(p.m, c, p.epoch, pol.own_ver(), 1, kp);
                }
                float units_f = kp * ell * 1048576.0f + 0.5f;
                if (units_f > 9.0e18f) units_f = 9.0e18f;
                long long units = (long long)units_f;
                if (units > 0) {
                    if (lane == 0)
                        atomicAdd((unsigned long long*)(dep + base + c), (unsigned long long)units);
                    pol.own_add(c, units);
                }
                float dx, dy, dz;
                {
                    float mu = mb.jmu;
                    float st = sqrtf(fmaxf(0.0f, 1.0f - mu * mu));
                    dx = st * mb.jcs; dy = st * mb.jsn; dz = mu;
                }
                p.x = ds_move(p.x, R0f, dx);
                p.y = ds_move(p.y, R0f, dy);
                p.z = ds_move(p.z, R0f, dz);
                {
                    float mu = sqrtf(ev.umu);
                    float kx = dx, ky = dy, kz = dz;
                    mc_rotate(kx, ky, kz, mu, ev.cs, ev.sn);
                    p.kx = kx; p.ky = ky; p.kz = kz;
                }
                p.lam = reemit_lambda(pol, T, nl, tc.q, 0, sb.uq, sb.urow, sb.ucdf,
                                      pol.own_q(c, tc.wq));
                p.tau = ev.tn;
                p.cell_events = 0;
                cnt.mrw += 1;
            }
        }
        if (!did_mrw) {
            float asca = 0.0f;
            asca = asca + rh * T.ksca[p.lam];
            if (ev.ua * alpha < asca) {
                const float mu = pol.hg(n, T.g[p.lam], ev.umu);
                mc_rotate(p.kx, p.ky, p.kz, mu, ev.cs, ev.sn);
                cnt.scatter += 1;
            } else {
                const SecR sb = pol.second(p.rng, n, k0, k1);
                if (lane == 0) atomicAdd((unsigned long long*)(dep + base + c), 1ull << MC_EUNIT_SHIFT);
                pol.own_add(c, 1ll << MC_EUNIT_SHIFT);
                p.lam = pol.template reemit<1>(T, nl, tc.q, 0, sb, pol.own_q(c, tc.wq), p.m, c,
                                               p.epoch, n);
                pol.iso_dir(n, ev, p.kx, p.ky, p.kz);
                cnt.absorb += 1;
            }
            p.tau = ev.tn;
        }
        if (did_mrw) Dw = wall_distance_ds(M, W, p);
        if (did_mrw || tried) {
            p.dsafe = 0.999999f * Dw;
            p.dmax = mc_dmax_of(Dw);
            p.fresh = 1;
        }
        if (late) cnt.late += 1;
    }
    return 1;
}

// Per-warp shared staging of the batch's chains: field f of lane l at sb[f * 32 + l].  The
// chain loops read their inputs as broadcasts, so the loads are issued ahead of the chain.
enum { TB_A0, TB_A1, TB_A2, TB_A3, TB_A4, TB_A5, TB_LAM, TB_ALPHA, TB_XH, TB_XL, TB_YH, TB_YL,
       TB_ZH, TB_ZL, TB_DS, TB_DM, TB_FR, TB_NF };

// Interactions of a trapped packet, up to 32 at a time across the warp (lane l takes the
// batch's interaction l), with exactly the decisions and the arithmetic of tail_fast_run's
// steps in the same order.  Everything an interaction needs that does not depend on the
// packet's path so far is computed by its own lane: the random numbers, the isotropic
// direction, the Henyey-Greenstein cosine and the reemission wavelength.  What does
// depend on the path runs as short chains over the lanes' values:
//   1. the wavelength chain: interaction l absorbs or scatters at the wavelength left by
//      the last absorption before it; each lane has precomputed its reemission (at a guess
//      of the packet's own deposits in the cell, checked in step 6) and the extinction and
//      scattering coefficients there, so a link is a compare and a select;
//   2. the directions: after an absorption the lane's isotropic direction, after a
//      scattering the previous direction rotated (rounds over runs of scatterings);
//   3. the positions: the moves' products are formed per lane, the double-single sums
//      are chained in interaction order;
//   4. per lane at its position: the wall distance (safety-distance refresh and MRW try),
//      the Rosseland mean at the own deposits of that moment, and whether a try jumps;
//   5. the safety-distance / distance-bound chain with the MRW tries, which marks the
//      interactions that need a wall solve; those lanes solve their walls side by side;
//   6. the exact reemission check.
// The batch is committed up to the first interaction that leaves this scheme: a crossing
// (applied here from its lane's wall solve), an MRW jump, an interaction placed beyond the
// wall by rounding, or an empty cell (each left to one tail_fast_run step), or a reemission
// whose guess was wrong (committed with the exact wavelength, the rest recomputed).  The
// deposits of the committed absorptions go to the cell in one atomic (int64 sums do not
// depend on the order).  Returns like tail_fast_run.
__device__ __forceinline__ int tail_batch_run(PktS& p, const McParams& P, const McModel& M,
                                              const DustTabs& T, Cnt& cnt, WarpPol& pol,
                                              TailCell& tc, float* __restrict__ sb, int budget,
                                              int& steps) {
    const unsigned FULL = 0xffffffffu;
    const int nl = P.nl;
    const uint32_t k0 = P.key0, k1 = P.key1;
    const int64_t base = M.cell_off;
    const int l = pol.lane;
    steps = 0;
    // batch size: 16 after a crossing or an MRW jump (half the batches end within 10
    // interactions), 32 after a batch committed whole
    int bcap = 16;
    // after an MRW jump the next step is most often another jump (two thirds of the jumps
    // of a trapped walk follow one directly): such steps are taken one at a time
    bool after_jump = false;
    while (steps < budget) {
        // room for one more step after the batch, all interactions on the same side of
        // late_after, none reaching the interaction cap
        int B = budget - steps - 1;
        if (B > bcap) B = bcap;
        const long long ne = p.nevents;
        if (P.late_after > 0 && ne < P.late_after && ne + B > P.late_after)
            B = (int)(P.late_after - ne);
        // within an epoch the late_after-th interaction (which parks) is left to mc_step
        if (P.phase == 0 && P.late_after > 0 && ne + B >= P.late_after)
            B = (int)(P.late_after - ne - 1);
        bool ok = p.ir >= 0 && B >= 1 && ne + B < (long long)P.max_inter;
        if (ok) {
            if (p.ir != tc.ir || p.itv != tc.itv || p.ip != tc.ip || p.epoch != tc.epoch) {
                tc.c = cell_of_s(M, p);
                tc.ir = p.ir; tc.itv = p.itv; tc.ip = p.ip; tc.epoch = p.epoch;
                tc.rho = __ldg(P.rho + base + tc.c);
                tc.wq = __ldg(P.wq + base + tc.c);
                tc.q = P.q[(int64_t)p.epoch * P.qstride + base + tc.c];
            }
            float a0 = 0.0f;
            a0 = a0 + tc.rho * T.kext[p.lam];
            ok = a0 > 0.0f;
        }
        if (!ok || after_jump) {
            const long long mj = cnt.mrw;
            int s1 = 0;
            const int r = tail_fast_run(p, P, M, T, cnt, pol, tc, 1, s1);
            steps += s1;
            if (r != 1) return r;
            after_jump = cnt.mrw != mj;
            continue;
        }
        const WallsCell& W = pol.cell_walls(M, P.fpool, p);
        const int c = tc.c;
        const float rh = tc.rho, wq = tc.wq;
        const float2 q = tc.q;
        pol.refill_at(p.rng, (uint32_t)p.nevents, k0, k1);
        long long u0 = 0;
#pragma unroll
        for (int i = 0; i < MC_OWN; ++i)
            if (pol.own.sc[i] == c) u0 = pol.own.u[i];

        // reemission of this lane's interaction if it is an absorption, at a guess of the own
        // deposits (half of the earlier interactions absorbed)
        const long long ug = u0 + ((long long)(l / 2 + 1) << MC_EUNIT_SHIFT);
        float qg = q.x + pol.rs.uq * q.y;
        qg = qg + (float)ug * wq;
        int gj;
        float gw;
        mc_row_search(T.F, qg, gj, gw);
        const int grow = gj + ((pol.rs.urow < gw) ? 1 : 0);
        const int glam = mc_cdf_search(T.cdf + (size_t)grow * nl, nl, pol.rs.ucdf);
        float ga = 0.0f;
        ga = ga + rh * T.kext[glam];
        float gs = 0.0f;
        gs = gs + rh * T.ksca[glam];

        // 1. wavelength chain
        int cl = p.lam;
        float ca = 0.0f;
        ca = ca + rh * T.kext[cl];
        float cs = 0.0f;
        cs = cs + rh * T.ksca[cl];
        unsigned amask = 0u;
        sb[TB_A0 * 32 + l] = pol.re.ua;
        sb[TB_A1 * 32 + l] = __int_as_float(glam);
        sb[TB_A2 * 32 + l] = ga;
        sb[TB_A3 * 32 + l] = gs;
        __syncwarp();
#pragma unroll 4
        for (int j = 0; j < B; ++j) {
            const float ua = sb[TB_A0 * 32 + j];
            const int la = __float_as_int(sb[TB_A1 * 32 + j]);
            const float aa = sb[TB_A2 * 32 + j];
            const float sa = sb[TB_A3 * 32 + j];
            sb[TB_LAM * 32 + j] = __int_as_float(cl);   // every lane stores the same value
            sb[TB_ALPHA * 32 + j] = ca;
            const bool ab = !(ua * ca < cs);
            cl = ab ? la : cl;
            ca = ab ? aa : ca;
            cs = ab ? sa : cs;
            amask |= (unsigned)ab << j;
        }
        __syncwarp();
        // lanes beyond the batch keep the packet's wavelength (their values are never used)
        const int mylam = l < B ? __float_as_int(sb[TB_LAM * 32 + l]) : p.lam;
        const float mya = l < B ? sb[TB_ALPHA * 32 + l] : 1.0f;
        const bool myab = (amask >> l) & 1u;
        float tau = __shfl_up_sync(FULL, pol.re.tn, 1);
        if (l == 0) tau = p.tau;
        const float sef = tau / mya;

        // 2. directions: in (before the interaction) and out (after it)
        float kix = 0.0f, kiy = 0.0f, kiz = 0.0f, kox = 0.0f, koy = 0.0f, koz = 0.0f;
        bool kin = false, kout = false;
        {
            const float ux = __shfl_up_sync(FULL, pol.ikx, 1);
            const float uy = __shfl_up_sync(FULL, pol.iky, 1);
            const float uz = __shfl_up_sync(FULL, pol.ikz, 1);
            if (l == 0) { kix = p.kx; kiy = p.ky; kiz = p.kz; kin = true; }
            else if ((amask >> (l - 1)) & 1u) { kix = ux; kiy = uy; kiz = uz; kin = true; }
            if (myab) { kox = pol.ikx; koy = pol.iky; koz = pol.ikz; kout = true; }
        }
        const float mu = pol.gconst ? pol.hgmu : hg_mu(T.g[mylam], pol.re.umu);
        // round r settles the r-th scattering of a run: the lanes that know their incoming
        // direction rotate it, then pass their outgoing one on (B rounds at most)
        for (int it = 0; it <= 32; ++it) {
            if (kin && !kout) {
                kox = kix; koy = kiy; koz = kiz;
                mc_rotate(kox, koy, koz, mu, pol.re.cs, pol.re.sn);
                kout = true;
            }
            const float vx = __shfl_up_sync(FULL, kox, 1);
            const float vy = __shfl_up_sync(FULL, koy, 1);
            const float vz = __shfl_up_sync(FULL, koz, 1);
            const int pk = __shfl_up_sync(FULL, kout ? 1 : 0, 1);
            if (!kin && l > 0 && pk) { kix = vx; kiy = vy; kiz = vz; kin = true; }
            if (__ballot_sync(FULL, l < B && !(kin && kout)) == 0u) break;
        }

        // 3. positions before (b) and after (a) each lane's move
        {
            const ds mx = ds_prod(sef, kix), my = ds_prod(sef, kiy), mz = ds_prod(sef, kiz);
            sb[TB_A0 * 32 + l] = mx.h; sb[TB_A1 * 32 + l] = mx.l;
            sb[TB_A2 * 32 + l] = my.h; sb[TB_A3 * 32 + l] = my.l;
            sb[TB_A4 * 32 + l] = mz.h; sb[TB_A5 * 32 + l] = mz.l;
        }
        __syncwarp();
        ds X = p.x, Y = p.y, Z = p.z;
#pragma unroll 4
        for (int j = 0; j < B; ++j) {
            sb[TB_XH * 32 + j] = X.h; sb[TB_XL * 32 + j] = X.l;
            sb[TB_YH * 32 + j] = Y.h; sb[TB_YL * 32 + j] = Y.l;
            sb[TB_ZH * 32 + j] = Z.h; sb[TB_ZL * 32 + j] = Z.l;
            X = ds_add(X, ds{sb[TB_A0 * 32 + j], sb[TB_A1 * 32 + j]});
            Y = ds_add(Y, ds{sb[TB_A2 * 32 + j], sb[TB_A3 * 32 + j]});
            Z = ds_add(Z, ds{sb[TB_A4 * 32 + j], sb[TB_A5 * 32 + j]});
        }
        __syncwarp();
        ds bx = p.x, by = p.y, bz = p.z, ax = X, ay = Y, az = Z;
        if (l < B) {
            bx = ds{sb[TB_XH * 32 + l], sb[TB_XL * 32 + l]};
            by = ds{sb[TB_YH * 32 + l], sb[TB_YL * 32 + l]};
            bz = ds{sb[TB_ZH * 32 + l], sb[TB_ZL * 32 + l]};
        }
        if (l < B - 1) {
            ax = ds{sb[TB_XH * 32 + l + 1], sb[TB_XL * 32 + l + 1]};
            ay = ds{sb[TB_YH * 32 + l + 1], sb[TB_YL * 32 + l + 1]};
            az = ds{sb[TB_ZH * 32 + l + 1], sb[TB_ZL * 32 + l + 1]};
        }

        // 4. wall distances, Rosseland means and jumps per lane
        PktS pq = p;
        pq.x = ax; pq.y = ay; pq.z = az;
        const float Dpost = wall_distance_ds(M, W, pq);
        float Dpre = __shfl_up_sync(FULL, Dpost, 1);
        {
            const float s0 = __shfl_sync(FULL, sef, 0);
            if (!(s0 < p.dsafe) && !p.fresh) {
                const float D0 = wall_distance_ds(M, W, p);
                if (l == 0) Dpre = D0;
            }
        }
        const unsigned below = amask & ((1u << l) - 1u);
        const long long ut = u0 + ((long long)__popc(below) << MC_EUNIT_SHIFT);
        float qm = q.x + 0.5f * q.y;
        qm = qm + (ut != 0 ? (float)ut * wq : 0.0f);
        int rj;
        float rw;
        mc_row_search(T.F, qm, rj, rw);
        float aR = 0.0f;
        aR = aR + rh * (T.kR[rj] + rw * (T.kR[rj + 1] - T.kR[rj]));
        const float R0f = 0.999f * Dpost;
        const bool jmp = R0f * aR >= P.mrw_gamma && R0f * mya >= P.mrw_tauthres;
        const long long ce = (long long)p.cell_events + l + 1, nv = ne + l + 1;
        const bool cond = P.mrw && (ce >= P.mrw_trigger ||
                                    (P.mrw_eager_after > 0 && nv > P.mrw_eager_after));
        const unsigned cmask = __ballot_sync(FULL, cond);
        const unsigned jmask = __ballot_sync(FULL, jmp);

        // 5. safety distance, distance bound and MRW tries
        float dsafe = p.dsafe, dmax = p.dmax;
        int fresh = p.fresh;
        unsigned fmask = 0u;
        int L = B;
        __syncwarp();
        sb[TB_A0 * 32 + l] = sef;
        sb[TB_A1 * 32 + l] = Dpre;
        sb[TB_A2 * 32 + l] = Dpost;
        sb[TB_A3 * 32 + l] = aR;
        __syncwarp();
#pragma unroll 4
        for (int j = 0; j < B; ++j) {
            const float s = sb[TB_A0 * 32 + j];
            const float dp = sb[TB_A1 * 32 + j];
            const float dq = sb[TB_A2 * 32 + j];
            const float a = sb[TB_ALPHA * 32 + j];
            const float r = sb[TB_A3 * 32 + j];
            // selects rather than branches: the same values, a shorter dependent chain
            const bool rf = !(s < dsafe) && !fresh;
            dsafe = rf ? 0.999999f * dp : dsafe;
            dmax = rf ? mc_dmax_of(dp) : dmax;
            const bool full = !(s < dsafe);
            dsafe = full ? 0.0f : dsafe - s;
            dmax = mc_dmax_after(dmax, s);
            const bool c1 = ((cmask >> j) & 1u) && 0.999f * dmax * a >= P.mrw_tauthres;
            const bool tried = c1 && 0.999f * dmax * r >= P.mrw_gamma;
            if (tried && ((jmask >> j) & 1u)) { L = j; break; }
            dsafe = tried ? 0.999999f * dq : dsafe;
            dmax = tried ? mc_dmax_of(dq) : dmax;
            fresh = tried ? 1 : 0;
            fmask |= (unsigned)full << j;
            sb[TB_DS * 32 + j] = dsafe;
            sb[TB_DM * 32 + j] = dmax;
            sb[TB_FR * 32 + j] = __int_as_float(fresh);
        }
        __syncwarp();
        const bool jumped = L < B;

        // wall solves of the interactions whose safety distance does not suffice
        bool cross = false, edge = false;
        ds swd = ds{0.0f, 0.0f};
        int wall = W_NONE;
        float tcell = 0.0f;
        if (((fmask >> l) & 1u) && l < L) {
            PktS pb = p;
            pb.x = bx; pb.y = by; pb.z = bz;
            pb.kx = kix; pb.ky = kiy; pb.kz = kiz;
            if (l > 0) pb.last_wall = W_NONE;
            swd = tail_wall(M, W, pb, wall);
            tcell = mya * swd.h;
            if (!(tcell > tau)) cross = true;
            else if (tau / mya > swd.h) edge = true;
        }

        // 6. exact reemission of the absorptions (own deposits known now)
        int lamx = glam;
        bool badg = false;
        if (myab && l < L) {
            const long long uo = u0 + ((long long)(__popc(below) + 1) << MC_EUNIT_SHIFT);
            float qq = q.x + pol.rs.uq * q.y;
            qq = qq + (float)uo * wq;
            int j2;
            float w2;
            mc_row_search(T.F, qq, j2, w2);
            const int row2 = j2 + ((pol.rs.urow < w2) ? 1 : 0);
            if (row2 != grow) {
                lamx = mc_cdf_search(T.cdf + (size_t)row2 * nl, nl, pol.rs.ucdf);
                badg = lamx != glam;
            }
        }

        // commit: the first lane that leaves the scheme decides
        int act = 0;           // 0 continue, 1 one tail_fast_run step, 2 crossing of lane Lc
        int Lc = L;
        if (jumped) act = 1;
        const unsigned abad = __ballot_sync(FULL, !(mya > 0.0f) && l < B);
        if (abad) {
            const int a = __ffs(abad) - 1;
            if (a < Lc) { Lc = a; act = 1; }
        }
        const unsigned cb = __ballot_sync(FULL, cross || edge);
        if (cb) {
            const int f = __ffs(cb) - 1;
            if (f < Lc) { Lc = f; act = ((__ballot_sync(FULL, cross) >> f) & 1u) ? 2 : 1; }
        }
        const unsigned gb = __ballot_sync(FULL, badg);
        if (gb) {
            const int s = __ffs(gb) - 1;
            if (s + 1 <= Lc) { Lc = s + 1; act = 0; }
        }
        const bool late = P.late_after > 0 && ne + 1 > P.late_after;
        int64_t* dep = late ? P.Elate : P.E;
        if (Lc > 0) {
            const int t = Lc - 1;
            p.x = ds{__shfl_sync(FULL, ax.h, t), __shfl_sync(FULL, ax.l, t)};
            p.y = ds{__shfl_sync(FULL, ay.h, t), __shfl_sync(FULL, ay.l, t)};
            p.z = ds{__shfl_sync(FULL, az.h, t), __shfl_sync(FULL, az.l, t)};
            p.kx = __shfl_sync(FULL, kox, t);
            p.ky = __shfl_sync(FULL, koy, t);
            p.kz = __shfl_sync(FULL, koz, t);
            p.tau = __shfl_sync(FULL, pol.re.tn, t);
            const int lx = __shfl_sync(FULL, lamx, t);
            const int lm = __shfl_sync(FULL, mylam, t);
            p.lam = ((amask >> t) & 1u) ? lx : lm;
            p.dsafe = sb[TB_DS * 32 + t];
            p.dmax = sb[TB_DM * 32 + t];
            p.fresh = __float_as_int(sb[TB_FR * 32 + t]);
            p.cell_events += Lc;
            p.nevents += Lc;
            p.last_wall = W_NONE;
            const unsigned cm = (Lc == 32) ? FULL : ((1u << Lc) - 1u);
            const int A = __popc(amask & cm);
            cnt.events += Lc;
            cnt.absorb += A;
            cnt.scatter += Lc - A;
            if (late) cnt.late += Lc;
            if (A > 0) {
                const long long units = (long long)A << MC_EUNIT_SHIFT;
                if (l == 0) atomicAdd((unsigned long long*)(dep + base + c), (unsigned long long)units);
                pol.own_add(c, units);
            }
            steps += Lc;
        }
        if (act == 2) {
            // crossing of lane Lc: its wall solve at the committed position and direction
            const ds sw = ds{__shfl_sync(FULL, swd.h, Lc), __shfl_sync(FULL, swd.l, Lc)};
            const int wl = __shfl_sync(FULL, wall, Lc);
            const float tc2 = __shfl_sync(FULL, tcell, Lc);
            p.x = ds_move2(p.x, sw, p.kx);
            p.y = ds_move2(p.y, sw, p.ky);
            p.z = ds_move2(p.z, sw, p.kz);
            p.tau = p.tau - tc2;
            p.dsafe = 0.0f;
            p.dmax = MC_DMAX_UNKNOWN;
            p.fresh = 1;
            p.ncross += 1;
            cnt.crossings += 1;
            p.cell_events = 0;
            steps += 1;
            switch (wl) {
                case W_ROUT:
                    p.ir += 1;
                    p.last_wall = W_RIN;
                    if (p.ir >= M.nr) {
                        cnt.escaped += 1;
                        if (P.escape && l == 0)
                            atomicAdd((unsigned long long*)(P.escape + (int64_t)p.m * nl + p.lam), 1ull);
                        return 2;
                    }
                    break;
                case W_RIN: p.ir -= 1; p.last_wall = W_ROUT; break;
                case W_TLO: p.itv -= 1; p.last_wall = W_THI; break;
                case W_THI: p.itv += 1; p.last_wall = W_TLO; break;
                case W_PLO: p.ip = (p.ip == 0) ? M.np - 1 : p.ip - 1; p.last_wall = W_PHI; break;
                case W_PHI: p.ip = (p.ip == M.np - 1) ? 0 : p.ip + 1; p.last_wall = W_PLO; break;
                default: cnt.killed += 1; return 2;
            }
            if (p.ncross > 100000000) {
                cnt.killed += 1;
                return 2;
            }
        } else if (act == 1) {
            const long long mj = cnt.mrw;
            int s1 = 0;
            const int r = tail_fast_run(p, P, M, T, cnt, pol, tc, 1, s1);
            steps += s1;
            if (r != 1) return r;
            after_jump = cnt.mrw != mj;
        }
        bcap = (act == 0 && Lc == B) ? 32 : 16;
    }
    return 1;
}

// Continuation of parked packets: one packet per warp (WarpPol), taken from a queue.
template <int NS, class G>
__global__ void __launch_bounds__(256) mc_continue_kernel(McParams P) {
    extern __shared__ float4 smem4[];
    float* sm = reinterpret_cast<float*>(smem4);
    __shared__ int s_stop;
    __shared__ long long s_total;
    if (threadIdx.x == 0) {
        s_stop = (*(volatile long long*)(P.stats + ST_STOP) != 0) ? 1 : 0;
        long long c = (long long)*(volatile const unsigned long long*)P.park_in_count;
        s_total = c < P.park_in_cap ? c : P.park_in_cap;
        atomicMin((unsigned long long*)(P.stats + MC_LSTAT + MC_LSTRIDE * P.lslot), (unsigned long long)globaltimer());
    }
    const float* tab = P.fpool;
    if (P.use_smem) {
        const float4* src = reinterpret_cast<const float4*>(P.fpool);
        int n4 = (P.dust_floats + 3) / 4;
        for (int i = threadIdx.x; i < n4; i += blockDim.x) smem4[i] = __ldg(src + i);
        tab = sm;
    }
    __syncthreads();
    const long long total = s_total;
    DustTabs T;
    T.kabs = tab + P.o_kabs; T.ksca = tab + P.o_ksca; T.kext = tab + P.o_kext; T.g = tab + P.o_g;
    T.F = tab + P.o_F; T.cdf = tab + P.o_cdf; T.kP = tab + P.o_kP; T.kR = tab + P.o_kR;
    T.mrw = tab + P.o_mrw;
    const int lane = threadIdx.x & 31;
    Cnt cnt = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
    bool stop = s_stop != 0;
    unsigned iter = 0;
    while (!stop) {
        unsigned long long g = 0;
        if (lane == 0) g = atomicAdd(P.queue, 1ull);
        g = __shfl_sync(0xffffffffu, g, 0);
        if ((long long)g >= total) break;
        typename G::Pkt p;
        WarpPol pol(lane, P.g_const, P.g0);
        park_load<G>(p, P.park_in[g], pol);
        // the packet's model, held in registers for the whole walk
        const McModel Mw = P.models[p.m];
        int live = 1;
        if (lane == 0) live = model_live(P, p.m) ? 1 : 0;
        bool alive = __shfl_sync(0xffffffffu, live, 0) != 0;
        TailCell tc;
        float* tsb = nullptr;
        if constexpr (NS == 1 && std::is_same<G, GeoS>::value) {
            __shared__ float s_tail[(MC_TAIL_SMEM / 4)];
            tsb = s_tail + (threadIdx.x >> 5) * (TB_NF * 32);
        }
        while (alive) {
            if constexpr (NS == 1 && std::is_same<G, GeoS>::value) {
                // fast steps up to the next periodic check, then one general step
                int nfast = 0;
                const int r = tail_batch_run(p, P, Mw, T, cnt, pol, tc, tsb, 4096 - (int)(iter & 4095u),
                                            nfast);
                iter += (unsigned)nfast;
                if (r == 0) alive = mc_step<NS, WarpPol, G>(p, P, Mw, T, cnt, pol);
                else if (r == 2) alive = false;
                else iter -= 1u;   // the budget ran out: the check below comes next
            } else {
                alive = mc_step<NS, WarpPol, G>(p, P, Mw, T, cnt, pol);
            }
            if (((++iter) & 4095u) == 0u) {
                int st = 0;
                if (lane == 0) {
                    if (*(volatile long long*)(P.stats + ST_STOP) != 0) st = 1;
                    if (P.abort_flag && *P.abort_flag != 0) {
                        atomicCAS((unsigned long long*)(P.stats + ST_STATUS), 0ull, (unsigned long long)PDGPU_ABORTED);
                        st = 1;
                    }
                    if (P.deadline_ns > 0 &&
                        (long long)globaltimer() - P.stats[ST_T0] > P.deadline_ns) {
                        atomicCAS((unsigned long long*)(P.stats + ST_STATUS), 0ull, (unsigned long long)PDGPU_TIMEOUT);
                        st = 1;
                    }
                    if (st) atomicExch((unsigned long long*)(P.stats + ST_STOP), 1ull);
                    else if (!model_live(P, p.m)) st = 2;   // this packet's model stopped
                }
                st = __shfl_sync(0xffffffffu, st, 0);
                if (st == 2) break;
                if (st) { stop = true; break; }
            }
        }
        if (p.nevents > cnt.maxev) cnt.maxev = p.nevents;
    }
    // every lane followed the same packets: only lane 0 reports
    if (lane == 0) {
        const long long v[9] = {cnt.killed, cnt.escaped, cnt.crossings, cnt.events, cnt.absorb,
                                cnt.scatter, cnt.mrw, cnt.late, cnt.parked};
        const int slot[9] = {ST_KILLED, ST_ESCAPED, ST_CROSSINGS, ST_EVENTS, ST_ABSORB, ST_SCATTER,
                             ST_MRW, ST_LATE, ST_PARKED};
        if (P.count_stats)
            for (int i = 0; i < 9; ++i)
                if (v[i]) atomicAdd((unsigned long long*)(P.stats + slot[i]), (unsigned long long)v[i]);
        int64_t* L = P.stats + MC_LSTAT + MC_LSTRIDE * P.lslot;
        atomicMax((unsigned long long*)(L + 1), (unsigned long long)globaltimer());
        atomicMax((unsigned long long*)(L + 2), (unsigned long long)cnt.maxev);
        if (cnt.events) atomicAdd((unsigned long long*)(L + 4), (unsigned long long)cnt.events);
        if (cnt.crossings) atomicAdd((unsigned long long*)(L + 5), (unsigned long long)cnt.crossings);
        if (cnt.absorb + cnt.mrw)
            atomicAdd((unsigned long long*)(L + 6), (unsigned long long)(cnt.absorb + cnt.mrw));
    }
}

// Per-epoch cell preparation: (q_lo, q_span) in erg/s/g from the absorbed energy.
struct PrepParams {
    const McModel* models;
    const double* dpool;
    const float* rho;
    const int64_t* src;       // energy the span is computed from
    float2* q;
    float* wq;                // when set: (float)(q_unit / cell mass) per cell
    int64_t total;            // total cells over models and species
    int32_t nm, ns;
    int32_t first;            // 1: first epoch (q_lo = 0, q_span = src/m)
    int32_t epoch;            // epoch k >= 1 (ratio b_{k+1}/b_k)
};

__device__ __forceinline__ int model_of_cell(const McModel* models, int nm, int ns, int64_t i) {
    int lo = 0, hi = nm;
    while (hi - lo > 1) {
        int mid = (lo + hi) >> 1;
        if (models[mid].cell_off <= i) lo = mid; else hi = mid;
    }
    return lo;
}

__device__ __forceinline__ double cell_mass(const McModel& M, const double* dp, float rho, int c) {
    int ip = c % M.np;
    int t = c / M.np;
    int it = t % M.nt;
    int ir = t / M.nt;
    double V = dp[M.off_vr + ir] * dp[M.off_vt + it] * dp[M.off_vp + ip];
    return (double)rho * V;
}

__global__ void mc_prep_kernel(PrepParams P) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int m = model_of_cell(P.models, P.nm, P.ns, i);
        const McModel& M = P.models[m];
        int c = (int)((i - M.cell_off) % M.ncell);
        double mass = cell_mass(M, P.dpool, P.rho[i], c);
        if (P.wq) P.wq[i] = mass > 0.0 ? (float)(M.q_unit / mass) : 0.0f;
        float2 out = make_float2(0.0f, 0.0f);
        if (mass > 0.0) {
            double e = (double)P.src[i];
            if (P.first) {
                out.y = (float)(e * M.q_unit / mass);
            } else {
                double R = (double)M.bnd[P.epoch + 1] / (double)M.bnd[P.epoch];
                out.x = (float)(e * M.q_unit / mass);
                out.y = (float)(e * M.q_unit * (R - 1.0) / mass);
            }
        }
        P.q[i] = out;
    }
}

struct TempParams {
    const McModel* models;
    const double* dpool;
    const float* rho;
    const int64_t* E;
    const int64_t* Elate;
    double* T;
    int64_t total;
    int32_t nm, ns;
    int32_t off_tinv, off_finv;   // dpool offsets
};

__global__ void mc_temperature_kernel(TempParams P) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < P.total;
         i += (int64_t)gridDim.x * blockDim.x) {
        int m = model_of_cell(P.models, P.nm, P.ns, i);
        const McModel& M = P.models[m];
        int64_t rel = i - M.cell_off;
        int s = (int)(rel / M.ncell);
        int c = (int)(rel % M.ncell);
        double mass = cell_mass(M, P.dpool, P.rho[i], c);
        int64_t E = P.E[i] + P.Elate[i];
        double T = 0.0;
        if (E > 0 && mass > 0.0) {
            const double* F = P.dpool + P.off_finv + (size_t)s * MC_NINV;
            const double* TV = P.dpool + P.off_tinv;
            double q = (double)E * M.q_unit / mass;
            if (q <= F[0]) {
                T = TV[0] * sqrt(sqrt(q / F[0]));
            } else if (q >= F[MC_NINV - 1]) {
                T = TV[MC_NINV - 1];
            } else {
                int lo = 0, hi = MC_NINV - 1;
                while (hi - lo > 1) {
                    int mid = lo + (hi - lo) / 2;
                    if (F[mid] <= q) lo = mid; else hi = mid;
                }
                T = TV[lo] + (TV[lo + 1] - TV[lo]) * ((q - F[lo]) / (F[lo + 1] - F[lo]));
            }
        }
        P.T[i] = T;
    }
}

__global__ void mc_start_kernel(int64_t* stats) {
    stats[ST_T0] = (int64_t)globaltimer();
    for (int l = 0; l < MC_MAX_LAUNCH; ++l) stats[MC_LSTAT + MC_LSTRIDE * l] = 0x7fffffffffffffffLL;
}

__global__ void mc_finish_kernel(int64_t* stats, int64_t packets) {
    stats[ST_PACKETS] = packets;
}

}  // namespace

// ---------------------------------------------------------------------------------------
// Host side: tables, geometry, schedule.  The same formulas as the CPU oracle, evaluated in
// the same order, so both consume identical tables.
// ---------------------------------------------------------------------------------------
struct pdgpu_mc_plan {
    int nm, ns, nl, K, npilot;
    pdgpu_mc_options opt;
    std::vector<float> fpool;       // dust tables first (dust_floats), then star CDFs
    std::vector<double> dpool;      // walls per model, Tinv, Finv
    std::vector<McModel> models;
    std::vector<int64_t> cum;       // [K][nm+1]
    int dust_floats;
    int o_kabs, o_ksca, o_kext, o_g, o_F, o_cdf, o_kP, o_kR, o_mrw;
    int off_tinv, off_finv;
    int64_t total_cells, total_nphot;
    // workspace layout
    size_t ws_fpool, ws_dpool, ws_models, ws_cum, ws_E, ws_D, ws_q, ws_escape, ws_stats,
        ws_queue, ws_total, tables_bytes, ws_Elate, ws_park, ws_park2, ws_parkcnt, ws_wq,
        ws_mdl, ws_mstat;
    bool use_mdl;                   // per-model deadlines set (pdgpu_mc_plan_set_model_deadlines)
    bool g_const;                   // one wavelength-independent asymmetry g0 for every species
    float g0;
    int64_t park_cap;
    int nqueue;
    bool epoch_drain;   // the last walks of each epoch launch resume one per warp
    int nlaunch;        // launches of the last run
    int device, nsm, block, grid;
    bool smem_tables;
    size_t smem_bytes;
    void* uploaded_ws;
    cudaEvent_t ev[2 * MC_MAX_LAUNCH];   // launch timing (time_launches)
    bool ev_ready;
    int ev_used;
};

namespace {

double planck_nu(double nu, double T) {
    double x = MC_H_PLANCK * nu / (MC_K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double pre = 2.0 * MC_H_PLANCK * nu * nu * nu / (MC_C_LIGHT * MC_C_LIGHT);
    return pre / expm1(x);
}

double dplanck_dT(double nu, double T) {
    double x = MC_H_PLANCK * nu / (MC_K_BOLTZ * T);
    if (x > 700.0) return 0.0;
    double em1 = expm1(x);
    double pre = 2.0 * MC_H_PLANCK * nu * nu * nu / (MC_C_LIGHT * MC_C_LIGHT);
    double bb = pre / em1;
    return bb * (x * exp(x) / em1) / T;
}

double mrw_survival(double y) {
    if (y < 0.005) return 1.0;
    double s = 0.0;
    for (int n = 1; n < 100000; ++n) {
        double a = (double)n * (double)n * MC_PI * MC_PI * y;
        if (a > 80.0) break;
        double t = exp(-a);
        s += (n & 1) ? t : -t;
    }
    return 2.0 * s;
}

const std::vector<float>& mrw_table() {
    static std::vector<float> tab;
    static std::once_flag once;
    std::call_once(once, [] {
        tab.resize(MC_NMRW);
        for (int i = 0; i < MC_NMRW; ++i) {
            double xi = (double)i / (double)(MC_NMRW - 1);
            if (i == MC_NMRW - 1) { tab[i] = 0.0f; continue; }
            if (i == 0) xi = 1.0e-7;
            double lo = 0.0, hi = 10.0;
            for (int it = 0; it < 100; ++it) {
                double mid = 0.5 * (lo + hi);
                if (mrw_survival(mid) > xi) lo = mid; else hi = mid;
            }
            tab[i] = (float)(0.5 * (lo + hi));
        }
    });
    return tab;
}

pdgpu_status build_dust(pdgpu_mc_plan* P, const pdgpu_dust_desc* d, std::vector<double>& nu,
                        std::vector<double>& dnu) {
    int nl = d->nlam, ns = d->nspec;
    nu.resize(nl);
    dnu.resize(nl);
    for (int l = 0; l < nl; ++l) nu[l] = MC_C_LIGHT / (d->lam_um[l] * 1.0e-4);
    for (int l = 0; l < nl; ++l) {
        if (l == 0) dnu[l] = 0.5 * fabs(nu[0] - nu[1]);
        else if (l == nl - 1) dnu[l] = 0.5 * fabs(nu[nl - 2] - nu[nl - 1]);
        else dnu[l] = 0.5 * fabs(nu[l - 1] - nu[l + 1]);
    }
    std::vector<float>& f = P->fpool;
    auto take = [&](size_t n) {
        int off = (int)f.size();
        f.resize(f.size() + n, 0.0f);
        return off;
    };
    P->o_kabs = take((size_t)ns * nl);
    P->o_ksca = take((size_t)ns * nl);
    P->o_kext = take((size_t)ns * nl);
    P->o_g = take((size_t)ns * nl);
    for (int i = 0; i < ns * nl; ++i) {
        f[P->o_kabs + i] = (float)d->kabs[i];
        f[P->o_ksca + i] = (float)d->ksca[i];
        f[P->o_kext + i] = f[P->o_kabs + i] + f[P->o_ksca + i];
        f[P->o_g + i] = d->g ? (float)d->g[i] : 0.0f;
    }
    P->o_F = take((size_t)ns * MC_NROW);
    P->o_cdf = take((size_t)ns * MC_NROW * nl);
    P->o_kP = take((size_t)ns * MC_NROW);
    P->o_kR = take((size_t)ns * MC_NROW);
    std::vector<double> cumv(nl);
    for (int s = 0; s < ns; ++s) {
        const double* ka = d->kabs + (size_t)s * nl;
        const double* ks = d->ksca + (size_t)s * nl;
        for (int j = 0; j < MC_NROW; ++j) {
            double T = MC_TROW_LO * pow(MC_TROW_HI / MC_TROW_LO, (double)j / (double)(MC_NROW - 1));
            double sumF = 0.0, sumB = 0.0, sumD = 0.0, sumDk = 0.0, c = 0.0;
            for (int l = 0; l < nl; ++l) {
                double B = planck_nu(nu[l], T);
                double dB = dplanck_dT(nu[l], T);
                sumF += ka[l] * B * dnu[l];
                sumB += B * dnu[l];
                sumD += dB * dnu[l];
                double ke = ka[l] + ks[l];
                if (ke > 0.0) sumDk += dB / ke * dnu[l];
                c += ka[l] * dB * dnu[l];
                cumv[l] = c;
            }
            double Fj = 4.0 * MC_PI * sumF;
            f[P->o_F + s * MC_NROW + j] = (float)Fj;
            float* row = &f[P->o_cdf + ((size_t)s * MC_NROW + j) * nl];
            for (int l = 0; l < nl; ++l)
                row[l] = (c > 0.0) ? (float)(cumv[l] / c) : (float)((l + 1.0) / nl);
            row[nl - 1] = 1.0f;
            f[P->o_kP + s * MC_NROW + j] = (float)(sumB > 0.0 ? sumF / sumB : 0.0);
            f[P->o_kR + s * MC_NROW + j] = (float)(sumDk > 0.0 ? sumD / sumDk : 0.0);
        }
    }
    P->o_mrw = take(MC_NMRW);
    const std::vector<float>& mt = mrw_table();
    for (int i = 0; i < MC_NMRW; ++i) f[P->o_mrw + i] = mt[i];
    P->dust_floats = (int)f.size();
    P->g_const = true;
    P->g0 = f[P->o_g];
    for (int i = 1; i < ns * nl; ++i)
        if (f[P->o_g + i] != P->g0) P->g_const = false;
    // pad to 16 bytes so the stellar CDFs start aligned
    while (f.size() % 4) f.push_back(0.0f);
    return PDGPU_OK;
}

int pick_device_props(int& nsm) {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return -1;
    if (cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return -1;
    return dev;
}

}  // namespace

extern "C" {

int32_t pdgpu_abi_version(void) { return PDGPU_ABI_VERSION; }

const char* pdgpu_status_string(pdgpu_status s) {
    switch (s) {
        case PDGPU_OK: return "ok";
        case PDGPU_INVALID_ARG: return "invalid argument";
        case PDGPU_TIMEOUT: return "time limit reached";
        case PDGPU_ABORTED: return "aborted by the host";
        case PDGPU_PACKET_CAP: return "packets hit the interaction cap";
        case PDGPU_OVERFLOW: return "fixed-point overflow";
        case PDGPU_CUDA_ERROR: return "CUDA error";
        case PDGPU_NO_DEVICE: return "no usable CUDA device";
        case PDGPU_WORKSPACE: return "workspace missing, too small or not uploaded";
        case PDGPU_TOO_LARGE: return "run needs more than the library's static scratch";
        default: return "unknown status";
    }
}

pdgpu_status pdgpu_mc_plan_create(int32_t nmodels, const pdgpu_model_desc* models,
                                  const pdgpu_dust_desc* dust, const pdgpu_mc_options* options,
                                  pdgpu_mc_plan** out) {
    if (!out) return PDGPU_INVALID_ARG;
    *out = nullptr;
    if (nmodels < 1 || !models || !dust || !options) return PDGPU_INVALID_ARG;
    if (dust->nlam < 2 || dust->nspec < 1 || dust->nspec > MC_MAX_SPEC || !dust->lam_um ||
        !dust->kabs || !dust->ksca)
        return PDGPU_INVALID_ARG;
    for (int l = 1; l < dust->nlam; ++l)
        if (!(dust->lam_um[l] > dust->lam_um[l - 1])) return PDGPU_INVALID_ARG;
    for (int i = 0; i < dust->nspec * dust->nlam; ++i)
        if (!(dust->kabs[i] >= 0.0) || !(dust->ksca[i] >= 0.0) || !std::isfinite(dust->kabs[i]) ||
            !std::isfinite(dust->ksca[i]))
            return PDGPU_INVALID_ARG;
    pdgpu_mc_plan* P = new (std::nothrow) pdgpu_mc_plan();
    if (!P) return PDGPU_INVALID_ARG;
    P->nm = nmodels;
    P->ns = dust->nspec;
    P->nl = dust->nlam;
    P->opt = *options;
    P->K = options->nepoch < 1 ? 1 : std::min(options->nepoch, MC_MAX_EPOCH);
    P->npilot = std::max(0, options->npilot);
    P->K = std::min(P->K, MC_MAX_LAUNCH - 2);
    P->npilot = std::min(P->npilot, MC_MAX_LAUNCH - 2 - P->K);   // K + npilot + 2 launches
    // fewer epochs when a model has too few packets for the first epoch to be non-empty
    for (int m = 0; m < nmodels; ++m)
        while (P->K > 1 && (models[m].nphot >> (P->K - 1)) == 0) P->K--;
    std::vector<double> nu, dnu;
    build_dust(P, dust, nu, dnu);
    const int ns = P->ns, nl = P->nl;
    // temperature inversion tables
    P->off_tinv = (int)P->dpool.size();
    for (int j = 0; j < MC_NINV; ++j)
        P->dpool.push_back(MC_TINV_LO * pow(MC_TINV_HI / MC_TINV_LO, (double)j / (double)(MC_NINV - 1)));
    P->off_finv = (int)P->dpool.size();
    for (int s = 0; s < ns; ++s) {
        const double* ka = dust->kabs + (size_t)s * nl;
        for (int j = 0; j < MC_NINV; ++j) {
            double sumF = 0.0;
            for (int l = 0; l < nl; ++l) sumF += ka[l] * planck_nu(nu[l], P->dpool[P->off_tinv + j]) * dnu[l];
            P->dpool.push_back(4.0 * MC_PI * sumF);
        }
    }
    int64_t cell_off = 0;
    P->total_nphot = 0;
    for (int m = 0; m < nmodels; ++m) {
        const pdgpu_model_desc& d = models[m];
        McModel M;
        memset(&M, 0, sizeof(M));
        if (d.nstar < 1 || !d.star_radius_cm || !d.star_temperature || d.nphot < 1 ||
            d.nphot > 4000000000LL ||
            !append_geometry(d.nr, d.ntheta, d.nphi, d.r_edges_cm, d.theta_edges, d.phi_edges, M,
                             P->dpool, P->fpool)) {
            delete P;
            return PDGPU_INVALID_ARG;
        }
        M.cell_off = cell_off;
        M.model_id = m;
        M.nphot = d.nphot;
        // stellar spectrum
        std::vector<double> Lnu(nl, 0.0);
        for (int s = 0; s < d.nstar; ++s) {
            double R = d.star_radius_cm[s];
            if (!(R > 0.0) || !(d.star_temperature[s] > 0.0)) { delete P; return PDGPU_INVALID_ARG; }
            for (int l = 0; l < nl; ++l)
                Lnu[l] += 4.0 * MC_PI * R * R * MC_PI * planck_nu(nu[l], d.star_temperature[s]) * dnu[l];
        }
        double L = 0.0;
        for (int l = 0; l < nl; ++l) L += Lnu[l];
        if (!(L > 0.0)) { delete P; return PDGPU_INVALID_ARG; }
        M.lum = L;
        M.off_star = (int)P->fpool.size();
        double cum = 0.0;
        for (int l = 0; l < nl; ++l) {
            cum += Lnu[l];
            P->fpool.push_back((float)(cum / L));
        }
        P->fpool[M.off_star + nl - 1] = 1.0f;
        while (P->fpool.size() % 4) P->fpool.push_back(0.0f);
        double eps = L / (double)d.nphot;
        M.q_unit = eps / (double)((int64_t)1 << MC_EUNIT_SHIFT);
        // epochs: b_k = N >> (K - k) (K shared by all models, see below)
        const int K = P->K;
        for (int k = 0; k <= MC_MAX_EPOCH; ++k) M.bnd[k] = d.nphot;
        M.bnd[0] = 0;
        for (int k = 1; k <= K; ++k) M.bnd[k] = d.nphot >> (K - k);
        P->models.push_back(M);
        cell_off += (int64_t)ns * M.ncell;
        P->total_nphot += d.nphot;
    }
    P->total_cells = cell_off;
    // per-epoch prefix sums of packet counts over models
    P->cum.assign((size_t)P->K * (nmodels + 1), 0);
    for (int k = 0; k < P->K; ++k) {
        int64_t acc = 0;
        for (int m = 0; m < nmodels; ++m) {
            P->cum[(size_t)k * (nmodels + 1) + m] = acc;
            acc += P->models[m].bnd[k + 1] - P->models[m].bnd[k];
        }
        P->cum[(size_t)k * (nmodels + 1) + nmodels] = acc;
    }
    // device properties and launch shape
    int nsm = 0;
    P->device = pick_device_props(nsm);
    P->nsm = nsm > 0 ? nsm : 1;
    P->block = options->block_threads > 0 ? options->block_threads : 256;
    if (P->block > 256) P->block = 256;
    size_t dust_bytes = ((size_t)P->dust_floats + 3) / 4 * 16;
    size_t cum_bytes = (size_t)(nmodels + 1) * sizeof(int64_t);
    int smem_max = 0;
    if (P->device >= 0)
        cudaDeviceGetAttribute(&smem_max, cudaDevAttrMaxSharedMemoryPerBlockOptin, P->device);
    // per-thread own-deposit caches of the per-thread transport launches
    size_t own_bytes = (size_t)P->block * MC_OWN * (sizeof(int) + sizeof(long long)) +
                       (size_t)P->block * sizeof(int);
    // (the continuation kernel's static staging of batched walks comes on top)
    P->smem_tables = (dust_bytes + cum_bytes + own_bytes + MC_TAIL_SMEM + 64) <= (size_t)smem_max;
    P->smem_bytes = (P->smem_tables ? dust_bytes : 0) + cum_bytes + own_bytes + 16;
    // workspace layout
    size_t o = 0;
    auto place = [&](size_t bytes) {
        o = (o + 255) / 256 * 256;
        size_t at = o;
        o += bytes;
        return at;
    };
    P->ws_fpool = place(P->fpool.size() * sizeof(float));
    P->ws_dpool = place(P->dpool.size() * sizeof(double));
    P->ws_models = place(P->models.size() * sizeof(McModel));
    P->ws_cum = place(P->cum.size() * sizeof(int64_t));
    P->tables_bytes = (o + 255) / 256 * 256;
    P->ws_E = place((size_t)P->total_cells * sizeof(int64_t));
    P->ws_D = place((size_t)P->total_cells * sizeof(int64_t));
    P->ws_q = place((size_t)P->K * P->total_cells * sizeof(float2));
    P->ws_Elate = place((size_t)P->total_cells * sizeof(int64_t));
    P->ws_wq = place((size_t)P->total_cells * sizeof(float));
    // room for every packet that outlives late_after in heavy-tailed runs (about 1 in 100
    // in the densest disks); a packet that finds the list full finishes in its epoch launch
    P->park_cap = std::max<int64_t>(65536, P->total_nphot / 16);
    P->ws_park = place((size_t)P->park_cap * sizeof(ParkRec));
    P->ws_park2 = place((size_t)P->park_cap * sizeof(ParkRec));
    // [parked after late_after, drained for the warp-per-packet launch, in flight, spare]
    P->ws_parkcnt = place(4 * sizeof(unsigned long long));
    P->ws_escape = place((size_t)nmodels * nl * sizeof(int64_t));
    P->ws_stats = place(MC_NSTAT * sizeof(int64_t));
    P->ws_mdl = place((size_t)nmodels * sizeof(int64_t));
    P->ws_mstat = place((size_t)nmodels * sizeof(int32_t));
    P->use_mdl = false;
    // with draining, every pilot and epoch launch is followed by a warp-per-packet launch
    P->epoch_drain = P->opt.drain_below >= 0 && 2 * (P->K + P->npilot) + 2 <= MC_MAX_LAUNCH;
    P->nqueue = (P->epoch_drain ? 2 : 1) * (P->K + P->npilot) + 2;   // one work counter per launch
    P->ws_queue = place((size_t)P->nqueue * sizeof(unsigned long long));
    P->ws_total = (o + 255) / 256 * 256;
    P->uploaded_ws = nullptr;
    P->ev_ready = false;
    P->ev_used = 0;
    if (options->time_launches && P->device >= 0) {
        P->ev_ready = true;
        for (int i = 0; i < 2 * MC_MAX_LAUNCH; ++i)
            if (cudaEventCreate(&P->ev[i]) != cudaSuccess) P->ev_ready = false;
    }
    *out = P;
    return PDGPU_OK;
}

void pdgpu_mc_plan_destroy(pdgpu_mc_plan* plan) {
    if (!plan) return;
    if (plan->ev_ready)
        for (int i = 0; i < 2 * MC_MAX_LAUNCH; ++i) cudaEventDestroy(plan->ev[i]);
    delete plan;
}

int32_t pdgpu_mc_plan_launch_ms(pdgpu_mc_plan* P, float* ms, int32_t capacity) {
    if (!P || !ms || !P->ev_ready) return 0;
    int n = std::min(P->ev_used, (int)capacity);
    for (int i = 0; i < n; ++i) {
        float t = 0.0f;
        if (cudaEventSynchronize(P->ev[2 * i + 1]) != cudaSuccess ||
            cudaEventElapsedTime(&t, P->ev[2 * i], P->ev[2 * i + 1]) != cudaSuccess)
            t = -1.0f;
        ms[i] = t;
    }
    return n;
}

pdgpu_status pdgpu_mc_plan_set_deadline(pdgpu_mc_plan* P, int64_t deadline_ns) {
    if (!P || deadline_ns < 0) return PDGPU_INVALID_ARG;
    P->opt.deadline_ns = deadline_ns;
    return PDGPU_OK;
}

pdgpu_status pdgpu_mc_plan_set_model_deadlines(pdgpu_mc_plan* P, const int64_t* deadline_ns,
                                               void* stream) {
    if (!P) return PDGPU_INVALID_ARG;
    if (!P->uploaded_ws) return PDGPU_WORKSPACE;
    std::vector<int64_t> d((size_t)P->nm, 0);
    bool any = false;
    if (deadline_ns)
        for (int m = 0; m < P->nm; ++m) {
            if (deadline_ns[m] < 0) return PDGPU_INVALID_ARG;
            d[m] = deadline_ns[m];
            any = any || d[m] > 0;
        }
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync((char*)P->uploaded_ws + P->ws_mdl, d.data(), d.size() * sizeof(int64_t),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    P->use_mdl = any;
    return PDGPU_OK;
}

pdgpu_status pdgpu_mc_plan_model_status(pdgpu_mc_plan* P, const void* ws, void* stream,
                                        int32_t* status) {
    if (!P || !ws || !status) return PDGPU_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(status, (const char*)ws + P->ws_mstat, (size_t)P->nm * sizeof(int32_t),
                        cudaMemcpyDeviceToHost, st) != cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    return PDGPU_OK;
}

pdgpu_status pdgpu_mc_plan_layout(const pdgpu_mc_plan* P, pdgpu_mc_layout* L) {
    if (!P || !L) return PDGPU_INVALID_ARG;
    L->tables_bytes = P->tables_bytes;
    L->energy_offset = P->ws_E;
    L->late_offset = P->ws_Elate;
    L->escape_offset = P->ws_escape;
    L->stats_offset = P->ws_stats;
    L->total_bytes = P->ws_total;
    L->total_cells = P->total_cells;
    L->nmodels = P->nm;
    L->nspec = P->ns;
    L->nlam = P->nl;
    L->smem_tables = P->smem_tables ? 1 : 0;
    return PDGPU_OK;
}

pdgpu_status pdgpu_mc_plan_upload(pdgpu_mc_plan* P, void* ws, size_t bytes, void* stream) {
    if (!P) return PDGPU_INVALID_ARG;
    if (!ws || bytes < P->ws_total) return PDGPU_WORKSPACE;
    if (P->device < 0) return PDGPU_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    char* w = (char*)ws;
    if (cudaMemcpyAsync(w + P->ws_fpool, P->fpool.data(), P->fpool.size() * sizeof(float),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(w + P->ws_dpool, P->dpool.data(), P->dpool.size() * sizeof(double),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(w + P->ws_models, P->models.data(), P->models.size() * sizeof(McModel),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemcpyAsync(w + P->ws_cum, P->cum.data(), P->cum.size() * sizeof(int64_t),
                        cudaMemcpyHostToDevice, st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_mdl, 0, (size_t)P->nm * sizeof(int64_t), st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    P->use_mdl = false;
    // pageable sources: make sure the copies finished before the host vectors can change
    if (cudaStreamSynchronize(st) != cudaSuccess) return PDGPU_CUDA_ERROR;
    P->uploaded_ws = ws;
    return PDGPU_OK;
}

// phase 0: epoch launch over the epoch's packets; phase 1: continuation of parked packets
static pdgpu_status launch_transport(pdgpu_mc_plan* P, char* w, const float* rho, int64_t* target,
                                     int epoch, uint32_t tag, int lslot, bool final_pass,
                                     int phase, cudaStream_t st) {
    McParams prm;
    memset(&prm, 0, sizeof(prm));
    prm.fpool = (const float*)(w + P->ws_fpool);
    prm.dpool = (const double*)(w + P->ws_dpool);
    prm.models = (const McModel*)(w + P->ws_models);
    prm.cum = (const int64_t*)(w + P->ws_cum) + (size_t)epoch * (P->nm + 1);
    prm.rho = rho;
    prm.wq = (const float*)(w + P->ws_wq);
    prm.E = target;
    prm.Elate = final_pass ? (int64_t*)(w + P->ws_Elate) : target;
    prm.q = (const float2*)(w + P->ws_q);
    prm.qstride = P->total_cells;
    prm.late_after = P->opt.late_after > 0 ? P->opt.late_after : 0;
    unsigned long long* counts = (unsigned long long*)(w + P->ws_parkcnt);
    ParkRec* listA = (ParkRec*)(w + P->ws_park);
    ParkRec* listB = (ParkRec*)(w + P->ws_park2);
    // phase 3: the packets drained from an epoch launch (list B), resumed one per warp with
    // the epoch's semantics (phase 0: deposits to the epoch's target, parking in list A)
    const int sem = phase == 3 ? 0 : phase;
    prm.park_out = (phase == 0 || phase == 3) ? listA : listB;
    prm.park_out_count = (phase == 0 || phase == 3) ? counts : counts + 1;
    prm.park_out_cap = P->park_cap;
    prm.park_in = phase == 1 ? listA : listB;
    prm.park_in_count = phase == 1 ? counts : counts + 1;
    prm.park_in_cap = P->park_cap;
    prm.drain_out = listB;
    prm.drain_out_count = counts + 1;
    prm.inflight = counts + 2;
    prm.drain_below = 0;
    prm.pilot = final_pass ? 0 : 1;
    prm.phase = sem;
    prm.lslot = lslot;
    prm.escape = final_pass ? (int64_t*)(w + P->ws_escape) : nullptr;
    prm.stats = (int64_t*)(w + P->ws_stats);
    prm.queue = (unsigned long long*)(w + P->ws_queue) + lslot;
    prm.abort_flag = P->opt.abort_flag;
    prm.deadline_ns = P->opt.deadline_ns;
    prm.mdeadline = (const int64_t*)(w + P->ws_mdl);
    prm.mstat = (int32_t*)(w + P->ws_mstat);
    prm.use_mdl = P->use_mdl ? 1 : 0;
    prm.total = phase == 0 ? P->cum[(size_t)epoch * (P->nm + 1) + P->nm] : P->park_cap;
    if ((phase == 1 || (phase == 0 && P->epoch_drain)) && P->opt.drain_below >= 0) {
        int64_t d = P->opt.drain_below;
        if (d == 0) {
            // as many packets as the warp-per-packet launch keeps running at once
            void (*ck)(McParams) = nullptr;
            switch (P->ns) {
                case 1: ck = P->opt.fp64_walls ? mc_continue_kernel<1, GeoD> : mc_continue_kernel<1, GeoS>; break;
                case 2: ck = P->opt.fp64_walls ? mc_continue_kernel<2, GeoD> : mc_continue_kernel<2, GeoS>; break;
                case 3: ck = P->opt.fp64_walls ? mc_continue_kernel<3, GeoD> : mc_continue_kernel<3, GeoS>; break;
                default: ck = P->opt.fp64_walls ? mc_continue_kernel<4, GeoD> : mc_continue_kernel<4, GeoS>; break;
            }
            int per = 0;
            if (cudaFuncSetAttribute(ck, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P->smem_bytes) != cudaSuccess ||
                cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, ck, P->block, P->smem_bytes) != cudaSuccess)
                return PDGPU_CUDA_ERROR;
            d = (int64_t)std::max(per, 1) * P->nsm * (P->block / 32);
        }
        prm.drain_below = d;
    }
    prm.nm = P->nm;
    prm.ns = P->ns;
    prm.nl = P->nl;
    prm.epoch = epoch;
    prm.tag = tag;
    prm.key0 = (uint32_t)(P->opt.seed & 0xffffffffu);
    prm.key1 = (uint32_t)(P->opt.seed >> 32);
    prm.mrw = P->opt.mrw;
    prm.mrw_trigger = P->opt.mrw_count_trigger;
    prm.mrw_eager_after = (int32_t)std::min<int64_t>(std::max<int64_t>(P->opt.mrw_eager_after, 0),
                                                     2000000000LL);
    prm.mrw_gamma = P->opt.mrw_gamma;
    prm.mrw_tauthres = P->opt.mrw_tauthres;
    int64_t mi = P->opt.max_interactions <= 0 ? 2000000000LL : P->opt.max_interactions;
    prm.max_inter = (int32_t)std::min<int64_t>(mi, 2000000000LL);
    prm.dust_floats = P->dust_floats;
    prm.use_smem = P->smem_tables ? 1 : 0;
    prm.o_kabs = P->o_kabs; prm.o_ksca = P->o_ksca; prm.o_kext = P->o_kext; prm.o_g = P->o_g;
    prm.o_F = P->o_F; prm.o_cdf = P->o_cdf; prm.o_kP = P->o_kP; prm.o_kR = P->o_kR;
    prm.o_mrw = P->o_mrw;
    prm.count_stats = final_pass ? 1 : 0;
    prm.g_const = P->g_const ? 1 : 0;
    prm.g0 = P->g0;
    if (prm.total <= 0) return PDGPU_OK;
    void (*kern)(McParams) = nullptr;
    const bool f64 = P->opt.fp64_walls != 0;
    if (phase <= 1) {
        switch (P->ns) {
            case 1: kern = f64 ? mc_transport_kernel<1, GeoD> : mc_transport_kernel<1, GeoS>; break;
            case 2: kern = f64 ? mc_transport_kernel<2, GeoD> : mc_transport_kernel<2, GeoS>; break;
            case 3: kern = f64 ? mc_transport_kernel<3, GeoD> : mc_transport_kernel<3, GeoS>; break;
            default: kern = f64 ? mc_transport_kernel<4, GeoD> : mc_transport_kernel<4, GeoS>; break;
        }
    } else {
        switch (P->ns) {
            case 1: kern = f64 ? mc_continue_kernel<1, GeoD> : mc_continue_kernel<1, GeoS>; break;
            case 2: kern = f64 ? mc_continue_kernel<2, GeoD> : mc_continue_kernel<2, GeoS>; break;
            case 3: kern = f64 ? mc_continue_kernel<3, GeoD> : mc_continue_kernel<3, GeoS>; break;
            default: kern = f64 ? mc_continue_kernel<4, GeoD> : mc_continue_kernel<4, GeoS>; break;
        }
    }
    if (cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)P->smem_bytes) !=
            cudaSuccess ||
        cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout,
                             (int)cudaSharedmemCarveoutMaxShared) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, P->block, P->smem_bytes) !=
            cudaSuccess ||
        per_sm < 1)
        return PDGPU_CUDA_ERROR;
    if (P->opt.blocks_per_sm > 0) per_sm = std::min(per_sm, (int)P->opt.blocks_per_sm);
    int64_t want = (prm.total + P->block - 1) / P->block;
    int grid = (int)std::min<int64_t>((int64_t)per_sm * P->nsm, std::max<int64_t>(want, 1));
    if (phase >= 1) grid = per_sm * P->nsm;  // parked count is only known on the device
    P->grid = grid;
    if (P->opt.time_launches && P->ev_ready) cudaEventRecord(P->ev[2 * lslot], st);
    kern<<<grid, P->block, P->smem_bytes, st>>>(prm);
    if (P->opt.time_launches && P->ev_ready) {
        cudaEventRecord(P->ev[2 * lslot + 1], st);
        P->ev_used = std::max(P->ev_used, lslot + 1);
    }
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

static pdgpu_status launch_prep(pdgpu_mc_plan* P, char* w, const float* rho, const int64_t* src,
                                int first, int epoch, cudaStream_t st) {
    PrepParams q;
    q.models = (const McModel*)(w + P->ws_models);
    q.dpool = (const double*)(w + P->ws_dpool);
    q.rho = rho;
    q.src = src;
    q.q = (float2*)(w + P->ws_q) + (size_t)epoch * P->total_cells;
    q.wq = (first && epoch == 0) ? (float*)(w + P->ws_wq) : nullptr;
    q.total = P->total_cells;
    q.nm = P->nm;
    q.ns = P->ns;
    q.first = first;
    q.epoch = epoch;
    int grid = (int)std::min<int64_t>((P->total_cells + 255) / 256, (int64_t)P->nsm * 8);
    mc_prep_kernel<<<std::max(grid, 1), 256, 0, st>>>(q);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_mc_plan_run(pdgpu_mc_plan* P, const float* rho, double* temperature, void* ws,
                               size_t bytes, void* stream) {
    if (!P || !rho || !temperature) return PDGPU_INVALID_ARG;
    if (!ws || bytes < P->ws_total || P->uploaded_ws != ws) return PDGPU_WORKSPACE;
    if (P->device < 0) return PDGPU_NO_DEVICE;
    cudaStream_t st = (cudaStream_t)stream;
    char* w = (char*)ws;
    int64_t* E = (int64_t*)(w + P->ws_E);
    int64_t* D = (int64_t*)(w + P->ws_D);
    int64_t* EL = (int64_t*)(w + P->ws_Elate);
    size_t cells_bytes = (size_t)P->total_cells * sizeof(int64_t);
    if (cudaMemsetAsync(E, 0, cells_bytes, st) != cudaSuccess ||
        cudaMemsetAsync(D, 0, cells_bytes, st) != cudaSuccess ||
        cudaMemsetAsync(EL, 0, cells_bytes, st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_parkcnt, 0, 4 * sizeof(unsigned long long), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_escape, 0, (size_t)P->nm * P->nl * sizeof(int64_t), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_stats, 0, MC_NSTAT * sizeof(int64_t), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_mstat, 0, (size_t)P->nm * sizeof(int32_t), st) != cudaSuccess ||
        cudaMemsetAsync(w + P->ws_queue, 0, (size_t)P->nqueue * sizeof(unsigned long long), st) !=
            cudaSuccess)
        return PDGPU_CUDA_ERROR;
    mc_start_kernel<<<1, 1, 0, st>>>((int64_t*)(w + P->ws_stats));
    pdgpu_status rc;
    int lslot = 0;
    P->ev_used = 0;
    unsigned long long* counts = (unsigned long long*)(w + P->ws_parkcnt);
    // one pilot or epoch launch; with draining, its last walks then resume one per warp
    auto epoch_launch = [&](int64_t* target, int epoch, uint32_t tag, bool final_pass) -> pdgpu_status {
        if (P->epoch_drain &&
            cudaMemsetAsync(counts + 1, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess)
            return PDGPU_CUDA_ERROR;
        pdgpu_status r = launch_transport(P, w, rho, target, epoch, tag, lslot++, final_pass, 0, st);
        if (r == PDGPU_OK && P->epoch_drain)
            r = launch_transport(P, w, rho, target, epoch, tag, lslot++, final_pass, 3, st);
        return r;
    };
    // first epoch: pilot passes write D (and stop at late_after), the real pass writes E
    for (int pass = P->npilot; pass >= 0; --pass) {
        if ((rc = launch_prep(P, w, rho, D, 1, 0, st)) != PDGPU_OK) return rc;
        if (pass > 0) {
            if (cudaMemsetAsync(D, 0, cells_bytes, st) != cudaSuccess) return PDGPU_CUDA_ERROR;
            rc = epoch_launch(D, 0, (uint32_t)pass, false);
        } else {
            rc = epoch_launch(E, 0, 0u, true);
        }
        if (rc != PDGPU_OK) return rc;
    }
    for (int k = 1; k < P->K; ++k) {
        if ((rc = launch_prep(P, w, rho, E, 0, k, st)) != PDGPU_OK) return rc;
        if ((rc = epoch_launch(E, k, 0u, true)) != PDGPU_OK) return rc;
    }
    // packets parked after late_after events finish here, each with its epoch's snapshot:
    // one per thread while there are many, the last few one per warp
    if (P->opt.late_after > 0) {
        if (cudaMemsetAsync(counts + 1, 0, 2 * sizeof(unsigned long long), st) != cudaSuccess)
            return PDGPU_CUDA_ERROR;
        if ((rc = launch_transport(P, w, rho, E, 0, 0u, lslot++, true, 1, st)) != PDGPU_OK) return rc;
        if ((rc = launch_transport(P, w, rho, E, 0, 0u, lslot++, true, 2, st)) != PDGPU_OK) return rc;
    }
    P->nlaunch = lslot;
    TempParams tp;
    tp.models = (const McModel*)(w + P->ws_models);
    tp.dpool = (const double*)(w + P->ws_dpool);
    tp.rho = rho;
    tp.E = E;
    tp.Elate = EL;
    tp.T = temperature;
    tp.total = P->total_cells;
    tp.nm = P->nm;
    tp.ns = P->ns;
    tp.off_tinv = P->off_tinv;
    tp.off_finv = P->off_finv;
    int grid = (int)std::min<int64_t>((P->total_cells + 255) / 256, (int64_t)P->nsm * 8);
    mc_temperature_kernel<<<std::max(grid, 1), 256, 0, st>>>(tp);
    mc_finish_kernel<<<1, 1, 0, st>>>((int64_t*)(w + P->ws_stats), P->total_nphot);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_mc_plan_stats(pdgpu_mc_plan* P, const void* ws, void* stream, pdgpu_mc_stats* S) {
    if (!P || !ws || !S) return PDGPU_INVALID_ARG;
    int64_t h[MC_NSTAT];
    cudaStream_t st = (cudaStream_t)stream;
    if (cudaMemcpyAsync(h, (const char*)ws + P->ws_stats, sizeof(h), cudaMemcpyDeviceToHost, st) !=
            cudaSuccess ||
        cudaStreamSynchronize(st) != cudaSuccess)
        return PDGPU_CUDA_ERROR;
    S->packets = h[ST_PACKETS];
    S->killed = h[ST_KILLED];
    S->escaped = h[ST_ESCAPED];
    S->crossings = h[ST_CROSSINGS];
    S->events = h[ST_EVENTS];
    S->absorptions = h[ST_ABSORB];
    S->scatterings = h[ST_SCATTER];
    S->mrw_steps = h[ST_MRW];
    S->status = (int32_t)h[ST_STATUS];
    S->launches = P->nlaunch;
    S->parked = h[ST_PARKED];
    S->drained = h[ST_DRAINED];
    S->late_units = h[ST_LATE];
    return PDGPU_OK;
}

size_t pdgpu_mctherm_workspace_bytes(int32_t nmodels, const pdgpu_model_desc* models,
                                     const pdgpu_dust_desc* dust, const pdgpu_mc_options* options) {
    pdgpu_mc_plan* P = nullptr;
    if (pdgpu_mc_plan_create(nmodels, models, dust, options, &P) != PDGPU_OK) return 0;
    size_t b = P->ws_total;
    pdgpu_mc_plan_destroy(P);
    return b;
}

pdgpu_status pdgpu_mctherm(int32_t nmodels, const pdgpu_model_desc* models, const pdgpu_dust_desc* dust,
                           const pdgpu_mc_options* options, const float* rho, double* temperature,
                           void* ws, size_t bytes, void* stream, pdgpu_mc_stats* stats) {
    pdgpu_mc_plan* P = nullptr;
    pdgpu_status rc = pdgpu_mc_plan_create(nmodels, models, dust, options, &P);
    if (rc != PDGPU_OK) return rc;
    rc = pdgpu_mc_plan_upload(P, ws, bytes, stream);
    if (rc == PDGPU_OK) rc = pdgpu_mc_plan_run(P, rho, temperature, ws, bytes, stream);
    pdgpu_mc_stats S;
    memset(&S, 0, sizeof(S));
    if (rc == PDGPU_OK) rc = pdgpu_mc_plan_stats(P, ws, stream, &S);
    if (rc == PDGPU_OK && S.status != PDGPU_OK) rc = S.status;
    if (stats) *stats = S;
    pdgpu_mc_plan_destroy(P);
    return rc;
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Scratch-free entry point: the plan workspace lives in a file-scope device array.
// ---------------------------------------------------------------------------------------
static __device__ __align__(256) unsigned char g_static_workspace[PDGPU_STATIC_WORKSPACE_BYTES];

namespace {
constexpr int kMaxDevices = 64;
std::mutex g_static_mutex;
void* g_static_address[kMaxDevices];  // device address of g_static_workspace per device

// Device address of the static scratch on the current device (looked up once per device,
// with that device current).  The host-side symbol is only a stand-in; kernels must get
// this address.
pdgpu_status static_workspace(void** out) {
    int dev = -1;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0) return PDGPU_NO_DEVICE;
    if (dev >= kMaxDevices) return PDGPU_NO_DEVICE;
    std::lock_guard<std::mutex> lock(g_static_mutex);
    if (!g_static_address[dev]) {
        void* p = nullptr;
        if (cudaGetSymbolAddress(&p, g_static_workspace) != cudaSuccess || !p)
            return PDGPU_CUDA_ERROR;
        g_static_address[dev] = p;
    }
    *out = g_static_address[dev];
    return PDGPU_OK;
}
}  // namespace

extern "C" pdgpu_status pdgpu_mctherm_static(int32_t nmodels, const pdgpu_model_desc* models,
                                             const pdgpu_dust_desc* dust,
                                             const pdgpu_mc_options* options, const float* rho,
                                             double* temperature, void* stream,
                                             pdgpu_mc_stats* stats) {
    if (!options) return PDGPU_INVALID_ARG;
    pdgpu_mc_options opt = *options;
    opt.time_launches = 0;  // no event objects on this path
    pdgpu_mc_plan* P = nullptr;
    pdgpu_status rc = pdgpu_mc_plan_create(nmodels, models, dust, &opt, &P);
    if (rc != PDGPU_OK) return rc;
    if (P->ws_total > (size_t)PDGPU_STATIC_WORKSPACE_BYTES) {
        pdgpu_mc_plan_destroy(P);
        return PDGPU_TOO_LARGE;
    }
    void* ws = nullptr;
    rc = static_workspace(&ws);
    const size_t bytes = PDGPU_STATIC_WORKSPACE_BYTES;
    if (rc == PDGPU_OK) rc = pdgpu_mc_plan_upload(P, ws, bytes, stream);
    if (rc == PDGPU_OK) rc = pdgpu_mc_plan_run(P, rho, temperature, ws, bytes, stream);
    pdgpu_mc_stats S;
    memset(&S, 0, sizeof(S));
    if (rc == PDGPU_OK) rc = pdgpu_mc_plan_stats(P, ws, stream, &S);
    if (rc == PDGPU_OK && S.status != PDGPU_OK) rc = S.status;
    if (stats) *stats = S;
    pdgpu_mc_plan_destroy(P);
    return rc;
}
