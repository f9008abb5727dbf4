// Direct Fourier transform of an image at arbitrary (u, v) points and its adjoint.
//
// The model visibilities of an interferometric fit, V(u, v) = sum_p F_p exp(-2 pi i
// (u x_p + v y_p)) with F in Jy per pixel, x, y the pixel offsets in radians and u, v in
// wavelengths; the chi^2 of pdspy's interferometry.chisq
// (pdspy/interferometry/libinterferometry.pyx:610-633) is formed from Re V and Im V by
// the caller.  pdspy samples images with galario's FFT interpolation
// (pdspy/interferometry/interpolate_model.py:11-57); a direct sum is exact at every uv
// point and has a simple, exact adjoint.
//
// Forward: eight threads per uv point, image tiles staged in shared memory and read by the
// whole block.  Adjoint: eight threads per pixel, uv tiles staged in shared memory.  Phases
// are formed in FP32 (|u x| of a few turns keeps the phase error ~1e-6 rad) and
// evaluated with sincospif; sums accumulate in FP32 per tile and in FP64 across tiles.
//
// Gridded sampling (the method of galario's sampleImage, Tazzari, Beaujean & Testi 2018,
// MNRAS 476, 4527, which pdspy calls in interpolate_model.py:20-27): the caller
// transforms the (zero-padded) image with a 2-D FFT; W(u_k, v_l) = (-1)^(k+l) G[l][k] is
// the transform of the image about its centre pixel (n/2, n/2), smooth for a centred
// source, and is interpolated bilinearly at each (u, v) (grid spacing du = 1 / (n dx));
// the centre's phase exp(-2 pi i (u xc + v yc)) is applied exactly.  One thread per uv
// point; points beyond the last full grid cell of the band return NaN.  The adjoint
// scatters the bilinear weights onto the grid (FP64 atomics); the caller finishes it with
// one more FFT.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/pdgpu.h"

namespace {

constexpr int DFT_TILE = 512;
// A block of 256 threads serves DFT_POINTS outputs (uv points forward, pixels adjoint);
// the DFT_GROUPS warps of the block split each staged tile by index modulo DFT_GROUPS, so
// every warp reads one shared-memory entry per step (a broadcast) and the group partial
// sums are added in a fixed order at the end: deterministic results and eight times the
// blocks of a thread-per-output launch (20,000 uv points fill every SM).
constexpr int DFT_GROUPS = 8;
constexpr int DFT_POINTS = 32;
static_assert(DFT_GROUPS * DFT_POINTS == 256, "one block of 256 threads");

__global__ void __launch_bounds__(256) dft_forward_kernel(int nx, int ny, float x0, float dx,
                                                          float y0, float dy, const float* img,
                                                          int nuv, const float* u,
                                                          const float* v, double* re,
                                                          double* im) {
    __shared__ float s_f[DFT_TILE];
    __shared__ float s_x[DFT_TILE];
    __shared__ float s_y[DFT_TILE];
    __shared__ double s_re[DFT_GROUPS][DFT_POINTS];
    __shared__ double s_im[DFT_GROUPS][DFT_POINTS];
    const int j = threadIdx.x % DFT_POINTS;
    const int g = threadIdx.x / DFT_POINTS;
    const int k = blockIdx.x * DFT_POINTS + j;
    const float uk = (k < nuv) ? u[k] : 0.0f;
    const float vk = (k < nuv) ? v[k] : 0.0f;
    const int npix = nx * ny;
    double ar = 0.0, ai = 0.0;
    for (int t0 = 0; t0 < npix; t0 += DFT_TILE) {
        int n = min(DFT_TILE, npix - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int p = t0 + i;
            s_f[i] = img[p];
            s_x[i] = x0 + (float)(p % nx) * dx;
            s_y[i] = y0 + (float)(p / nx) * dy;
        }
        __syncthreads();
        float tr = 0.0f, ti = 0.0f;
        for (int i = g; i < n; i += DFT_GROUPS) {
            float f = s_f[i];
            if (f == 0.0f) continue;
            float ph = 2.0f * (uk * s_x[i] + vk * s_y[i]);
            float sn, cs;
            sincospif(ph, &sn, &cs);
            tr += f * cs;
            ti -= f * sn;
        }
        ar += tr;
        ai += ti;
    }
    s_re[g][j] = ar;
    s_im[g][j] = ai;
    __syncthreads();
    if (g == 0 && k < nuv) {
        double r = s_re[0][j], q = s_im[0][j];
        for (int h = 1; h < DFT_GROUPS; ++h) {
            r += s_re[h][j];
            q += s_im[h][j];
        }
        re[k] = r;
        im[k] = q;
    }
}

__global__ void __launch_bounds__(256) dft_adjoint_kernel(int nx, int ny, float x0, float dx,
                                                          float y0, float dy, int nuv,
                                                          const float* u, const float* v,
                                                          const double* gre, const double* gim,
                                                          double* gimg) {
    __shared__ float s_u[DFT_TILE];
    __shared__ float s_v[DFT_TILE];
    __shared__ float s_gr[DFT_TILE];
    __shared__ float s_gi[DFT_TILE];
    __shared__ double s_acc[DFT_GROUPS][DFT_POINTS];
    const int j = threadIdx.x % DFT_POINTS;
    const int g = threadIdx.x / DFT_POINTS;
    const int p = blockIdx.x * DFT_POINTS + j;
    const int npix = nx * ny;
    const float xp = x0 + (float)(p % nx) * dx;
    const float yp = y0 + (float)(p / nx) * dy;
    double acc = 0.0;
    for (int t0 = 0; t0 < nuv; t0 += DFT_TILE) {
        int n = min(DFT_TILE, nuv - t0);
        __syncthreads();
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            s_u[i] = u[t0 + i];
            s_v[i] = v[t0 + i];
            s_gr[i] = (float)gre[t0 + i];
            s_gi[i] = (float)gim[t0 + i];
        }
        __syncthreads();
        float t = 0.0f;
        for (int i = g; i < n; i += DFT_GROUPS) {
            float ph = 2.0f * (s_u[i] * xp + s_v[i] * yp);
            float sn, cs;
            sincospif(ph, &sn, &cs);
            // Re V = sum F cos, Im V = -sum F sin
            t += s_gr[i] * cs - s_gi[i] * sn;
        }
        acc += t;
    }
    s_acc[g][j] = acc;
    __syncthreads();
    if (g == 0 && p < npix) {
        double a = s_acc[0][j];
        for (int h = 1; h < DFT_GROUPS; ++h) a += s_acc[h][j];
        gimg[p] = a;
    }
}


// Grid index of the four corners of (fu, fv), their weights and the (-1)^(k+l) signs.
struct Bilin {
    int64_t idx[4];
    float w[4];
};

__device__ __forceinline__ bool bilin_of(int n, float fu, float fv, Bilin& b) {
    const float lim = 0.5f * (float)n - 1.0f;
    if (!(fabsf(fu) < lim) || !(fabsf(fv) < lim)) return false;
    const float fk = floorf(fu), fl = floorf(fv);
    const int k0 = (int)fk, l0 = (int)fl;
    const float t = fu - fk, s = fv - fl;
    const float wk[2] = {1.0f - t, t};
    const float wl[2] = {1.0f - s, s};
#pragma unroll
    for (int a = 0; a < 2; ++a)
#pragma unroll
        for (int c = 0; c < 2; ++c) {
            const int k = k0 + c, l = l0 + a;
            const int km = ((k % n) + n) % n, lm = ((l % n) + n) % n;
            const float sg = ((k + l) & 1) ? -1.0f : 1.0f;
            b.idx[2 * a + c] = (int64_t)lm * n + km;
            b.w[2 * a + c] = sg * wk[c] * wl[a];
        }
    return true;
}

__global__ void __launch_bounds__(256) vis_grid_sample_kernel(int n, const float2* __restrict__ G,
                                                              double du, double dv, double xc,
                                                              double yc, int nuv,
                                                              const float* __restrict__ u,
                                                              const float* __restrict__ v,
                                                              double* re, double* im) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nuv) return;
    const double uk = (double)u[k], vk = (double)v[k];
    Bilin b;
    if (!bilin_of(n, (float)(uk / du), (float)(vk / dv), b)) {
        re[k] = __longlong_as_double(0x7ff8000000000000ll);
        im[k] = __longlong_as_double(0x7ff8000000000000ll);
        return;
    }
    float wr = 0.0f, wi = 0.0f;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        const float2 g = __ldg(G + b.idx[c]);
        wr += b.w[c] * g.x;
        wi += b.w[c] * g.y;
    }
    double sn, cs;
    sincospi(-2.0 * (uk * xc + vk * yc), &sn, &cs);
    re[k] = (double)wr * cs - (double)wi * sn;
    im[k] = (double)wr * sn + (double)wi * cs;
}

__global__ void __launch_bounds__(256) vis_grid_sample_adjoint_kernel(
    int n, double du, double dv, double xc, double yc, int nuv, const float* __restrict__ u,
    const float* __restrict__ v, const double* __restrict__ gre, const double* __restrict__ gim,
    double2* H) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nuv) return;
    const double uk = (double)u[k], vk = (double)v[k];
    Bilin b;
    if (!bilin_of(n, (float)(uk / du), (float)(vk / dv), b)) return;
    double sn, cs;
    sincospi(-2.0 * (uk * xc + vk * yc), &sn, &cs);
    // conj(g) P with g = gre + i gim, P = cs + i sn
    const double hr = gre[k] * cs + gim[k] * sn;
    const double hi = gre[k] * sn - gim[k] * cs;
#pragma unroll
    for (int c = 0; c < 4; ++c) {
        atomicAdd(&H[b.idx[c]].x, (double)b.w[c] * hr);
        atomicAdd(&H[b.idx[c]].y, (double)b.w[c] * hi);
    }
}

}  // namespace

extern "C" {

pdgpu_status pdgpu_vis_dft(int32_t nx, int32_t ny, double x0_rad, double dx_rad, double y0_rad,
                           double dy_rad, const float* image, int32_t nuv, const float* u,
                           const float* v, double* re, double* im, void* stream) {
    if (nx < 1 || ny < 1 || nuv < 1 || !image || !u || !v || !re || !im) return PDGPU_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    const int blocks = (nuv + DFT_POINTS - 1) / DFT_POINTS;
    dft_forward_kernel<<<blocks, 256, 0, st>>>(nx, ny, (float)x0_rad, (float)dx_rad,
                                               (float)y0_rad, (float)dy_rad, image, nuv, u, v,
                                               re, im);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_vis_dft_adjoint(int32_t nx, int32_t ny, double x0_rad, double dx_rad,
                                   double y0_rad, double dy_rad, int32_t nuv, const float* u,
                                   const float* v, const double* grad_re, const double* grad_im,
                                   double* grad_image, void* stream) {
    if (nx < 1 || ny < 1 || nuv < 1 || !u || !v || !grad_re || !grad_im || !grad_image)
        return PDGPU_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    int npix = nx * ny;
    const int blocks = (npix + DFT_POINTS - 1) / DFT_POINTS;
    dft_adjoint_kernel<<<blocks, 256, 0, st>>>(nx, ny, (float)x0_rad, (float)dx_rad,
                                               (float)y0_rad, (float)dy_rad, nuv, u, v, grad_re,
                                               grad_im, grad_image);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_vis_grid_sample(int32_t n, const float* grid, double du, double dv, double xc,
                                   double yc, int32_t nuv, const float* u, const float* v,
                                   double* re, double* im, void* stream) {
    if (n < 4 || (n & 1) || !(du > 0.0) || !(dv > 0.0) || nuv < 1 || !grid || !u || !v || !re ||
        !im)
        return PDGPU_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    vis_grid_sample_kernel<<<(nuv + 255) / 256, 256, 0, st>>>(n, (const float2*)grid, du, dv, xc,
                                                             yc, nuv, u, v, re, im);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

pdgpu_status pdgpu_vis_grid_sample_adjoint(int32_t n, double du, double dv, double xc, double yc,
                                           int32_t nuv, const float* u, const float* v,
                                           const double* grad_re, const double* grad_im,
                                           double* grad_grid, void* stream) {
    if (n < 4 || (n & 1) || !(du > 0.0) || !(dv > 0.0) || nuv < 1 || !u || !v || !grad_re ||
        !grad_im || !grad_grid)
        return PDGPU_INVALID_ARG;
    cudaStream_t st = (cudaStream_t)stream;
    vis_grid_sample_adjoint_kernel<<<(nuv + 255) / 256, 256, 0, st>>>(
        n, du, dv, xc, yc, nuv, u, v, grad_re, grad_im, (double2*)grad_grid);
    return cudaGetLastError() == cudaSuccess ? PDGPU_OK : PDGPU_CUDA_ERROR;
}

}  // extern "C"
