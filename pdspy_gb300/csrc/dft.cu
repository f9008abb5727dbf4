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
// Forward: four threads per uv point, image tiles staged in shared memory and read by the
// whole block.  Adjoint: four threads per pixel, uv tiles staged in shared memory.  Phases
// are formed in FP32 (|u x| of a few turns keeps the phase error ~1e-6 rad) and
// evaluated with sincospif; sums accumulate in FP32 per tile and in FP64 across tiles.
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/pdgpu.h"

namespace {

constexpr int DFT_TILE = 512;
// A block of 256 threads serves DFT_POINTS outputs (uv points forward, pixels adjoint);
// the DFT_GROUPS warp pairs of the block split each staged tile by index modulo
// DFT_GROUPS, so every warp reads one shared-memory entry per step (a broadcast) and the
// group partial sums are added in a fixed order at the end: deterministic results and
// four times the blocks of a thread-per-output launch.
constexpr int DFT_GROUPS = 4;
constexpr int DFT_POINTS = 64;
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

}  // extern "C"
