/*
 * CPU oracle of the ray-traced images behind pdspy's Model.run_image / run_sed
 * (radmc3d branch: pdspy/modeling/Model.py:515-577 and :608-650; the arithmetic is in the
 * external RADMC-3D binary, "radmc3d image" / "radmc3d spectrum", pdspy/radmc3d/run.py).
 * TEST INFRASTRUCTURE ONLY: loaded by tests/ and the CPU-baseline leg of bench.py.
 *
 * Restated method: the formal solution of the transfer equation along straight rays
 * through the spherical grid, traced from the observer into the model (front to back),
 * I = sum_i W_i S_i (1 - exp(-dtau_i)), W_{i+1} = W_i exp(-dtau_i), with per-cell
 * extinction alpha = sum_s rho_s kext_s and source S = B_nu(T) sum_s rho_s kabs_s / alpha
 * (thermal emission, no scattering source), plus the star as a point source attenuated
 * along the central ray.  Pixels whose rays pass near cells smaller than the pixel are
 * refined into 4^L sub-rays (same rule as the GPU path).  Output is the pixel-averaged
 * intensity at 1 pc in erg s^-1 cm^-2 Hz^-1 ster^-1 (radmc3d/read.pyx:25-152 units).
 */
#ifndef PDSPY_RAYTRACE_ORACLE_H
#define PDSPY_RAYTRACE_ORACLE_H
#include <stdint.h>

#include "mcrt_oracle.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int npix_x, npix_y;
    double pixel_cm;          /* pixel size in the source plane (cm)                 */
    double incl_deg, pa_deg, phi_deg;
    int nostar;
    int max_refine;           /* maximum refinement level L (4^L sub-rays per pixel) */
    double refine_factor;     /* sub-pixel size <= factor * radial cell width        */
} orc_camera;

/* alpha, S: per cell and camera wavelength, [nlam][ncell] (float, as the GPU path).
 * star_flux[nlam]: stellar intensity-equivalent flux at 1 pc (erg/s/cm^2/Hz), i.e.
 * pi B_nu(T*) R*^2 / pc^2 summed over stars, added to the pixel containing the origin.
 * image[nlam][ny][nx] receives the pixel-averaged intensity (double).
 * If seg_out != NULL, the sub-ray segments of pixel (seg_px, seg_py) are written as
 * (cell, length) pairs for the float64 autograd reference; returns their count. */
int orc_image(const orc_grid* grid, int nlam, const float* alpha, const float* S,
              const double* star_flux, const orc_camera* cam, double* image);

/* Per-pixel sub-ray refinement levels (for tests). */
void orc_refine_levels(const orc_grid* grid, const orc_camera* cam, int* levels);

/* Segments of one sub-ray: writes up to cap (cell, length_cm) pairs; returns count. */
int orc_ray_segments(const orc_grid* grid, const orc_camera* cam, int px, int py, int sub,
                     int level, int* cells, double* lengths, int cap);

#ifdef __cplusplus
}
#endif
#endif
