"""Float64 references for the ray tracer: per-ray segments from the CPU oracle, combined
in torch so autograd gives reference gradients."""
import numpy as np
import torch

from oracle import orc
from pdspy_gb300 import thermal


def segments(model, npix, pixel_cm, levels, incl=0.0, pa=0.0, phi=0.0):
    """[(pixel, [(cells, lengths) per sub-ray])], plus the star's line of sight."""
    r, t, p = thermal.grid_arrays(model.grid)
    out = []
    for py in range(npix):
        for px in range(npix):
            L = int(levels[py, px])
            rays = [orc.ray_segments(r, t, p, npix, pixel_cm, px, py, s, L, incl, pa, phi)
                    for s in range(4 ** L)]
            out.append(rays)
    star = orc.ray_segments(r, t, p, npix, pixel_cm, 0, 0, -1, 0, incl, pa, phi)
    return out, star


def image(alpha, S, segs, star_segs, star_flux, npix, pixel_cm, nostar=False):
    """Pixel-averaged intensity at 1 pc [nlam, npix, npix] (float64, differentiable)."""
    nl = alpha.shape[0]
    pix = []
    for rays in segs:
        acc = torch.zeros(nl, dtype=torch.float64, device=alpha.device)
        for cells, lens in rays:
            if len(cells) == 0:
                continue
            c = torch.as_tensor(cells, dtype=torch.long, device=alpha.device)
            ln = torch.as_tensor(lens, dtype=torch.float64, device=alpha.device)
            dt = alpha[:, c] * ln
            cum = torch.cumsum(dt, dim=1) - dt
            acc = acc + (torch.exp(-cum) * S[:, c] * (-torch.expm1(-dt))).sum(1)
        pix.append(acc / len(rays))
    img = torch.stack(pix, dim=1).reshape(nl, npix, npix)
    if not nostar:
        c = torch.as_tensor(star_segs[0], dtype=torch.long, device=alpha.device)
        ln = torch.as_tensor(star_segs[1], dtype=torch.float64, device=alpha.device)
        tau = (alpha[:, c] * ln).sum(1)
        omega = (pixel_cm / 3.085677581e18) ** 2
        sf = torch.as_tensor(np.asarray(star_flux, dtype=np.float64), device=alpha.device)
        add = torch.zeros_like(img)
        add[:, npix // 2, npix // 2] = sf * torch.exp(-tau) / omega
        img = img + add
    return img


def dft(image, u, v, x0, dx, y0, dy):
    """Dense float64 DFT: Re, Im of sum F exp(-2 pi i (u x + v y))."""
    ny, nx = image.shape
    x = x0 + torch.arange(nx, dtype=torch.float64, device=image.device) * dx
    y = y0 + torch.arange(ny, dtype=torch.float64, device=image.device) * dy
    ph_x = 2 * np.pi * u[:, None] * x[None, :]           # [K, nx]
    ph_y = 2 * np.pi * v[:, None] * y[None, :]           # [K, ny]
    cx, sx, cy, sy = torch.cos(ph_x), torch.sin(ph_x), torch.cos(ph_y), torch.sin(ph_y)
    # exp(-i(a+b)) = (cos a cos b - sin a sin b) - i (sin a cos b + cos a sin b)
    A = cx @ image.T      # [K, ny]: sum_i F[j,i] cos(a_i)
    B = sx @ image.T
    re = (A * cy - B * sy).sum(1)
    im = -(B * cy + A * sy).sum(1)
    return re, im
