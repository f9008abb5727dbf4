"""This package's host-side builders against golden fixtures produced by the reference
pdspy's own code (tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

from pdspy_gb300 import constants as K
from pdspy_gb300.modeling import Disk, Star, UlrichEnvelopeExtended

G = np.load(os.path.join(os.path.dirname(__file__), "golden", "pdspy_builders.npz"))


def centres(w):
    return 0.5 * (w[1:] + w[:-1])


def test_disk_density_matches_pdspy():
    r, th, ph = centres(G["disk_w1"]), centres(G["disk_w2"]), centres(G["disk_w3"])
    d = Disk(mass=1e-4, rmin=0.1, rmax=100.0, plrho=2.25, h0=0.1, plh=1.25)
    assert np.allclose(d.density(r, th, ph), G["disk_rho"], rtol=1e-12, atol=0)


def test_mirrored_disk_density_matches_pdspy():
    r, th, ph = centres(G["disk_w1"]), centres(G["disk2_w2"]), centres(G["disk_w3"])
    d = Disk(mass=3e-3, rmin=0.5, rmax=60.0, plrho=2.1, h0=0.05, plh=1.1)
    assert np.allclose(d.density(r, th, ph), G["disk2_rho"], rtol=1e-12, atol=0)


def test_ulrich_envelope_density_matches_pdspy():
    r, th = centres(G["env_w1"]), centres(G["env_w2"])
    e = UlrichEnvelopeExtended(mass=0.05, rmin=0.1, rmax=1e4, rcent=100.0, cavpl=1.0,
                               cavrfact=0.2, theta_open=20.0, zoffset=1.0)
    rho = e.density(r, th, np.array([np.pi]))
    assert np.allclose(rho, G["env_rho"], rtol=1e-10, atol=0)


def test_star_radius_and_constants_match_pdspy():
    s = Star(mass=0.5, luminosity=0.9064, temperature=4000.0)
    assert s.radius == pytest.approx(G["star_radius_rsun"][0], rel=1e-15)
    mine = [K.AU, K.M_sun, K.R_sun, K.L_sun, K.sigma, K.h, K.k, K.c, K.pc, K.Jy, K.pi_pdspy]
    assert np.array_equal(np.array(mine), G["constants"])


def test_temperature_layout_matches_reference_reshape():
    """pdspy turns RADMC-3D's x-fastest temperature file into (nr, ntheta, nphi) with
    reshape((n3, n2, n1)).transpose(2, 1, 0) (Model.py:250-254); the GPU path writes the
    numpy C-order (nr, ntheta, nphi) array directly, which must be the same array."""
    n1, n2, n3 = 4, 3, 2
    T = np.arange(n1 * n2 * n3, dtype=float).reshape(n1, n2, n3)   # our layout
    file_order = np.array([T[ix, iy, iz] for iz in range(n3) for iy in range(n2)
                           for ix in range(n1)])                    # write.py:283-286 order
    ref = np.transpose(file_order.reshape((n3, n2, n1)), axes=(2, 1, 0))
    assert np.array_equal(ref, T)
