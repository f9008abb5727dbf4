"""Device density builders (pdspy_gb300.builders) against pdspy's own builders (golden
fixtures from pdspy/modeling/Disk.py and UlrichEnvelopeExtended.py, tests/golden/) and
their gradients against float64 central differences.  CPU only: the builders are torch
code that runs on either device."""
import os

import numpy as np
import pytest
import torch

from pdspy_gb300 import builders

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "pdspy_builders.npz")


def _c(w):
    return 0.5 * (w[1:] + w[:-1])


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLDEN)


def _rel(a, b):
    m = b > 0
    assert np.array_equal(a > 0, m)
    return np.abs(a[m] / b[m] - 1).max()


def test_disk_matches_pdspy(gold):
    ph = _c(gold["disk_w3"])
    a = builders.disk_density(_c(gold["disk_w1"]), _c(gold["disk_w2"]), ph, 1e-4, 0.1, 100.0,
                              2.25, 0.1, 1.25).numpy()
    assert _rel(a, gold["disk_rho"]) < 1e-11
    b = builders.disk_density(_c(gold["disk_w1"]), _c(gold["disk2_w2"]), ph, 3e-3, 0.5, 60.0,
                              2.1, 0.05, 1.1).numpy()
    assert _rel(b, gold["disk2_rho"]) < 1e-11


def test_ulrich_envelope_matches_pdspy(gold):
    rho = builders.ulrich_envelope_density(_c(gold["env_w1"]), _c(gold["env_w2"]),
                                           _c(gold["disk_w3"]), 0.05, 0.1, 1e4, 100.0, 1.0, 0.2,
                                           20.0, 1.0).numpy()
    assert np.all(np.isfinite(rho))
    assert _rel(rho, gold["env_rho"]) < 1e-9


def test_streamline_root_is_brenths():
    from scipy.optimize import brenth
    rng = np.random.default_rng(0)
    x = np.concatenate([10 ** rng.uniform(-4, 3, 3000), rng.uniform(0.5, 1.5, 1000)])
    mu = np.cos(rng.uniform(1e-3, np.pi - 1e-3, x.size))
    got = builders.streamline_mu0(torch.as_tensor(x), torch.as_tensor(mu)).numpy()
    f = lambda m0, xx, mm: m0 ** 3 - m0 * (1 - xx) - mm * xx
    ref = np.array([brenth(f, -1.0, 1.0, args=(a, b)) for a, b in zip(x, mu)])
    # near x = 1, mu = +-1 the root is a near-triple root and brenth stops at its xtol
    assert np.max(np.abs(got - ref)) < 1e-7


def test_envelope_gradients_vs_central_differences():
    r = np.logspace(-1, 4, 41)
    th = np.linspace(0.01, np.pi - 0.01, 33)
    ph = np.array([np.pi])
    rng = np.random.default_rng(1)
    w = torch.as_tensor(rng.random((40, 32, 1)))
    rc, cp, co = _c(r), _c(th), ph

    def L(mass, rcent):
        return (builders.ulrich_envelope_density(rc, cp, co, mass, 0.1, 1e4, rcent, 1.0, 0.2,
                                                 20.0, 1.0) * w).sum() * 1e20

    m = torch.tensor(0.05, dtype=torch.float64, requires_grad=True)
    R = torch.tensor(100.0, dtype=torch.float64, requires_grad=True)
    L(m, R).backward()
    for var, g, x0 in ((0, m.grad, 0.05), (1, R.grad, 100.0)):
        h = x0 * 1e-6
        a = [0.05, 100.0]
        b = [0.05, 100.0]
        a[var] += h
        b[var] -= h
        D = torch.float64
        fd = (L(torch.tensor(a[0], dtype=D), torch.tensor(a[1], dtype=D)) -
              L(torch.tensor(b[0], dtype=D), torch.tensor(b[1], dtype=D))) / (2 * h)
        assert abs(float(g) / float(fd) - 1) < 1e-5, (var, float(g), float(fd))
    # the cavity factor carries a gradient; the cavity shape only moves the (discontinuous)
    # mask, so cavpl, theta_open and zoffset have none
    p = [torch.tensor(v, dtype=torch.float64, requires_grad=True) for v in (1.0, 0.2, 20.0, 1.0)]
    out = builders.ulrich_envelope_density(rc, cp, co, 0.05, 0.1, 1e4, 100.0, *p)
    (out * w).sum().backward()
    assert torch.isfinite(p[1].grad) and float(p[1].grad) != 0.0
    assert all(v.grad is None or float(v.grad) == 0.0 for v in (p[0], p[2], p[3]))


def test_disk_gradients_vs_central_differences():
    r = np.logspace(-1, 2, 31)
    th = np.linspace(0, np.pi, 41)
    rc, tc, pc = _c(r), _c(th), np.array([np.pi])
    rng = np.random.default_rng(2)
    w = torch.as_tensor(rng.random((30, 40, 1)))
    x0 = [1e-3, 2.2, 0.1, 1.2]

    def L(v):
        return (builders.disk_density(rc, tc, pc, v[0], 0.1, 100.0, v[1], v[2], v[3]) * w).sum()

    v = [torch.tensor(a, dtype=torch.float64, requires_grad=True) for a in x0]
    L(v).backward()
    for i in range(4):
        h = x0[i] * 1e-6
        a = list(x0); b = list(x0)
        a[i] += h; b[i] -= h
        fd = (L([torch.tensor(t, dtype=torch.float64) for t in a]) -
              L([torch.tensor(t, dtype=torch.float64) for t in b])) / (2 * h)
        assert abs(float(v[i].grad) / float(fd) - 1) < 1e-5
