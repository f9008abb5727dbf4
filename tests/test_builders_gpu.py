"""Device density builders on the GPU: the same fields as on the host."""
import numpy as np
import pytest
import torch

from pdspy_gb300 import builders

pytestmark = pytest.mark.gpu


def test_builders_on_gpu_match_host(cuda):
    r = np.logspace(-1, 4, 257)
    th = np.linspace(0, np.pi, 257)
    rc, tc, pc = 0.5 * (r[1:] + r[:-1]), 0.5 * (th[1:] + th[:-1]), np.array([np.pi])
    m = torch.tensor(0.05, dtype=torch.float64, device=cuda, requires_grad=True)
    g = builders.ulrich_envelope_density(rc, tc, pc, m, 0.1, 1e4, 100.0, 1.0, 0.2, 20.0, 1.0)
    h = builders.ulrich_envelope_density(rc, tc, pc, 0.05, 0.1, 1e4, 100.0, 1.0, 0.2, 20.0, 1.0)
    assert g.device.type == "cuda"
    assert torch.allclose(g.detach().cpu(), h, rtol=1e-12, atol=0)
    g.sum().backward()
    assert torch.isfinite(m.grad)
    d = builders.disk_density(rc, tc, pc, torch.tensor(1e-2, dtype=torch.float64, device=cuda),
                              0.1, 100.0, 2.25, 0.1, 1.25)
    e = builders.disk_density(rc, tc, pc, 1e-2, 0.1, 100.0, 2.25, 0.1, 1.25)
    assert torch.allclose(d.cpu(), e, rtol=1e-12, atol=0)
