"""GPU thermal Monte Carlo against the CPU oracle, bit for bit, on the benchmark
configurations at their own grid sizes and with the production settings of pdspy's
run_disk_model.py:251-255 (modified random walk, gamma 2, tauthres 10, count trigger 100)
and the product's default epoch schedule (8 epochs, 2 pilot passes, packets feeding later
epochs for their first 1e5 events, eager MRW beyond 1e4 events).  Packet counts are cut
where the oracle would take minutes; the grids, densities and dust are the configurations'.
"""
import numpy as np
import pytest
import torch

from pdspy_gb300 import thermal, workloads
from tests import _cases

pytestmark = pytest.mark.gpu

MRW = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)


def _gpu(models, nphot, **kw):
    plan = thermal.ThermalPlan([m.grid for m in models], nphot, **kw)
    rho, T = plan.new_buffers()
    rho.copy_(torch.from_numpy(np.concatenate(
        [thermal.stack_density(m.grid).reshape(-1) for m in models])))
    plan.run(rho, T)
    torch.cuda.synchronize()
    st = plan.check_status()
    return plan, plan.energy().cpu().numpy(), T.cpu().numpy(), st


def _check_models(models, nphot, seed, **kw):
    plan, E, T, st = _gpu(models, nphot, seed=seed, **MRW, **kw)
    off = 0
    ev = 0
    for i, m in enumerate(models):
        ref = _cases.run_oracle(m, nphot, seed=seed, model_id=i, **MRW, **kw)
        n = ref["energy"].size
        assert np.array_equal(E[off:off + n], ref["energy"].reshape(-1)), i
        assert np.array_equal(T[off:off + n], ref["temperature"].reshape(-1)), i
        ev += ref["stats"]["events"]
        off += n
    assert off == E.size
    assert st["events"] == ev
    return st


def test_config0_plain_disk_bit_exact(cuda):
    """100 x 100 cells over [0, pi], Mdisk 1e-4, 1e5 packets: the whole configuration."""
    _check_models([workloads.small_disk()], 100000, seed=0)


def test_config2_every_walker_bit_exact(cuda):
    """All 64 walker disks of the batched workload on their own grids (nr 64-256,
    ntheta 64-192) in one batched plan, 2e3 packets each."""
    _check_models(workloads.walker_models(n=64, seed=0), 2000, seed=0)


def test_config1_disk_envelope_bit_exact(cuda):
    """256 x 256 cells to 1e4 au, disk + Ulrich envelope (two species), 1e4 packets."""
    _check_models([workloads.disk_envelope(nr=256, ntheta=256)], 10000, seed=1)


def test_config4_spiral_bit_exact(cuda):
    """128^3 cells with phi walls, two grain populations, one spiral phase, 1e5 packets."""
    m = workloads.spiral_disk(nr=128, ntheta=128, nphi=128, mass=1e-4, phase=1.0)
    _check_models([m], 100000, seed=0)
