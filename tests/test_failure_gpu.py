"""Failure detection of the thermal launches without a GPU fault: the device-side deadline
and the abort flag end a run with a status the host reads, and the plan (and the CUDA
context) stay usable for the next run."""
import subprocess

import numpy as np
import pytest
import torch

from pdspy_gb300 import _lib, thermal
from tests import _cases

pytestmark = pytest.mark.gpu


def _plan(**kw):
    m, extra = _cases.case("two_species_mrw")
    plan = thermal.ThermalPlan([m.grid], 20000, seed=3, **extra, **kw)
    rho, T = plan.new_buffers()
    rho.copy_(torch.from_numpy(thermal.stack_density(m.grid).reshape(-1)))
    return plan, rho, T


def test_deadline_ends_the_run_and_the_plan_recovers(cuda):
    ref, rho0, T0 = _plan()
    ref.run(rho0, T0)
    ref.check_status()
    plan, rho, T = _plan(timelimit=2e-5)          # 20 microseconds of device time
    plan.run(rho, T)
    with pytest.raises(subprocess.TimeoutExpired):
        plan.check_status()
    plan.set_timelimit(None)                       # the same plan, no budget
    plan.run(rho, T)
    plan.check_status()
    assert torch.equal(T, T0) and torch.equal(plan.energy(), ref.energy())


def test_abort_flag_stops_the_run(cuda):
    flag = torch.ones(1, dtype=torch.int32, device=cuda)
    plan, rho, T = _plan(abort_flag=flag.data_ptr())
    plan.run(rho, T)
    with pytest.raises(_lib.PdgpuError) as e:
        plan.check_status()
    assert e.value.status == 3                     # PDGPU_ABORTED
    flag.zero_()
    plan.run(rho, T)
    st = plan.check_status()
    assert st["status"] == 0 and st["packets"] == 20000


def test_one_walker_timeout_leaves_the_others_unchanged(cuda):
    """A batched plan with a per-model limit: the walker whose limit is 1 ns stops alone
    (status 2, its packets dropped); every other walker's energies and temperatures are
    bit for bit those of the same plan run without limits."""
    from pdspy_gb300 import workloads
    models = workloads.walker_models(n=4, seed=8, scale=0.2)
    plan = thermal.ThermalPlan([m.grid for m in models], 3000, seed=4, mrw=True,
                               mrw_count_trigger=10)
    rho, T = plan.new_buffers()
    rho.copy_(torch.from_numpy(np.concatenate([thermal.stack_density(m.grid).reshape(-1)
                                               for m in models])))
    plan.run(rho, T)
    plan.check_status()
    assert list(plan.model_status()) == [0, 0, 0, 0]
    E0, T0 = plan.energy().clone(), T.clone()
    plan.set_model_timelimits([None, 1e-9, None, 3600.0])
    plan.run(rho, T)
    st = plan.check_status()                       # the launch as a whole completes
    assert st["status"] == 0
    assert list(plan.model_status()) == [0, 2, 0, 0]
    off = 0
    for i, (ns, nr, nt, np_) in enumerate(plan.shapes):
        n = ns * nr * nt * np_
        if i != 1:
            assert torch.equal(plan.energy()[off:off + n], E0[off:off + n]), i
            assert torch.equal(T[off:off + n], T0[off:off + n]), i
        off += n
    plan.set_model_timelimits(None)               # cleared: every walker finishes again
    plan.run(rho, T)
    plan.check_status()
    assert list(plan.model_status()) == [0, 0, 0, 0]
    assert torch.equal(plan.energy(), E0) and torch.equal(T, T0)
