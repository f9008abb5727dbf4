"""GPU thermal Monte Carlo against the CPU oracle.

With the same seed both implementations draw identical Philox streams and evaluate the
same IEEE operations, and the energy is accumulated in int64, so the absorbed-energy
arrays must be equal bit for bit, and so must the temperatures derived from them.
"""
import numpy as np
import pytest
import torch

from pdspy_gb300 import thermal, workloads
from tests import _cases

pytestmark = pytest.mark.gpu

CASES = ["disk_full", "disk_mirror", "two_species_mrw", "spiral_3d", "parked", "parked_mrw2"]


def _gpu_run(models, nphot, **kw):
    plan = thermal.ThermalPlan([m.grid for m in models], nphot, **kw)
    rho, T = plan.new_buffers()
    rho.copy_(torch.from_numpy(np.concatenate(
        [thermal.stack_density(m.grid).reshape(-1) for m in models])))
    plan.run(rho, T)
    torch.cuda.synchronize()
    stats = plan.check_status()
    return plan, plan.energy().cpu().numpy(), T.cpu().numpy(), stats


@pytest.mark.parametrize("name", CASES)
def test_plain_bit_exact(cuda, name):
    m, kw = _cases.case(name)
    nphot = 4000
    plan, E, T, st = _gpu_run([m], nphot, seed=11, **kw)
    ref = _cases.run_oracle(m, nphot, seed=11, **kw)
    assert np.array_equal(E, ref["energy"].reshape(-1)), name
    assert np.array_equal(T, ref["temperature"].reshape(-1)), name
    for k in ("escaped", "killed", "absorptions", "scatterings", "crossings", "events",
              "mrw_steps"):
        assert st[k] == ref["stats"][k], (name, k)
    assert np.array_equal(plan.escape().cpu().numpy()[0], ref["escape"])
    if name.startswith("parked"):
        assert st["parked"] > 0 and st["late_units"] > 0


@pytest.mark.parametrize("name", ["disk_full", "two_species_mrw", "spiral_3d", "parked",
                                  "parked_mrw2"])
def test_fp64_geometry_bit_exact(cuda, name):
    """The precision-reference instantiation (FP64 positions and walls) against the
    oracle's FP64 geometry."""
    m, kw = _cases.case(name)
    nphot = 3000
    plan, E, T, st = _gpu_run([m], nphot, seed=5, fp64_walls=True, **kw)
    ref = _cases.run_oracle(m, nphot, seed=5, fp64_walls=True, **kw)
    assert np.array_equal(E, ref["energy"].reshape(-1)), name
    assert np.array_equal(T, ref["temperature"].reshape(-1)), name
    for k in ("escaped", "killed", "crossings", "events", "mrw_steps"):
        assert st[k] == ref["stats"][k], (name, k)


@pytest.mark.parametrize("variant", [dict(drain_below=-1), dict(drain_below=10 ** 9),
                                     dict(block_threads=128, blocks_per_sm=1)])
def test_continuation_schedules_change_nothing(cuda, variant):
    """Resumed long walks one per thread or drained to one per warp, and other block
    schedules -- the same interactions either way."""
    models = workloads.walker_models(n=4, seed=8, scale=0.2)
    kw = dict(seed=4, mrw=True, mrw_count_trigger=10, late_after=60, mrw_eager_after=120)
    _, E1, T1, s1 = _gpu_run(models, 3000, **kw)
    _, E2, T2, s2 = _gpu_run(models, 3000, **variant, **kw)
    assert s1["parked"] > 0
    if variant.get("drain_below") == 10 ** 9:
        assert s2["drained"] > 0
    if variant.get("drain_below") == -1:
        assert s2["drained"] == 0
    assert np.array_equal(E1, E2) and np.array_equal(T1, T2)
    for k in ("events", "crossings", "absorptions", "scatterings", "mrw_steps", "late_units"):
        assert s1[k] == s2[k], k


def test_batched_matches_each_model(cuda):
    models = workloads.walker_models(n=3, seed=5, scale=0.15)
    nphot = [3000, 1500, 4500]
    plan, E, T, st = _gpu_run(models, nphot, seed=2)
    off = 0
    for i, m in enumerate(models):
        ref = _cases.run_oracle(m, nphot[i], seed=2, model_id=i)
        n = ref["energy"].size
        assert np.array_equal(E[off:off + n], ref["energy"].reshape(-1)), i
        assert np.array_equal(T[off:off + n], ref["temperature"].reshape(-1)), i
        off += n


def test_run_thermal_api_fills_grid_temperature(cuda):
    m, _ = _cases.case("disk_full")
    m.run_thermal(nphot=2000, code="gb300", iseed=4, verbose=False, setthreads=8)
    assert isinstance(m.grid.temperature, list) and len(m.grid.temperature) == 1
    T = m.grid.temperature[0]
    assert T.dtype == np.float64 and T.shape == m.grid.density[0].shape
    ref = _cases.run_oracle(m, 2000, seed=4)
    assert np.array_equal(T, ref["temperature"][0])


def test_graph_replay_reproduces(cuda):
    m, _ = _cases.case("disk_full")
    plan = thermal.ThermalPlan([m.grid], 3000, seed=9)
    rho, T = plan.new_buffers()
    rho.copy_(torch.from_numpy(thermal.stack_density(m.grid).reshape(-1)))
    g = plan.capture(rho, T)
    g.replay()
    torch.cuda.synchronize()
    E1 = plan.energy().clone()
    g.replay()
    torch.cuda.synchronize()
    assert torch.equal(E1, plan.energy())
    ref = _cases.run_oracle(m, 3000, seed=9)
    assert np.array_equal(E1.cpu().numpy(), ref["energy"].reshape(-1))


def test_autotune_picks_a_schedule_and_caches_it(cuda, tmp_path):
    models = workloads.walker_models(n=3, seed=5, scale=0.15)
    cache = str(tmp_path / "sched.json")
    best, times = thermal.autotune(models, 3000, probe_nphot=1500, cache=cache,
                                   modified_random_walk=True, mrw_count_trigger=20)
    assert best in thermal.SCHEDULES and len(times) == len(thermal.SCHEDULES)
    again, t2 = thermal.autotune(models, 3000, cache=cache)
    assert again == best and t2 == times
    # the chosen schedule gives the same temperatures as the default one
    _, E1, T1, _ = _gpu_run(models, 3000, seed=1, mrw=True, **best)
    _, E2, T2, _ = _gpu_run(models, 3000, seed=1, mrw=True)
    assert np.array_equal(E1, E2) and np.array_equal(T1, T2)
