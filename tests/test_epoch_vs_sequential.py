"""The deterministic epoch form of Bjorkman & Wood against the classic sequential form
(the reference algorithm: every absorption reads the running temperature), both in the
CPU oracle, compared by the per-cell criterion: over an ensemble of seeds, the mean
temperatures agree within 4 sigma of the seed-to-seed scatter in every heated cell crossed
>= 1e3 times per run.

The epoch form takes a cell's reemission temperature (and MRW mean opacities) at the
epoch snapshot plus the packet's own deposits in that cell.  Without the own-deposit term
(own_heating=0) a packet trapped in an optically thick cell does not heat the cell it
reemits from, and the inner-rim midplane of the config-0 disk comes out several sigma
colder than sequential B&W.
"""
import numpy as np
import pytest

from pdspy_gb300 import workloads
from tests import _cases

MRW = dict(mrw=True, mrw_gamma=2.0, mrw_tauthres=10.0, mrw_count_trigger=100)


def test_epoch_and_sequential_agree_within_four_sigma():
    m = workloads.small_disk(nr=24, ntheta=24, mass=1e-4, g=0.6)
    E, S, C = [], [], 0
    for seed in range(8):
        a = _cases.run_oracle(m, 20000, seed=seed, crossings=True, **MRW)
        b = _cases.run_oracle(m, 20000, seed=100 + seed, sequential=True, **MRW)
        E.append(a["temperature"])
        S.append(b["temperature"])
        C = C + a["crossings"]
    z, _ = _cases.four_sigma(np.array(E), np.array(S), C)
    assert z.size >= 50
    assert np.all(np.abs(z) < 4.0), np.abs(z).max()
    assert np.median(np.abs(z)) < 1.0


@pytest.mark.slow
def test_config0_epoch_matches_sequential_per_cell():
    """Config 0 as specified (100 x 100 cells over [0, pi], Mdisk 1e-4, 1e5 packets,
    production MRW, the product's epoch schedule): 16 seeds of each form.  Every cell
    crossed >= 1e3 times per run is within 4 sigma; the z values look like noise (median
    |z| near 0.67, few beyond 3 sigma for a t-statistic from 16 + 16 runs)."""
    seeds = range(16)
    E, C = _cases.oracle_ensemble("small_disk", {}, 100000, seeds, **MRW)
    S, _ = _cases.oracle_ensemble("small_disk", {}, 100000, [1000 + s for s in seeds],
                                  sequential=True, **MRW)
    z, rel = _cases.four_sigma(E, S, C)
    assert z.size >= 1200
    assert np.all(np.abs(z) < 4.0), np.abs(z).max()
    assert np.median(np.abs(z)) < 0.8
    assert np.mean(np.abs(z) > 3.0) < 0.015
    assert abs(np.mean(z)) < 0.3


@pytest.mark.slow
def test_heavy_walker_epoch_matches_sequential_per_cell():
    """Walker 36 of the batched workload (one of the walkers with the longest walks: dense
    inner rim, walks of 1e7-1e8 interactions in both forms), 1e4 packets, production MRW and
    schedule, 16 seeds of each form: every cell crossed >= 1e3 times per run within 4 sigma."""
    seeds = range(16)
    E, C = _cases.oracle_ensemble("walker_model", {"i": 36}, 10000, seeds, **MRW)
    S, _ = _cases.oracle_ensemble("walker_model", {"i": 36}, 10000, [1000 + s for s in seeds],
                                  sequential=True, **MRW)
    z, rel = _cases.four_sigma(E, S, C)
    assert z.size >= 30
    assert np.all(np.abs(z) < 4.0), np.abs(z).max()
    assert np.median(np.abs(z)) < 1.0
